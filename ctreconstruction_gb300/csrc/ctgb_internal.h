// Internal layout of the geometry table and helpers shared by the host
// table builder (geometry.cpp) and the CUDA kernels.
#pragma once
#include <stdint.h>
#include <vector>
#include "../../include/ctgb.h"

namespace ctgb {

// Scalars at the start of the table.  All arrays that follow are float32,
// addressed by offsets counted in floats from the table base.
struct TableHeader {
    int32_t nx, ny, nz, nu, nv, nviews;
    int32_t curved, flavour;
    float eps_fwd, eps_bp;        // weight clamps (|w| < eps -> 0); 0 disables
    float dx, dy, dz;             // signed voxel spacings: dx, -dy, -dz
    float du_bp, dv_bp;           // backprojector detector pitches: du (or du/SDD if curved), -dv
    float sad, sdd;
    float src0x, src0y, src0z;    // SourceInit
    float det0y;                  // DetectorInit[1]
    float dtheta;                 // angle[1] - angle[0]
    float du_fwd, dv_fwd;         // forward detector pitches (du or du/SDD; dv)
    float u0_fwd;                 // forward u coordinate of column boundary 0
    int32_t pad0;
    int64_t off_xplane, off_yplane, off_zplane;   // forward voxel boundary planes (n+1)
    int64_t off_xpix, off_ypix, off_zpix;         // backprojector voxel centres (n)
    int64_t off_ki, off_pp;                       // backprojector detector planes (nu+1, nv+1)
    int64_t off_views;                            // first view record
    int64_t view_stride;                          // floats per view record
};

// Per-view record: kViewScalars floats, then the column and row tables.
enum ViewField {
    VF_AXIS = 0,   // dominant axis of the forward projector (0 x, 1 y, 2 z), stored as float
    VF_SX, VF_SY, VF_SZ,          // forward source position
    VF_COS, VF_SIN,               // cos/sin of the view angle
    VF_BPSZ,                      // backprojector source z (SourceInit z + H*theta/2pi)
    VF_ANGLE,
    VF_EUX, VF_EUY,               // detector u axis (cos, sin)
    VF_EWX, VF_EWY,               // detector normal (sin, -cos)
    // Detector-row boundaries in the forward projector's z units:
    // B(r) = (S_z - Bz[r]) / dz (dz signed) = VF_B0 + r * VF_DB exactly for
    // the uniform rows of every supported detector; both from float64.
    VF_B0, VF_DB,
    kViewScalars = 16
};
// Column/row tables inside a view record (offsets in floats from the record start):
//   Bx[nu+1], By[nu+1]  world x/y of column boundaries
//   Px[nu],   Py[nu]    world x/y of column centres
//   Bz[nv+1]            world z of row boundaries
//   Pz[nv]              world z of row centres
struct ViewOffsets {
    int64_t bx, by, px, py, bz, pz, stride;
};

inline
#ifdef __CUDACC__
__host__ __device__
#endif
ViewOffsets view_offsets(int nu, int nv) {
    ViewOffsets o;
    o.bx = kViewScalars;
    o.by = o.bx + (nu + 1);
    o.px = o.by + (nu + 1);
    o.py = o.px + nu;
    o.bz = o.py + nu;
    o.pz = o.bz + (nv + 1);
    o.stride = o.pz + nv;
    o.stride = (o.stride + 31) & ~int64_t(31);  // 128-byte aligned records
    return o;
}

// A full circular orbit whose view count is a multiple of 4 (float32 cosines
// and sines repeat, rotated, every quarter of the views): the geometry table
// then holds views v + views/4 as exact quarter-turn rotations of view v
// (geometry.cpp), except in the view groups {g + k views/4} listed in
// *broken, where the forward's dominant axis does not alternate between x
// and y (45-degree ties).
bool quarter_turn_views(const ctgb_params *p, std::vector<int> *broken);
// The forward's slice centres (plane + half a spacing, in float) of a square
// grid are exact negatives of each other under the reflections a quarter
// turn makes (x_i = y_(n-1-i) = -x_(n-1-i) = -y_i), so the four views of a
// rotation group see their slices at exactly +-the same source distance.
bool slice_centres_antisymmetric(const ctgb_params *p);

}  // namespace ctgb
