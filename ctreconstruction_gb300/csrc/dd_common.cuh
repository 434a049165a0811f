// Device helpers shared by the DD forward projector and its matched adjoint.
#pragma once
#include <cuda_runtime.h>
#include "ctgb_internal.h"

namespace ctgb {

// Transverse axes of a dominant axis A (distance_forward,
// python/Reconstruction_numba.py:896-1055):
//   A = x: b1 = y (U lines), b2 = z (V lines)
//   A = y: b1 = x,           b2 = z
//   A = z: b1 = x,           b2 = y
template <int A> struct Axes {
    static constexpr int B1 = (A == 0) ? 1 : 0;
    static constexpr int B2 = (A == 2) ? 1 : 2;
};

// The four boundary lines of one detector pixel, as slope/intercept pairs in
// the (A, b) planes, and the intersection length (distance_forward :898-908).
struct PixelLines {
    float sU1, iU1, sU2, iU2;   // b1 coordinate of the left/right column-boundary rays
    float sV1, iV1, sV2, iV2;   // b2 coordinate of the lower/upper row-boundary rays
    float L;                    // |d_A| / (cos(atan t1) cos(atan t2))
};

__device__ __forceinline__ float view_scalar(const float *V, int f) { return V[f]; }

template <int A>
__device__ __forceinline__ PixelLines pixel_lines(const float *__restrict__ V, const ViewOffsets &vo, int r, int c,
                                                  float dA_abs) {
    constexpr int B1 = Axes<A>::B1, B2 = Axes<A>::B2;
    const float S[3] = {V[VF_SX], V[VF_SY], V[VF_SZ]};
    const float pz = V[vo.pz + r];
    const float pcx = V[vo.px + c], pcy = V[vo.py + c];
    // U points (column boundaries c, c+1 at the pixel-centre z), V points
    // (pixel-centre x/y at row boundaries r+1, r), centre point.
    const float U1[3] = {V[vo.bx + c], V[vo.by + c], pz};
    const float U2[3] = {V[vo.bx + c + 1], V[vo.by + c + 1], pz};
    const float V1[3] = {pcx, pcy, V[vo.bz + r + 1]};
    const float V2[3] = {pcx, pcy, V[vo.bz + r]};
    const float C[3] = {pcx, pcy, pz};
    PixelLines L;
    L.sU1 = (S[B1] - U1[B1]) / (S[A] - U1[A]);
    L.iU1 = -L.sU1 * S[A] + S[B1];
    L.sU2 = (S[B1] - U2[B1]) / (S[A] - U2[A]);
    L.iU2 = -L.sU2 * S[A] + S[B1];
    L.sV1 = (S[B2] - V1[B2]) / (S[A] - V1[A]);
    L.iV1 = -L.sV1 * S[A] + S[B2];
    L.sV2 = (S[B2] - V2[B2]) / (S[A] - V2[A]);
    L.iV2 = -L.sV2 * S[A] + S[B2];
    const float t1 = (S[B1] - C[B1]) / (S[A] - C[A]);
    const float t2 = (S[B2] - C[B2]) / (S[A] - C[A]);
    // 1/cos(atan t) = sqrt(1 + t^2)
    L.L = dA_abs * sqrtf(1.0f + t1 * t1) * sqrtf(1.0f + t2 * t2);
    return L;
}

// Detector-row boundaries on one slice of an x/y-dominant view, in voxel
// units along z.  Row boundary r of the column whose ray factor is tau meets
// the slice at
//     Z(r) = A + tau * (B0 + r * dB),   A = (S_z - zplane_0) / dz,
// (B0, dB from the view record).  In float32 a position near z index 512
// carries up to 3e-5 voxel of rounding, which is 3e-5 of a row's weight: the
// forward projector and its matched adjoint would each be that far from the
// exact weights, and from each other.  So both evaluate Z from the same float
// inputs as if in exact arithmetic: Z at a base row R as an unevaluated sum
// (integer part + small remainder) by error-free products and sums, and rows
// R + j near it as remainder + j * tau * dB in plain float (|value| < 64, so
// below 4e-6 voxel of rounding).  The intrinsics keep the compiler from
// fusing the products that the error terms recover.
struct ZFrame {
    float ibf;   // integer part of Z(R), as a float
    float f;     // Z(R) - ibf (small; may be slightly negative)
    float sg;    // tau * dB, the local step per row
};

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ ZFrame row_frame(float A, float tau, float B0, float dB, float R) {
    const float p1 = __fmul_rn(tau, B0), e1 = fmaf(tau, B0, -p1);    // tau B0 = p1 + e1
    const float sg = __fmul_rn(tau, dB), es = fmaf(tau, dB, -sg);    // tau dB = sg + es
    const float p2 = __fmul_rn(R, sg), e2 = fmaf(R, sg, -p2);        // R sg = p2 + e2
    float s1, t1, s2, t2;
    two_sum(A, p1, s1, t1);
    two_sum(s1, p2, s2, t2);
    const float lo = fmaf(R, es, __fadd_rn(__fadd_rn(t1, t2), __fadd_rn(e1, e2)));
    ZFrame z;
    z.ibf = floorf(s2);
    z.f = __fadd_rn(__fsub_rn(s2, z.ibf), lo);
    z.sg = sg;
    return z;
}

// One axis of a pixel footprint on one slice: the covered cell range and the
// quantities weight_calculator1/2 (python/GPUFuncs_numba.py:16-47) need.
struct Span {
    int s, e;        // first/last cell index (may lie outside the volume)
    float lo, hi;    // footprint end points
    float inv_len;   // 1 / |hi - lo|
};

__device__ __forceinline__ Span make_span(float c1, float c2, float p0, float inv_d) {
    Span sp;
    int i1 = __float2int_rd((c1 - p0) * inv_d);
    int i2 = __float2int_rd((c2 - p0) * inv_d);
    sp.s = min(i1, i2);
    sp.e = max(i1, i2);
    sp.lo = fminf(c1, c2);
    sp.hi = fmaxf(c1, c2);
    sp.inv_len = (sp.s == sp.e) ? 0.0f : __frcp_rn(sp.hi - sp.lo);
    return sp;
}

// Overlap fraction of cell k (planes p_k, p_k1) with the footprint.  DESC:
// the axis's planes decrease with the index (weight_calculator1), else
// weight_calculator2.  |w| < eps -> 0.
template <bool DESC>
__device__ __forceinline__ float span_weight(const Span &sp, int k, float p_k, float p_k1, float abs_d, float eps) {
    float w;
    if (sp.s == sp.e) return 1.0f;
    if (DESC) {
        if (k == sp.s) w = (sp.hi - p_k1) * sp.inv_len;
        else if (k == sp.e) w = (p_k - sp.lo) * sp.inv_len;
        else w = abs_d * sp.inv_len;
    } else {
        if (k == sp.s) w = (p_k1 - sp.lo) * sp.inv_len;
        else if (k == sp.e) w = (sp.hi - p_k) * sp.inv_len;
        else w = abs_d * sp.inv_len;
    }
    return fabsf(w) < eps ? 0.0f : w;
}

__device__ __forceinline__ const TableHeader &header(const void *T) {
    return *reinterpret_cast<const TableHeader *>(T);
}

}  // namespace ctgb
