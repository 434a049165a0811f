// DD forward projector: proj = A vol.
//
// Semantics follow distance_forward (python/Reconstruction_numba.py:805-1117)
// with distance_project_on_{x,y,z} (python/GPUFuncs_numba.py:88-240): for each
// detector pixel and each slice along the view's dominant axis, the pixel's
// footprint (the four boundary rays cut by the slice's centre plane) is
// overlapped with the voxel grid of that slice; overlap fractions (weight
// calculators, clamped below eps) times the pixel's intersection length are
// accumulated.
//
// GB300 layout: one thread per detector pixel accumulates the whole ray sum in
// a register (no atomics; the reference launches one thread per (pixel, slice)
// and atomically adds into the pixel).  A block covers a 32x4 detector tile of
// one view, so a warp's footprints are adjacent along the transverse axis and
// its volume reads are unit-stride rows.  For x-dominant views the volume is
// read from a [z][x][y] copy (ctgb_transpose_xy) so that rows stay unit-stride.
// Per-pixel line set-up happens once per view; the slice loop does four FMAs,
// four floor-conversions and the (usually 2x2) weighted gather per slice.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "dd_common.cuh"
#include "status.h"
#include "tma.cuh"
#include "updates.cuh"

namespace ctgb {

constexpr int kFwdTileU = 32, kFwdTileV = 4;

template <int A>
__device__ __forceinline__ float project_pixel(const TableHeader &h, const float *__restrict__ T,
                                               const float *__restrict__ V, const ViewOffsets &vo,
                                               const float *__restrict__ vol, const float *__restrict__ vol_xzy,
                                               int r, int c) {
    constexpr int B1 = Axes<A>::B1, B2 = Axes<A>::B2;
    const float d[3] = {h.dx, h.dy, h.dz};
    const int n[3] = {h.nx, h.ny, h.nz};
    const float *planes[3] = {T + h.off_xplane, T + h.off_yplane, T + h.off_zplane};
    const float *__restrict__ pa = planes[A];
    const float *__restrict__ pb1 = planes[B1];
    const float *__restrict__ pb2 = planes[B2];
    const PixelLines ln = pixel_lines<A>(V, vo, r, c, fabsf(d[A]));
    const float p0b1 = pb1[0], p0b2 = pb2[0];
    const float inv_db1 = 1.0f / d[B1], inv_db2 = 1.0f / d[B2];
    const float abs_db1 = fabsf(d[B1]), abs_db2 = fabsf(d[B2]);
    const float eps = h.eps_fwd;
    const int nA = n[A], nb1 = n[B1], nb2 = n[B2];
    // Element strides of (slice, b1 index, b2 index) in the layout this axis reads.
    long long st_s, st_k, st_l;
    const float *__restrict__ src = vol;
    if (A == 1) { st_s = h.nx; st_k = 1; st_l = (long long)h.nx * h.ny; }
    else if (A == 2) { st_s = (long long)h.nx * h.ny; st_k = 1; st_l = h.nx; }
    else if (vol_xzy) { src = vol_xzy; st_s = h.ny; st_k = 1; st_l = (long long)h.nx * h.ny; }
    else { st_s = 1; st_k = h.nx; st_l = (long long)h.nx * h.ny; }

    float acc = 0.0f;
    for (int s = 0; s < nA; ++s) {
        const float pc = pa[s] + d[A] * 0.5f;
        const Span u = make_span(ln.sU1 * pc + ln.iU1, ln.sU2 * pc + ln.iU2, p0b1, inv_db1);
        const Span v = make_span(ln.sV1 * pc + ln.iV1, ln.sV2 * pc + ln.iV2, p0b2, inv_db2);
        const int k0 = max(u.s, 0), k1 = min(u.e, nb1 - 1);
        const int l0 = max(v.s, 0), l1 = min(v.e, nb2 - 1);
        const float *__restrict__ row = src + s * st_s;
        for (int l = l0; l <= l1; ++l) {
            // z (and y for A = z) planes decrease with the index; x planes increase.
            const float w2 = (B2 == 0) ? span_weight<false>(v, l, pb2[l], pb2[l + 1], abs_db2, eps)
                                       : span_weight<true>(v, l, pb2[l], pb2[l + 1], abs_db2, eps);
            float part = 0.0f;
            for (int k = k0; k <= k1; ++k) {
                const float w1 = (B1 == 0) ? span_weight<false>(u, k, pb1[k], pb1[k + 1], abs_db1, eps)
                                           : span_weight<true>(u, k, pb1[k], pb1[k + 1], abs_db1, eps);
                part += __ldg(row + k * st_k + l * st_l) * w1;
            }
            acc += part * w2;
        }
    }
    return acc * ln.L;
}

__global__ void __launch_bounds__(kFwdTileU * kFwdTileV)
dd_forward_kernel(const float *__restrict__ T, const float *__restrict__ vol, const float *__restrict__ vol_xzy,
                  float *__restrict__ proj, int view0) {
    const TableHeader &h = header(T);
    const int c = blockIdx.x * kFwdTileU + threadIdx.x;
    const int r = blockIdx.y * kFwdTileV + threadIdx.y;
    const int vi = blockIdx.z;
    if (c >= h.nu || r >= h.nv) return;
    const ViewOffsets vo = view_offsets(h.nu, h.nv);
    const float *__restrict__ V = T + h.off_views + (long long)(view0 + vi) * h.view_stride;
    const int axis = (int)V[VF_AXIS];
    float val;
    if (axis == 1) val = project_pixel<1>(h, T, V, vo, vol, vol_xzy, r, c);
    else if (axis == 0) val = project_pixel<0>(h, T, V, vo, vol, vol_xzy, r, c);
    else val = project_pixel<2>(h, T, V, vo, vol, vol_xzy, r, c);
    proj[((long long)vi * h.nv + r) * h.nu + c] = val;
}

// One 32 x 32 tile (bx, by) of slice z of the [z][y][x] -> [z][x][y] copy.
__device__ __forceinline__ void transpose_tile(float (&tile)[32][33], const float *__restrict__ in,
                                               float *__restrict__ out, int nx, int ny, int bx, int by, int z) {
    const int x0 = bx * 32, y0 = by * 32;
    const float *src = in + (long long)z * nx * ny;
    float *dst = out + (long long)z * nx * ny;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        int x = x0 + threadIdx.x, y = y0 + j;
        if (x < nx && y < ny) tile[j][threadIdx.x] = src[(long long)y * nx + x];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        int y = y0 + threadIdx.x, x = x0 + j;
        if (x < nx && y < ny) dst[(long long)x * ny + y] = tile[threadIdx.x][j];
    }
}

__global__ void transpose_xy_kernel(const float *__restrict__ in, float *__restrict__ out, int nx, int ny) {
    __shared__ float tile[32][33];
    transpose_tile(tile, in, out, nx, ny, blockIdx.x, blockIdx.y, blockIdx.z);
}

// Batched transpose: job j's tiles are items item0 .. item0 + tx * ty * nz - 1.
struct TransJob {
    const float *in;
    float *out;
    int nx, ny, nz, tx, ty, item0;
};

__global__ void transpose_xy_batch_kernel(const TransJob *__restrict__ jobs, int njobs, int nitems) {
    __shared__ float tile[32][33];
    int j = 0;
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        while (j + 1 < njobs && it >= jobs[j + 1].item0) ++j;
        const TransJob &jb = jobs[j];
        const int local = it - jb.item0, per = jb.tx * jb.ty;
        const int z = local / per, t = local - z * per;
        transpose_tile(tile, jb.in, jb.out, jb.nx, jb.ny, t % jb.tx, t / jb.tx, z);
        __syncthreads();   // the tile is rewritten by the next item
    }
}


// ---------------------------------------------------------------------------
// TMA forward projector for views whose dominant axis is x (XD) or y.
//
// One warp = one CTA owns a tile of kTU = 32 detector columns (one per lane) x
// TR = 32 (or 16) rows of one view.  It walks the slices along the dominant
// axis; for each slice the tile's footprint on the slice (a window of the
// volume, at most kPX x PZ = 64 x 48 (32) voxels) is brought into shared
// memory by TMA boxes of 64 x 1 x 8 voxels, completing on an mbarrier.
// Out-of-volume voxels arrive as zeros (TMA OOB fill), which is the
// reference's bounds test.
// Tile height: the per-slice work (window, column taps, warp votes) is shared
// by the tile's rows, so taller tiles spend less per pixel but hold more
// accumulators and a taller patch.  At 512^3 / 720 views, 1024 x 768: 16 rows
// (32-row patch, 24 CTAs per SM) 131.6 ms, 24 rows 129.3, 32 rows (48-row
// patch, 16 CTAs per SM) 113.2, 40 rows 127.0, 48 rows 128.9, 64 rows 163.1.
// At that geometry a detector row spans at most 1.18 voxel rows.  Geometries
// whose rows span more than 1.3 voxel rows take 16-row tiles, which fit rows
// of up to 1.75 voxel rows in their 32-row patch.
//
// Maths per pixel and slice (same result as the weight-calculator loop):
//   * the column footprint [x1', x2'] and row boundaries z'_j are linear in
//     q = pc - S_a (every boundary ray passes through the source), so both
//     footprint widths are |q| times a per-pixel constant and the reference's
//     two weight denominators become K_pixel / q^2 — one factor per slice;
//   * h(m) = sum_k P[m][k] * overlap_x(k) for the lane's column (2-4 taps,
//     overlaps in voxel units), and the row integral over [z'_j, z'_j+1] is
//     h at each end cell times its covered part plus any whole cell between;
//     consecutive rows share their boundary cell's h.
// Slices whose window exceeds the patch, or whose footprint is wider than 4
// voxels, are integrated cell by cell from global memory (compact, rare path).
constexpr int kTU = 32, kBoxX = 64, kBoxZ = 8, kPX = kBoxX;

// Tiles of TR = 32 or 16 detector rows.  PZ patch rows hold a tile whose rows
// each span up to 1.3 (TR = 32) or 1.75 (TR = 16) voxel rows, with the
// window's margins and box rounding; MINB CTAs per SM fit the registers and
// shared memory.  The host picks TR per call (fwd_tile_rows).
template <int TR>
struct FwdTile {
    static constexpr int PZ = TR == 32 ? 48 : 32;
    static constexpr int MINB = TR == 32 ? 16 : 24;
};

// Patch buffers per CTA: 2 overlaps each slice's TMA with the previous
// slice's compute inside the warp; 1 halves shared memory so twice as many
// warps are resident and hide the load latency across warps instead.
#ifndef CTGB_FWD_BUFS
#define CTGB_FWD_BUFS 1
#endif
constexpr int kFwdBufs = CTGB_FWD_BUFS;

template <int TR>
struct FwdTmaSmem {
    float buf[kFwdBufs][FwdTile<TR>::PZ][kPX];
    // per-slice row values of the fallback path; with one patch buffer they
    // live in it (no copy is in flight while a slice is computed)
    float spill[kFwdBufs == 1 ? 1 : TR][kTU];
    uint64_t bar[2];
};

struct TileWindow {
    int kb, lb, nbz;     // patch origin (kb multiple of 4) and number of 8-row boxes
    bool active, fits;
    ZFrame zf;           // the lane's row boundaries on the slice: tile row j at zf.ibf + zf.f + j * zf.sg
};

// h(m): the lane's column footprint (NT taps) applied to the patch row of
// local cell m (z index m + frame integer part).
template <int NT>
struct PatchCells {
    const float *base;   // &patch[0][k0 - kb]
    int lb;              // window base minus the frame's integer part
    float ov0, ov1, ov2, ov3;
    __device__ __forceinline__ float operator()(int m) const {
        const float *p = base + (m - lb) * kPX;
        float v = p[0] * ov0 + p[1] * ov1;
        if (NT > 2) v = fmaf(p[2], ov2, v);
        if (NT > 3) v = fmaf(p[3], ov3, v);
        return v;
    }
};

// Integrate h over consecutive row boundaries of two chains of N rows (rows
// 0..N-1 and N..2N-1), stepped together so that each chain's floor/lookup
// latency overlaps the other's.  MID: a row may cover three cells (one whole
// cell in the middle); rows never cover four (checked per slice by the
// caller).  No data-dependent branches.  Chain a is the .x and chain b the
// .y of float2 pairs, so the boundary positions, floors, fractions, cell
// values and row sums of both chains take one packed f32x2 operation each (147.9 -> 137.4 ms per 512^3 / 720-view forward against
// the scalar pair); acc2[j] holds rows j and N + j.  Boundary j of the tile
// sits at local z f + j * sg (the frame of row_frame; cells are local too,
// PatchCells adds the frame's integer part).
template <int NT, bool MID, int N>
__device__ __forceinline__ void sweep_rows2(const PatchCells<NT> &H, float f, float sg, float g, float2 *acc2) {
    const float2 sg2 = make_float2(sg, sg), f2 = make_float2(f, f), g2 = make_float2(g, g);
    const float2 neg1 = make_float2(-1.0f, -1.0f), mag = make_float2(-12582912.0f, -12582912.0f);
    auto o = [&](int t) { return t == 0 ? H.ov0 : (t == 1 ? H.ov1 : (t == 2 ? H.ov2 : H.ov3)); };
    // h for both chains: NT cells of each chain's row, weighted by the column footprint.
    auto H2 = [&](int ma, int mb) {
        const float *pa = H.base + (ma - H.lb) * kPX, *pb = H.base + (mb - H.lb) * kPX;
        float2 h = __fmul2_rn(make_float2(pa[0], pb[0]), make_float2(o(0), o(0)));
#pragma unroll
        for (int t = 1; t < NT; ++t) h = __ffma2_rn(make_float2(pa[t], pb[t]), make_float2(o(t), o(t)), h);
        return h;
    };
    // floor of both boundaries (round-down add of 1.5*2^23), the floors as
    // floats, and the fractions.
    auto split = [&](float2 z, int &ma, int &mb, float2 &f, float2 &fr) {
        const float2 t = __fadd2_rd(z, make_float2(12582912.0f, 12582912.0f));
        ma = __float_as_int(t.x) - 0x4B400000;
        mb = __float_as_int(t.y) - 0x4B400000;
        f = __fadd2_rn(t, mag);                                     // floor as float
        fr = __ffma2_rn(f, neg1, z);                                // z - floor
    };
    // Row [z0, z1] with cells m0 = floor z0 and m1 = floor z1 = m0 + d:
    // h1 (z1 - m1) + h0 (m1 - z0) for d <= 1 (for d = 0 both cells are m0),
    // plus (hm - h0) for a three-cell row (d = 2, only with MID), which turns
    // h0's share into h0 (m0 + 1 - z0) and adds the whole middle cell hm.
    // Carrying z0 instead of the end term h0 (z0 - m0) saves the per-row
    // difference of end terms (117.0 -> 112.1 ms per 512^3 / 720-view forward
    // with the three-cell case's selects as saturated factors).
    float2 z0 = __ffma2_rn(make_float2(0.0f, (float)N), sg2, f2), f0, fr0;
    int m0a, m0b;   // only addresses h0; later rows need only the float floors
    split(z0, m0a, m0b, f0, fr0);
    float2 h0 = H2(m0a, m0b);
#pragma unroll
    for (int j = 0; j < N; ++j) {
        const float2 z1 = __ffma2_rn(make_float2((float)(j + 1), (float)(N + j + 1)), sg2, f2);
        int m1a, m1b;
        float2 f1, fr1;
        split(z1, m1a, m1b, f1, fr1);
        const float2 h1 = H2(m1a, m1b);
        float2 r = __ffma2_rn(h1, fr1, __fmul2_rn(h0, __fadd2_rn(f1, make_float2(-z0.x, -z0.y))));
        if (MID) {
            // the middle cell of a three-cell row is m1 - 1 (read for every
            // row; the window's one-cell margin keeps it inside the patch);
            // max(d - 1, 0) is 1 for d = 2 and 0 otherwise, so (hm - h0)
            // enters only there
            const float2 d = __ffma2_rn(f0, neg1, f1);
            const float2 hm = H2(m1a - 1, m1b - 1);
            r = __ffma2_rn(__fadd2_rn(hm, make_float2(-h0.x, -h0.y)),
                           make_float2(__saturatef(d.x - 1.0f), __saturatef(d.y - 1.0f)), r);
        }
        acc2[j] = __ffma2_rn(r, g2, acc2[j]);
        h0 = h1; z0 = z1; f0 = f1;
    }
}

template <int NT, bool MID, int TR>
__device__ __forceinline__ void sweep_tile(const float *patch, int lb, const float *ov, const ZFrame &zf, float g,
                                           float2 *acc) {
    PatchCells<NT> H;
    H.base = patch;
    H.lb = lb - (int)zf.ibf;
    H.ov0 = ov[0]; H.ov1 = ov[1]; H.ov2 = ov[2]; H.ov3 = ov[3];
    sweep_rows2<NT, MID, TR / 2>(H, zf.f, zf.sg, g, acc);
}

// The views of one launch (relative to view0): every x- (or y-) dominant
// view of the call goes into one launch, so a scan whose dominant axis
// alternates every few views still fills the GPU with one grid per axis.
constexpr int kFwdListViews = 2048;
struct FwdViewList {
    int v[kFwdListViews];
};

// Barriers initialised and patch buffers zeroed once per CTA (taps past the
// loaded boxes then read finite zeros).
template <int TR>
__device__ __forceinline__ void fwd_smem_init(FwdTmaSmem<TR> &sm) {
    const int lane = threadIdx.x;
    if (lane == 0) {
        mbar_init(&sm.bar[0], 1);
        mbar_init(&sm.bar[1], 1);
        fence_mbar_init();
    }
    float4 *z = reinterpret_cast<float4 *>(&sm.buf[0][0][0]);
    for (int i = lane; i < kFwdBufs * FwdTile<TR>::PZ * kPX / 4; i += 32) z[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncwarp();
}

// One detector tile (kTU columns x TR rows, tile (tu, tv)) of view vi
// (relative to view0): the body of the single-scan and the batched forward
// kernels.  phase_bits carries the barriers' phases from tile to tile; every
// copy a tile issues is consumed before it returns.  The stored value goes
// through the epilogue epi (the projection itself, or an iterative
// driver's residual).  Returns false when a bounded wait ran out (the
// tile's copies drained first).
template <bool XD, int TR>
__device__ __forceinline__ bool fwd_tile(FwdTmaSmem<TR> &sm, const CUtensorMap *tmp, bool TMA,
                                         const float *__restrict__ T, const float *__restrict__ src, long long st_k,
                                         float *__restrict__ proj, int view0, int vi, int tu, int tv,
                                         const FwdEpi &epi, uint32_t &phase_bits, int *status) {
    constexpr int kTR = TR, kPZ = FwdTile<TR>::PZ;
    const TableHeader &h = header(T);
    const int lane = threadIdx.x;
    const int c0 = tu * kTU, r0 = tv * kTR;
    const int nu = h.nu, nv = h.nv;
    const ViewOffsets vo = view_offsets(nu, nv);
    const float *__restrict__ V = T + h.off_views + (long long)(view0 + vi) * h.view_stride;
    const int c = c0 + lane;

    const float *__restrict__ pa = T + (XD ? h.off_xplane : h.off_yplane);
    const float *__restrict__ pb = T + (XD ? h.off_yplane : h.off_xplane);
    const float *__restrict__ pzp = T + h.off_zplane;
    const float da = XD ? h.dx : h.dy, db = XD ? h.dy : h.dx, dz = h.dz;
    const int nA = XD ? h.nx : h.ny, nB = XD ? h.ny : h.nx, nZ = h.nz;
    // Strides of src in (slice, transverse, z): [z][x][y] copy or [z][y][x] volume.
    const long long st_s = XD ? (st_k == 1 ? (long long)h.ny : 1LL) : (long long)h.nx;
    const long long st_l = (long long)h.nx * h.ny;
    const float Sa = XD ? V[VF_SX] : V[VF_SY], Sb = XD ? V[VF_SY] : V[VF_SX], Sz = V[VF_SZ];
    const float *__restrict__ Ba = V + (XD ? vo.bx : vo.by);
    const float *__restrict__ Bb = V + (XD ? vo.by : vo.bx);
    const float *__restrict__ Pa = V + (XD ? vo.px : vo.py);
    const float *__restrict__ Pb = V + (XD ? vo.py : vo.px);
    const float *__restrict__ Pzr = V + vo.pz;

    // Column constants (lanes beyond nu use the last column and do not write).
    const int cc = min(c, nu - 1);
    const float inv_db = 1.0f / db, inv_dz = 1.0f / dz;
    const float Eb0 = (Sb - Bb[cc]) / (Sa - Ba[cc]) * inv_db;
    const float Eb1 = (Sb - Bb[cc + 1]) / (Sa - Ba[cc + 1]) * inv_db;
    const float Cb = (Sb - pb[0]) * inv_db;
    const float invD = 1.0f / (Sa - Pa[cc]);
    const float t1 = (Sb - Pb[cc]) * invD;
    const float A = (Sz - pzp[0]) * inv_dz;
    // Row boundaries: B(r) = B0 + r dB (uniform rows), placed on each slice by
    // row_frame from the tile's first row.
    const float B0 = V[VF_B0], dB = V[VF_DB], rowspan_max = fabsf(dB);
    float *spill_rows = kFwdBufs == 1 ? &sm.buf[0][0][0] : &sm.spill[0][0];
    static_assert(kTR * kTU <= kPZ * kPX, "fallback rows must fit the patch buffer");

    // Per-slice tile window: the union of every lane's exact footprint cells
    // (the same expressions the sweep evaluates, so every cell the sweep
    // touches lies inside the window), widened by one cell.
    auto window = [&](int s) {
        TileWindow w;
        const float q = pa[s] + 0.5f * da - Sa;
        const float xa = fmaf(Eb0, q, Cb), xb = fmaf(Eb1, q, Cb);
        const float tau = q * invD;
        w.zf = row_frame(A, tau, B0, dB, (float)r0);
        const float za = w.zf.f, zb = fmaf((float)kTR, w.zf.sg, w.zf.f);   // local z of boundaries 0, kTR
        const int ib = (int)w.zf.ibf;
        const int klo = __reduce_min_sync(0xffffffffu, (int)floorf(fminf(xa, xb))) - 1;
        const int khi = __reduce_max_sync(0xffffffffu, (int)floorf(fmaxf(xa, xb))) + 1;
        const int llo = __reduce_min_sync(0xffffffffu, ib + (int)floorf(fminf(za, zb))) - 1;
        const int lhi = __reduce_max_sync(0xffffffffu, ib + (int)floorf(fmaxf(za, zb))) + 1;
        w.active = !(khi < 0 || klo >= nB || lhi < 0 || llo >= nZ);
        w.kb = (klo >= 0 ? klo : klo - 3) / 4 * 4;           // floor to a multiple of 4
        w.lb = llo;
        w.nbz = (lhi - llo + kBoxZ) / kBoxZ;
        w.fits = TMA && (khi + 4 - w.kb <= kPX) && (w.nbz * kBoxZ <= kPZ);
        return w;
    };

    float2 acc[kTR / 2];   // rows j (.x) and kTR / 2 + j (.y)
#pragma unroll
    for (int j = 0; j < kTR / 2; ++j) acc[j] = make_float2(0.0f, 0.0f);
    uint32_t pending_bits = 0u;   // bit b: TMA outstanding for buffer b (phase_bits: its phase parity)
    bool failed = false;

    auto issue = [&](int s, const TileWindow &w, int b) {
        if (!(w.active && w.fits)) return;
        if (lane == 0) {
            mbar_arrive_expect_tx(&sm.bar[b], (uint32_t)(w.nbz * kBoxZ * kBoxX * 4));
            for (int iz = 0; iz < w.nbz; ++iz)
                tma_load_3d(&sm.buf[b][iz * kBoxZ][0], tmp, w.kb, s, w.lb + iz * kBoxZ, &sm.bar[b]);
        }
        pending_bits |= 1u << b;
    };

    TileWindow wcur = window(0);
    issue(0, wcur, 0);
    for (int s = 0; s < nA; ++s) {
        const int b = kFwdBufs == 2 ? (s & 1) : 0;
        TileWindow wnext;
        if (kFwdBufs == 2 && s + 1 < nA) {
            wnext = window(s + 1);
            issue(s + 1, wnext, b ^ 1);
        }
        if (wcur.active) {
            if ((pending_bits >> b) & 1u) {
                if (!mbar_wait(&sm.bar[b], (phase_bits >> b) & 1u, status)) { failed = true; break; }
                phase_bits ^= 1u << b;
                pending_bits &= ~(1u << b);
            }
            const float q = pa[s] + 0.5f * da - Sa;
            const float g = 1.0f / (q * q);
            const float xa = fmaf(Eb0, q, Cb), xb = fmaf(Eb1, q, Cb);
            const float lo = fminf(xa, xb), hi = fmaxf(xa, xb);
            float fk;
            const int k0 = floor_split(lo, &fk);
            // Row extent in cells: |dB tau|, the frame's step.
            const float rows_ext = fabsf(wcur.zf.sg);
            const bool wide = __any_sync(0xffffffffu, (hi - fk) > 4.0f || rows_ext > 1.99f);
            if (wcur.fits && !wide) {
                float ov[4];
#pragma unroll
                for (int t = 0; t < 4; ++t)
                    ov[t] = fmaxf(0.0f, fminf(fk + (float)(t + 1), hi) - fmaxf(fk + (float)t, lo));
                int ntl = 2;
#pragma unroll
                for (int t = 2; t < 4; ++t) ntl = (ov[t] > 0.0f) ? t + 1 : ntl;
                const int nt = __reduce_max_sync(0xffffffffu, ntl);
                const bool mid = __any_sync(0xffffffffu, rows_ext > 0.99f);
                const float *patch = &sm.buf[b][0][k0 - wcur.kb];
                if (nt == 2) {
                    if (mid) sweep_tile<2, true, TR>(patch, wcur.lb, ov, wcur.zf, g, acc);
                    else sweep_tile<2, false, TR>(patch, wcur.lb, ov, wcur.zf, g, acc);
                } else if (nt == 3) {
                    if (mid) sweep_tile<3, true, TR>(patch, wcur.lb, ov, wcur.zf, g, acc);
                    else sweep_tile<3, false, TR>(patch, wcur.lb, ov, wcur.zf, g, acc);
                } else {
                    if (mid) sweep_tile<4, true, TR>(patch, wcur.lb, ov, wcur.zf, g, acc);
                    else sweep_tile<4, false, TR>(patch, wcur.lb, ov, wcur.zf, g, acc);
                }
            } else {
                // Cell-by-cell overlap from global memory; row values go through
                // shared memory so the row loop stays rolled (small code).
                const float *__restrict__ slab = src + (long long)s * st_s;
                const int ka = max(k0, 0), kz = min((int)floorf(hi), nB - 1);
                // Row boundaries in the slice's frame (local z, integer part ib).
                const int ib = (int)wcur.zf.ibf;
                for (int j = 0; j < kTR; ++j) {
                    const float za = fmaf((float)j, wcur.zf.sg, wcur.zf.f);
                    const float zb = fmaf((float)(j + 1), wcur.zf.sg, wcur.zf.f);
                    const float zlo = fminf(za, zb), zhi = fmaxf(za, zb);
                    const int l0 = max((int)floorf(zlo) + ib, 0), l1 = min((int)floorf(zhi) + ib, nZ - 1);
                    float v = 0.0f;
                    for (int l = l0; l <= l1; ++l) {
                        const float wz = fminf((float)(l - ib + 1), zhi) - fmaxf((float)(l - ib), zlo);
                        const float *__restrict__ row = slab + (long long)l * st_l;
                        float hx = 0.0f;
                        for (int k = ka; k <= kz; ++k)
                            hx += __ldg(row + k * st_k) * (fminf((float)(k + 1), hi) - fmaxf((float)k, lo));
                        v += hx * wz;
                    }
                    spill_rows[j * kTU + lane] = v;
                }
                __syncwarp();
#pragma unroll
                for (int j = 0; j < kTR / 2; ++j) {
                    acc[j].x = fmaf(spill_rows[j * kTU + lane], g, acc[j].x);
                    acc[j].y = fmaf(spill_rows[(kTR / 2 + j) * kTU + lane], g, acc[j].y);
                }
            }
        }
        __syncwarp();
        if (kFwdBufs == 1 && s + 1 < nA) {
            wnext = window(s + 1);
            issue(s + 1, wnext, 0);
        }
        wcur = wnext;
    }
    if (failed) {
        // Let copies still in flight land before the CTA exits (bounded).
        for (int b = 0; b < kFwdBufs; ++b)
            if ((pending_bits >> b) & 1u) mbar_wait(&sm.bar[b], (phase_bits >> b) & 1u, status);
        return false;
    }
    if (c >= nu) return true;
    const float dEb = fabsf(Eb1 - Eb0);
    const float absInvD = fabsf(invD);
    const float base = fabsf(da) * sqrtf(1.0f + t1 * t1) / (dEb * absInvD);
#pragma unroll
    for (int j = 0; j < kTR; ++j) {
        const int r = r0 + j;
        if (r < nv) {
            const float t2 = (Sz - Pzr[r]) * invD;
            const float K = base * sqrtf(1.0f + t2 * t2) / rowspan_max;
            const long long i = ((long long)vi * nv + r) * nu + c;
            proj[i] = fwd_epilogue(epi, i, (j < kTR / 2 ? acc[j].x : acc[j - kTR / 2].y) * K);
        }
    }
    return true;
}

template <bool XD, bool TMA, int TR>
__global__ void __launch_bounds__(32, FwdTile<TR>::MINB)
dd_forward_tma_kernel(const __grid_constant__ CUtensorMap tm, const float *__restrict__ T,
                      const float *__restrict__ src, long long st_k, float *__restrict__ proj, int view0,
                      const __grid_constant__ FwdViewList views, int ntu, int *status) {
    extern __shared__ __align__(128) unsigned char smraw[];
    FwdTmaSmem<TR> &sm = *reinterpret_cast<FwdTmaSmem<TR> *>(smraw);
    fwd_smem_init<TR>(sm);
    uint32_t phase_bits = 0u;
    const FwdEpi epi = {kFwdStore, 0.0f, nullptr, nullptr};
    fwd_tile<XD, TR>(sm, &tm, TMA, T, src, st_k, proj, view0, views.v[blockIdx.x], blockIdx.y % ntu,
                     blockIdx.y / ntu, epi, phase_bits, status);
}

// Batched forward: the views of many scans (one axis, one tile height) in one
// persistent launch.  Job j covers items [item0, item0 + nitems): view
// views[list0 + k] (relative to the job's view0) x tile t for item
// item0 + k * ntiles + t.  Each CTA walks items blockIdx.x, + gridDim.x, ...
// in increasing order, so its job index only moves forward.
struct __align__(128) FwdJob {
    CUtensorMap tm;            // the scan's volume ([z][x][y] copy for x-dominant views) as a TMA tensor
    const float *T;            // geometry table
    const float *src;          // the volume layout the kernel reads
    float *proj;               // output of views view0 .. view0 + nviews - 1 (projections or residual)
    long long st_k;            // 1: x-dominant views read the [z][x][y] copy
    int view0, ntu, ntiles, tma;
    int item0, nitems, list0, pad;
    FwdEpi epi;
};

template <bool XD, int TR>
__global__ void __launch_bounds__(32, FwdTile<TR>::MINB)
dd_forward_batch_kernel(const FwdJob *__restrict__ jobs, int njobs, const int *__restrict__ views, int nitems,
                        int *status) {
    extern __shared__ __align__(128) unsigned char smraw[];
    FwdTmaSmem<TR> &sm = *reinterpret_cast<FwdTmaSmem<TR> *>(smraw);
    fwd_smem_init<TR>(sm);
    uint32_t phase_bits = 0u;
    int j = 0;
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        while (j + 1 < njobs && it >= jobs[j + 1].item0) ++j;
        const FwdJob &jb = jobs[j];
        const int local = it - jb.item0;
        const int k = local / jb.ntiles, t = local - k * jb.ntiles;
        if (!fwd_tile<XD, TR>(sm, &jb.tm, jb.tma != 0, jb.T, jb.src, jb.st_k, jb.proj, jb.view0,
                              views[jb.list0 + k], t % jb.ntu, t / jb.ntu, jb.epi, phase_bits, status))
            return;
    }
}

}  // namespace ctgb

using namespace ctgb;

static int check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return CTGB_OK;
}

// Dominant axis of each view, by the table builder's float64 rule
// (distance_forward, python/Reconstruction_numba.py:896, :966).
static void view_axes(const ctgb_params *p, int view0, int nviews, std::vector<int> &axes) {
    const double *S0 = p->source_init, *D0 = p->detector_init, *O = p->rotation_origin;
    const double sad = std::sqrt((S0[0] - O[0]) * (S0[0] - O[0]) + (S0[1] - O[1]) * (S0[1] - O[1]) +
                                 (S0[2] - O[2]) * (S0[2] - O[2]));
    const double sdd = std::sqrt((S0[0] - D0[0]) * (S0[0] - D0[0]) + (S0[1] - D0[1]) * (S0[1] - D0[1]) +
                                 (S0[2] - D0[2]) * (S0[2] - D0[2]));
    const double step = (p->end_angle - p->start_angle) / p->nviews;
    axes.resize(nviews);
    for (int i = 0; i < nviews; ++i) {
        const double th = (view0 + i) * step + p->start_angle;
        const double S[3] = {-sad * std::sin(th), sad * std::cos(th), p->source_init[2]};
        const double D[3] = {(sdd - sad) * std::sin(th), -(sdd - sad) * std::cos(th), p->detector_init[2]};
        const double ax = std::fabs(S[0] - D[0]), ay = std::fabs(S[1] - D[1]), az = std::fabs(S[2] - D[2]);
        axes[i] = (ax >= ay && ax >= az) ? 0 : (ay >= ax && ay >= az) ? 1 : 2;
    }
}

// Tile height for a scan.  At a slice the kernel's row boundaries are
// z_j = A + B_j * tau with tau = q / D, the in-plane distances from the source
// to the slice and to the pixel column along the pixel's ray, so a detector
// row spans dv / dz * tau voxel rows.  D >= SDD (the detector's line or arc
// lies at SDD from the source), and for a ray that meets the volume q is at
// most the source's in-plane distance to the volume centre plus the volume's
// in-plane half-diagonal.
static int fwd_tile_rows(const ctgb_params *p) {
    const double *S0 = p->source_init, *D0 = p->detector_init, *O = p->rotation_origin;
    const double *C = p->flavour == CTGB_FLAVOUR_PYCUDA ? p->recon_center : p->phantom_center;
    const double sad = std::hypot(S0[0] - O[0], S0[1] - O[1]);
    const double sdd = std::hypot(S0[0] - D0[0], S0[1] - D0[1]);
    if (!(sdd > 0.0) || !(p->dz > 0.0)) return 16;
    const double q = sad + std::hypot(C[0] - O[0], C[1] - O[1]) + 0.5 * std::hypot(p->nx * p->dx, p->ny * p->dy);
    return p->dv / p->dz * q / sdd <= 1.3 ? 32 : 16;
}

template <int TR>
static void launch_fwd_tma(bool xd, bool tma, dim3 grid, cudaStream_t st, const CUtensorMap &tm, const float *T,
                           const float *src, long long stk, float *d_proj, int view0, const FwdViewList &list,
                           int ntu, int *status) {
    const int smem = (int)sizeof(FwdTmaSmem<TR>);
    auto kernel = xd ? (tma ? dd_forward_tma_kernel<true, true, TR> : dd_forward_tma_kernel<true, false, TR>)
                     : (tma ? dd_forward_tma_kernel<false, true, TR> : dd_forward_tma_kernel<false, false, TR>);
    kernel<<<grid, 32, smem, st>>>(tm, T, src, stk, d_proj, view0, list, ntu, status);
}

template <int TR>
static cudaError_t fwd_smem_limits() {
    static std::atomic<unsigned long long> attr[4];
    const void *kernels[4] = {(const void *)dd_forward_tma_kernel<true, true, TR>,
                              (const void *)dd_forward_tma_kernel<false, true, TR>,
                              (const void *)dd_forward_tma_kernel<true, false, TR>,
                              (const void *)dd_forward_tma_kernel<false, false, TR>};
    for (int k = 0; k < 4; ++k) {
        cudaError_t e = smem_limit_once(kernels[k], (int)sizeof(FwdTmaSmem<TR>), attr[k]);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

extern "C" int ctgb_forward(const ctgb_params *p, const void *d_table, const float *d_vol, const float *d_vol_xzy,
                            float *d_proj, int32_t view0, int32_t nviews, void *stream) {
    clear_error();
    if (!p) return set_error(CTGB_ERR_ARG, "ctgb_forward: NULL argument");
    if (view0 < 0 || nviews < 0 || view0 + nviews > p->nviews)
        return set_error(CTGB_ERR_ARG, "ctgb_forward: view range [%d,%d) outside [0,%d)", view0, view0 + nviews,
                         p->nviews);
    if (nviews == 0) return CTGB_OK;   // nothing to read or write (an empty output has no storage)
    if (!d_table || !d_vol || !d_proj) return set_error(CTGB_ERR_ARG, "ctgb_forward: NULL argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const float *T = static_cast<const float *>(d_table);
    const long long view_elems = (long long)p->nu * p->nv;

    // x/y-dominant views run dd_forward_tma_kernel (TMA patches when the
    // volume layout allows 16-byte row strides, global loads otherwise);
    // z-dominant views run the per-pixel kernel.
    CUtensorMap tm_y, tm_x;
    const uint32_t box[3] = {kBoxX, 1, kBoxZ};
    bool tma_y = (p->nx % 4 == 0), tma_x = (p->ny % 4 == 0) && d_vol_xzy != nullptr;
    if (tma_y) {
        const uint64_t d[3] = {(uint64_t)p->nx, (uint64_t)p->ny, (uint64_t)p->nz};
        tma_y = ctgb_make_tmap_3d(&tm_y, d_vol, d, box);
    }
    if (tma_x) {
        const uint64_t d[3] = {(uint64_t)p->ny, (uint64_t)p->nx, (uint64_t)p->nz};
        tma_x = ctgb_make_tmap_3d(&tm_x, d_vol_xzy, d, box);
    }
    if (!tma_y) std::memset(&tm_y, 0, sizeof tm_y);
    if (!tma_x) std::memset(&tm_x, 0, sizeof tm_x);
    int *status = ctgb_status_ptr();
    if (!status) return set_error(CTGB_ERR_CUDA, "ctgb_forward: device status word unavailable");
    const int tr = fwd_tile_rows(p);
    {
        cudaError_t e = tr == 32 ? fwd_smem_limits<32>() : fwd_smem_limits<16>();
        if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "dd_forward smem attribute: %s", cudaGetErrorString(e));
    }
    const int ntu = (p->nu + kTU - 1) / kTU, ntv = (p->nv + tr - 1) / tr;
    const bool tiles_ok = (long long)ntu * ntv <= 65535;
    const float *src_x = d_vol_xzy ? d_vol_xzy : d_vol;
    const long long stk_x = d_vol_xzy ? 1LL : (long long)p->nx;

    // z-dominant views: runs of consecutive views, per-pixel kernel.
    std::vector<int> axes;
    view_axes(p, view0, nviews, axes);
    auto axis_of = [&](int i) { return (axes[i] == 2 || !tiles_ok) ? 2 : axes[i]; };
    for (int i = 0; i < nviews;) {
        int j = i + 1;
        while (j < nviews && (axis_of(j) == 2) == (axis_of(i) == 2)) ++j;
        if (axis_of(i) == 2)
            for (int v = i; v < j; v += 65535) {
                const int n = (j - v) < 65535 ? (j - v) : 65535;
                dim3 block(kFwdTileU, kFwdTileV);
                dim3 grid((p->nu + kFwdTileU - 1) / kFwdTileU, (p->nv + kFwdTileV - 1) / kFwdTileV, n);
                dd_forward_kernel<<<grid, block, 0, st>>>(T, d_vol, d_vol_xzy, d_proj + (long long)v * view_elems,
                                                          view0 + v);
            }
        i = j;
    }
    // x- and y-dominant views: one launch per axis (per kFwdListViews views).
    for (int a = 0; a < 2; ++a) {
        FwdViewList list;
        int n = 0;
        auto flush = [&]() {
            if (n == 0) return;
            const dim3 grid(n, ntu * ntv);
            const bool xd = a == 0, tma = xd ? tma_x : tma_y;
            const CUtensorMap &tm = xd ? tm_x : tm_y;
            const float *src = xd ? src_x : d_vol;
            const long long stk = xd ? stk_x : 1LL;
            if (tr == 32) launch_fwd_tma<32>(xd, tma, grid, st, tm, T, src, stk, d_proj, view0, list, ntu, status);
            else launch_fwd_tma<16>(xd, tma, grid, st, tm, T, src, stk, d_proj, view0, list, ntu, status);
            n = 0;
        };
        for (int i = 0; i < nviews; ++i) {
            if (axis_of(i) != a) continue;
            list.v[n++] = i;
            if (n == kFwdListViews) flush();
        }
        flush();
    }
    return check_launch("dd_forward");
}

extern "C" int ctgb_forward_tile_rows(const ctgb_params *p, int32_t *rows) {
    clear_error();
    if (!p || !rows) return set_error(CTGB_ERR_ARG, "ctgb_forward_tile_rows: NULL argument");
    *rows = fwd_tile_rows(p);
    return CTGB_OK;
}

extern "C" int ctgb_forward_launches(const ctgb_params *p, int32_t view0, int32_t nviews, int32_t *launches) {
    clear_error();
    if (!p || !launches) return set_error(CTGB_ERR_ARG, "ctgb_forward_launches: NULL argument");
    if (view0 < 0 || nviews < 0 || view0 + nviews > p->nviews)
        return set_error(CTGB_ERR_ARG, "ctgb_forward_launches: view range outside [0,%d)", p->nviews);
    const int tr = fwd_tile_rows(p);
    const int ntu = (p->nu + kTU - 1) / kTU, ntv = (p->nv + tr - 1) / tr;
    const bool tiles_ok = (long long)ntu * ntv <= 65535;
    std::vector<int> axes;
    view_axes(p, view0, nviews, axes);
    auto axis_of = [&](int i) { return (axes[i] == 2 || !tiles_ok) ? 2 : axes[i]; };
    int count = 0, per_axis[2] = {0, 0};
    for (int i = 0; i < nviews;) {
        int j = i + 1;
        while (j < nviews && (axis_of(j) == 2) == (axis_of(i) == 2)) ++j;
        if (axis_of(i) == 2) count += (j - i + 65534) / 65535;
        i = j;
    }
    for (int i = 0; i < nviews; ++i)
        if (axis_of(i) != 2) ++per_axis[axis_of(i)];
    for (int a = 0; a < 2; ++a) count += (per_axis[a] + kFwdListViews - 1) / kFwdListViews;
    *launches = count;
    return CTGB_OK;
}

extern "C" int ctgb_transpose_xy(const float *d_vol, float *d_vol_xzy, int32_t nx, int32_t ny, int32_t nz,
                                 void *stream) {
    clear_error();
    if (!d_vol || !d_vol_xzy || nx < 1 || ny < 1 || nz < 1 || nz > 65535)
        return set_error(CTGB_ERR_ARG, "ctgb_transpose_xy: bad arguments");
    dim3 grid((nx + 31) / 32, (ny + 31) / 32, nz), block(32, 8);
    transpose_xy_kernel<<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(d_vol, d_vol_xzy, nx, ny);
    return check_launch("transpose_xy_kernel");
}

// ---- batched forward (many scans per launch) ---------------------------------
namespace {

constexpr uint32_t kFwdPlanMagic = 0x31424643u;

struct FwdPlanGroup {
    int32_t xd, tr, njobs, nitems;
    int64_t off_jobs, off_views;
};

// Host and device copies of a plan are the same bytes: this head, then per
// group its FwdJob array (128-byte aligned, as CUtensorMap) and view list,
// then the TransJobs.
struct FwdPlanHead {
    uint32_t magic;
    int32_t ngroups;
    int32_t ntrans, trans_items;
    int64_t off_trans, total;
    FwdPlanGroup g[4];
};

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

int device_sms(int *sms) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "SM count: %s", cudaGetErrorString(e));
    return CTGB_OK;
}

// Lays the plan out (and fills it when out != nullptr).
int build_fwd_plan(const ctgb_fwd_job *jobs, int njobs, unsigned char *out, size_t bytes, size_t *need) {
    if (!jobs || njobs < 1) return set_error(CTGB_ERR_ARG, "batched forward: no jobs");
    struct Scan {
        int tr, ntu, ntiles;
        std::vector<int> views[2];   // [0] x-dominant, [1] y-dominant (relative view indices)
    };
    std::vector<Scan> sc(njobs);
    for (int i = 0; i < njobs; ++i) {
        const ctgb_fwd_job &jb = jobs[i];
        const ctgb_params *p = jb.params;
        if (!p || !jb.table || !jb.vol || !jb.out)
            return set_error(CTGB_ERR_ARG, "batched forward: job %d has a NULL argument", i);
        if (jb.view0 < 0 || jb.nviews < 0 || jb.view0 + jb.nviews > p->nviews)
            return set_error(CTGB_ERR_ARG, "batched forward: job %d view range outside the scan", i);
        if (jb.epilogue < CTGB_FWD_STORE || jb.epilogue > CTGB_FWD_EM_RATIO)
            return set_error(CTGB_ERR_ARG, "batched forward: job %d unknown epilogue %d", i, jb.epilogue);
        if (jb.epilogue != CTGB_FWD_STORE && (!jb.p0 || (jb.epilogue != CTGB_FWD_EM_RATIO && !jb.a1)))
            return set_error(CTGB_ERR_ARG, "batched forward: job %d epilogue needs p0 and a1", i);
        std::vector<int> axes;
        view_axes(p, jb.view0, jb.nviews, axes);
        sc[i].tr = fwd_tile_rows(p);
        sc[i].ntu = (p->nu + kTU - 1) / kTU;
        sc[i].ntiles = sc[i].ntu * ((p->nv + sc[i].tr - 1) / sc[i].tr);
        for (int v = 0; v < jb.nviews; ++v) {
            if (axes[v] == 2)
                return set_error(CTGB_ERR_ARG, "batched forward: job %d view %d is z-dominant (not batched)", i,
                                 jb.view0 + v);
            sc[i].views[axes[v]].push_back(v);
        }
    }
    FwdPlanHead head;
    std::memset(&head, 0, sizeof head);
    head.magic = kFwdPlanMagic;
    size_t off = align_up(sizeof head, 128);
    const int trs[2] = {32, 16};
    for (int a = 0; a < 2; ++a)
        for (int t = 0; t < 2; ++t) {
            FwdPlanGroup g;
            std::memset(&g, 0, sizeof g);
            g.xd = a == 0;
            g.tr = trs[t];
            long long items = 0, nviews = 0;
            for (int i = 0; i < njobs; ++i)
                if (sc[i].tr == g.tr && !sc[i].views[a].empty()) {
                    ++g.njobs;
                    items += (long long)sc[i].views[a].size() * sc[i].ntiles;
                    nviews += (long long)sc[i].views[a].size();
                }
            if (!g.njobs) continue;
            if (items > 0x7fffffffLL) return set_error(CTGB_ERR_SIZE, "batched forward: too many tiles");
            g.nitems = (int32_t)items;
            g.off_jobs = (int64_t)off;
            off = align_up(off + sizeof(FwdJob) * g.njobs, 128);
            g.off_views = (int64_t)off;
            off = align_up(off + sizeof(int32_t) * nviews, 128);
            head.g[head.ngroups++] = g;
        }
    long long titems = 0;
    for (int i = 0; i < njobs; ++i)
        if (jobs[i].vol_xzy && !sc[i].views[0].empty()) {
            const ctgb_params *p = jobs[i].params;
            ++head.ntrans;
            titems += (long long)((p->nx + 31) / 32) * ((p->ny + 31) / 32) * p->nz;
        }
    if (titems > 0x7fffffffLL) return set_error(CTGB_ERR_SIZE, "batched forward: too many transpose tiles");
    head.trans_items = (int32_t)titems;
    head.off_trans = (int64_t)off;
    off = align_up(off + sizeof(TransJob) * head.ntrans, 128);
    head.total = (int64_t)off;
    *need = off;
    if (!out) return CTGB_OK;
    if (bytes < off) return set_error(CTGB_ERR_SIZE, "batched forward: plan buffer of %zu bytes below %zu", bytes, off);
    std::memset(out, 0, off);
    std::memcpy(out, &head, sizeof head);
    for (int gi = 0; gi < head.ngroups; ++gi) {
        const FwdPlanGroup &g = head.g[gi];
        const int a = g.xd ? 0 : 1;
        FwdJob *dj = reinterpret_cast<FwdJob *>(out + g.off_jobs);
        int32_t *dv = reinterpret_cast<int32_t *>(out + g.off_views);
        int k = 0, item = 0, list = 0;
        for (int i = 0; i < njobs; ++i) {
            if (sc[i].tr != g.tr || sc[i].views[a].empty()) continue;
            const ctgb_fwd_job &jb = jobs[i];
            const ctgb_params *p = jb.params;
            FwdJob &f = dj[k++];
            const uint32_t box[3] = {kBoxX, 1, kBoxZ};
            bool tma;
            if (g.xd) {
                const uint64_t d[3] = {(uint64_t)p->ny, (uint64_t)p->nx, (uint64_t)p->nz};
                tma = jb.vol_xzy && p->ny % 4 == 0 && ctgb_make_tmap_3d(&f.tm, jb.vol_xzy, d, box);
                f.src = jb.vol_xzy ? jb.vol_xzy : jb.vol;
                f.st_k = jb.vol_xzy ? 1LL : (long long)p->nx;
            } else {
                const uint64_t d[3] = {(uint64_t)p->nx, (uint64_t)p->ny, (uint64_t)p->nz};
                tma = p->nx % 4 == 0 && ctgb_make_tmap_3d(&f.tm, jb.vol, d, box);
                f.src = jb.vol;
                f.st_k = 1LL;
            }
            if (!tma) std::memset(&f.tm, 0, sizeof f.tm);
            f.T = static_cast<const float *>(jb.table);
            f.proj = jb.out;
            f.view0 = jb.view0;
            f.ntu = sc[i].ntu;
            f.ntiles = sc[i].ntiles;
            f.tma = tma ? 1 : 0;
            f.item0 = item;
            f.nitems = (int)sc[i].views[a].size() * sc[i].ntiles;
            f.list0 = list;
            f.epi.mode = jb.epilogue;
            f.epi.eps = jb.eps;
            f.epi.p0 = jb.p0;
            f.epi.a1 = jb.a1;
            for (int v : sc[i].views[a]) dv[list++] = v;
            item += f.nitems;
        }
    }
    TransJob *tj = reinterpret_cast<TransJob *>(out + head.off_trans);
    int k = 0, item = 0;
    for (int i = 0; i < njobs; ++i)
        if (jobs[i].vol_xzy && !sc[i].views[0].empty()) {
            const ctgb_params *p = jobs[i].params;
            TransJob &t = tj[k++];
            t.in = jobs[i].vol;
            t.out = jobs[i].vol_xzy;
            t.nx = p->nx; t.ny = p->ny; t.nz = p->nz;
            t.tx = (p->nx + 31) / 32; t.ty = (p->ny + 31) / 32;
            t.item0 = item;
            item += t.tx * t.ty * t.nz;
        }
    return CTGB_OK;
}

template <bool XD, int TR>
cudaError_t launch_fwd_batch(const FwdPlanGroup &g, const unsigned char *d_plan, int grid, cudaStream_t st,
                             int *status) {
    static std::atomic<unsigned long long> attr;
    cudaError_t e = smem_limit_once((const void *)dd_forward_batch_kernel<XD, TR>, (int)sizeof(FwdTmaSmem<TR>), attr);
    if (e != cudaSuccess) return e;
    dd_forward_batch_kernel<XD, TR><<<grid, 32, sizeof(FwdTmaSmem<TR>), st>>>(
        reinterpret_cast<const FwdJob *>(d_plan + g.off_jobs), g.njobs,
        reinterpret_cast<const int *>(d_plan + g.off_views), g.nitems, status);
    return cudaGetLastError();
}

}  // namespace

extern "C" int ctgb_batch_forward_plan_bytes(const ctgb_fwd_job *jobs, int32_t njobs, size_t *bytes) {
    clear_error();
    if (!bytes) return set_error(CTGB_ERR_ARG, "ctgb_batch_forward_plan_bytes: NULL argument");
    return build_fwd_plan(jobs, njobs, nullptr, 0, bytes);
}

extern "C" int ctgb_batch_forward_plan(const ctgb_fwd_job *jobs, int32_t njobs, void *host_plan, size_t bytes) {
    clear_error();
    if (!host_plan) return set_error(CTGB_ERR_ARG, "ctgb_batch_forward_plan: NULL plan");
    size_t need = 0;
    return build_fwd_plan(jobs, njobs, static_cast<unsigned char *>(host_plan), bytes, &need);
}

extern "C" int ctgb_batch_forward(const void *host_plan, const void *d_plan, int32_t ctas_per_sm, void *stream) {
    clear_error();
    if (!host_plan || !d_plan || ctas_per_sm < 1)
        return set_error(CTGB_ERR_ARG, "ctgb_batch_forward: bad arguments");
    const FwdPlanHead &head = *static_cast<const FwdPlanHead *>(host_plan);
    if (head.magic != kFwdPlanMagic) return set_error(CTGB_ERR_ARG, "ctgb_batch_forward: not a forward plan");
    if (reinterpret_cast<uintptr_t>(d_plan) % 128)
        return set_error(CTGB_ERR_ARG, "ctgb_batch_forward: device plan must be 128-byte aligned");
    int sms = 0;
    if (int st = device_sms(&sms)) return st;
    int *status = ctgb_status_ptr();
    if (!status) return set_error(CTGB_ERR_CUDA, "ctgb_batch_forward: device status word unavailable");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const unsigned char *dp = static_cast<const unsigned char *>(d_plan);
    if (head.ntrans > 0) {
        const int grid = std::min(head.trans_items, sms * 16);
        transpose_xy_batch_kernel<<<grid, dim3(32, 8), 0, st>>>(reinterpret_cast<const TransJob *>(dp + head.off_trans),
                                                               head.ntrans, head.trans_items);
        if (int e = check_launch("transpose_xy_batch_kernel")) return e;
    }
    for (int gi = 0; gi < head.ngroups; ++gi) {
        const FwdPlanGroup &g = head.g[gi];
        const long long want = (long long)sms * ctas_per_sm;
        const int grid = (int)std::min<long long>(g.nitems, want);
        cudaError_t e;
        if (g.tr == 32) e = g.xd ? launch_fwd_batch<true, 32>(g, dp, grid, st, status)
                                 : launch_fwd_batch<false, 32>(g, dp, grid, st, status);
        else e = g.xd ? launch_fwd_batch<true, 16>(g, dp, grid, st, status)
                      : launch_fwd_batch<false, 16>(g, dp, grid, st, status);
        if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "dd_forward_batch_kernel: %s", cudaGetErrorString(e));
    }
    return CTGB_OK;
}
