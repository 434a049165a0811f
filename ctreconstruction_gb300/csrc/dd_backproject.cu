// DD backprojectors.
//
// 1. FDK-weighted DD backprojection, the reference's backward():
//    distance_backproj (python/Reconstruction_numba.py:371-482) with
//    flat_/curved_distance_backproj_arb (python/GPUFuncs_numba.py:391-686;
//    python/GPUFuncs_pycuda.py:837-956).  Per voxel and view: the 8 voxel
//    corners are rotated by -theta, the min/max source->corner slopes are
//    mapped onto the detector plane y = DetectorY (or to -atan(slope) for an
//    arc detector), the covered detector cells are weighted by overlap fraction
//    and the sum is scaled by R^2/(R - y_c)^2 and dtheta.
//
//    GB300 layout: one thread owns a column of voxels (fixed x, y) and keeps
//    their sums on chip across all views (no atomics; the reference launches
//    one kernel per view and atomically adds).  Everything that does not
//    depend on z — the four rotated xy corners, the u footprint, the distance
//    weight — is computed once per (column, view); per voxel only the v
//    footprint (two products and a min/max per z end) is new.  Two forms:
//    bp_fdk_walk_kernel walks the detector rows under the column on the raw
//    projections (and shares each set-up between the columns of a rotation
//    orbit on symmetric scans); bp_fdk_integ_kernel looks the rows up in
//    integrated projections.  With
//    angle2 = 0 the reference's corner slopes are (S_z - z_c) / (S_y - y_c); the
//    min/max over the 8 corners equals the min/max over {S_z - z_lo, S_z - z_hi}
//    x {min, max of 1/(S_y - y_c)}.
//
// 2. Matched DD backprojection: the exact adjoint of ctgb_forward.  Per voxel
//    and view, the candidate detector pixels are those whose projected footprint
//    can touch the voxel's cross-section on its slice (projected corners plus a
//    one-pixel margin); for each, the forward projector's own line set-up and
//    weights (dd_common.cuh) are re-evaluated on that slice, so the weight a
//    voxel receives is bit-for-bit the weight the forward gives it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "dd_common.cuh"
#include "status.h"
#include "tma.cuh"
#include "updates.cuh"

namespace ctgb {

constexpr int kBpTileX = 32, kBpTileY = 4;

// ---------------------------------------------------------------------------
// Helpers of the FDK-weighted backprojectors.  With the source outside the
// volume every corner depth 1/(S_y - y_c) is positive, so the min/max over the
// 8 corner slopes reduces to one product per z end (v_footprint).

__device__ __forceinline__ float fast_rcp(float x) { return __fdividef(1.0f, x); }

// v footprint (detector-row units) of the voxel with centre height zc: with
// every corner depth factor i = 1/(S_y - y_c) in [imin, imax], imin > 0, the
// min/max of (S_z - z_end) * i over the 8 corners are n_small * (imax if
// n_small < 0 else imin) and n_big * (imax if n_big > 0 else imin).
__device__ __forceinline__ void v_footprint(float zc, float hz, float Sz, float imin, float imax, float Mv, float Av,
                                            float *lo, float *hi) {
    const float n1 = Sz - (zc - hz), n2 = Sz - (zc + hz);
    const float ns = fminf(n1, n2), nb = fmaxf(n1, n2);
    const float a = ns * ((ns < 0.0f) ? imax : imin);
    const float b = nb * ((nb > 0.0f) ? imax : imin);
    const float va = fmaf(a, Mv, Av), vb = fmaf(b, Mv, Av);
    *lo = fminf(va, vb);
    *hi = fmaxf(va, vb);
}

// ---------------------------------------------------------------------------
// FDK-weighted DD backprojection over integrated projections (default when
// the caller supplies a workspace).
//
// integrate_rows_kernel writes, per view and detector column l, the running
// sums C(m) = sum_{m' < m} Q[m'][l] (m = 0..nv) next to Q itself as float2
// (C, Q) — the "integrated" projections.  The integral of the piecewise
// constant column over any row interval [a, b] is then
// (C + Q frac)(b) - (C + Q frac)(a): two lookups, whatever the footprint's
// size.  The backprojector (one thread per voxel column x 16 voxels, all views
// in registers) does, per voxel and view, two lookups per u cell of the
// column's footprint; within a 16-voxel chunk that does not straddle the
// source height the v footprint ends move linearly with z, so they are one
// FMA each.  Running sums are accumulated in double and stored rounded, so
// each lookup carries one float32 rounding of the prefix, not a drifting sum.
#ifndef CTGB_BI_Z
#define CTGB_BI_Z 16
#endif
constexpr int kBiZ = CTGB_BI_Z;   // z voxels per thread
#ifndef CTGB_BI_BLOCKS
#define CTGB_BI_BLOCKS 8
#endif
constexpr int kBiBlocks = CTGB_BI_BLOCKS;   // resident CTAs per SM the register budget is sized for
// CTA shape (voxel columns in x and y); warps are kBiTX x (32 / kBiTX)
// patches.  At 512^3 / 720 views, 4 x 32 took 195 ms against 210 ms for
// 32 x 4 (2 x 64: 201, 8 x 16: 199, 16 x 8: 205, 1 x 128: 211): a compact
// warp patch keeps its 32 footprints on fewer detector rows and columns at
// every view angle, so each lookup touches fewer cache lines.
#ifndef CTGB_BI_TX
#define CTGB_BI_TX 4
#endif
#ifndef CTGB_BI_TY
#define CTGB_BI_TY 32
#endif
constexpr int kBiTX = CTGB_BI_TX, kBiTY = CTGB_BI_TY;
static_assert(kBiTX * kBiTY == 128 && 32 % kBiTX == 0, "bp_fdk_integ_kernel: 128-thread CTAs of whole warps");

// Column l of view v (t = v * nu + l): running sums C(m) next to the values.
__device__ __forceinline__ void integrate_rows_one(const float *__restrict__ proj, float2 *__restrict__ out, int nu,
                                                   int nv, long long t) {
    const int v = (int)(t / nu), l = (int)(t % nu);
    const float *__restrict__ q = proj + (long long)v * nu * nv + l;
    float2 *__restrict__ o = out + (long long)v * (nv + 1) * nu + l;
    double c = 0.0;
    for (int m = 0; m < nv; ++m) {
        const float x = __ldg(q + (long long)m * nu);
        o[(long long)m * nu] = make_float2((float)c, x);
        c += x;
    }
    o[(long long)nv * nu] = make_float2((float)c, 0.0f);
}

__global__ void integrate_rows_kernel(const float *__restrict__ proj, float2 *__restrict__ out, int nu, int nv,
                                      int nviews) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)nu * nviews) return;
    integrate_rows_one(proj, out, nu, nv, t);
}

template <int NT>
__device__ __forceinline__ float integ_taps(const float2 *__restrict__ rlo, const float2 *__restrict__ rhi,
                                            float flo, float fhi, const float *ov) {
    float s = 0.0f;
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        const float2 a = __ldg(rlo + t), b = __ldg(rhi + t);
        s = fmaf(ov[t], fmaf(b.y, fhi, b.x) - fmaf(a.y, flo, a.x), s);
    }
    return s;
}

// CLAMP: some footprint of the chunk may leave the detector's rows [0, nv];
// without it every footprint lies inside (checked per warp by the caller),
// and every footprint is at least 1e-4 rows wide (also checked).
template <int NT, bool LINEAR, bool CLAMP>
__device__ __forceinline__ void integ_voxels(const float2 *__restrict__ IQ, int nu, int nv, int lbase,
                                             const float *ov, float lo0, float hi0, float dlo, float dhi,
                                             float zfirst, float dzs, float hz, float Sz, float imin, float imax,
                                             float Mv, float Av, float *acc) {
    const float fnv = (float)nv;
#pragma unroll
    for (int j = 0; j < kBiZ; ++j) {
        // Both ends as one float2: position, floor and fraction in packed
        // adds (186 ms against 190 ms with scalar ends at 512^3 / 720).
        float vlo, vhi;
        float2 v2;
        if (LINEAR) {
            v2 = __ffma2_rn(make_float2((float)j, (float)j), make_float2(dlo, dhi), make_float2(lo0, hi0));
        } else {
            v_footprint(zfirst + (float)j * dzs, hz, Sz, imin, imax, Mv, Av, &vlo, &vhi);
            v2 = make_float2(vlo, vhi);
        }
        const float rw = fast_rcp(v2.y - v2.x);
        if (CLAMP) v2 = make_float2(fminf(fmaxf(v2.x, 0.0f), fnv), fminf(fmaxf(v2.y, 0.0f), fnv));
        const float2 t2 = __fadd2_rd(v2, make_float2(12582912.0f, 12582912.0f));
        const int mlo = __float_as_int(t2.x) - 0x4B400000, mhi = __float_as_int(t2.y) - 0x4B400000;
        const float2 u2 = __ffma2_rn(__fadd2_rn(t2, make_float2(-12582912.0f, -12582912.0f)),
                                     make_float2(-1.0f, -1.0f), v2);
        const float ulo = u2.x, uhi = u2.y;
        const float2 *rlo = IQ + mlo * nu + lbase;
        const float2 *rhi = IQ + mhi * nu + lbase;
        // ov[] carries the view's distance weight; the (C, Q) pairs of each
        // end are summed over the taps with packed FMAs, 2 per tap (190 ms
        // against 196 ms for 4 scalar operations per tap at 512^3 / 720).
        float2 sa = make_float2(0.0f, 0.0f), sb = make_float2(0.0f, 0.0f);
#pragma unroll
        for (int t = 0; t < NT; ++t) {
            const float2 o2 = make_float2(ov[t], ov[t]);
            sa = __ffma2_rn(o2, __ldg(rlo + t), sa);
            sb = __ffma2_rn(o2, __ldg(rhi + t), sb);
        }
        acc[j] = fmaf(fmaf(sb.y, uhi, sb.x) - fmaf(sa.y, ulo, sa.x), rw, acc[j]);
    }
}

template <int NT, bool LINEAR>
__device__ __forceinline__ void integ_dispatch(bool clamp, const float2 *__restrict__ IQ, int nu, int nv, int lbase,
                                               const float *ov, float lo0, float hi0, float dlo, float dhi,
                                               float zfirst, float dzs, float hz, float Sz, float imin, float imax,
                                               float Mv, float Av, float *acc) {
    if (clamp)
        integ_voxels<NT, LINEAR, true>(IQ, nu, nv, lbase, ov, lo0, hi0, dlo, dhi, zfirst, dzs, hz, Sz, imin, imax,
                                       Mv, Av, acc);
    else
        integ_voxels<NT, LINEAR, false>(IQ, nu, nv, lbase, ov, lo0, hi0, dlo, dhi, zfirst, dzs, hz, Sz, imin,
                                        imax, Mv, Av, acc);
}

// Per-launch values of a backprojection (table, integrated projections,
// views, scale).  The single-scan kernels take them from their parameters,
// which the column bodies can read at any use for free.  The batched kernels
// read them from the job in global memory: JobSrc re-loads a field at every
// use (a volatile load is not hoisted out of the view loop), so the seven
// values are not held in registers across it — held there, they pushed the
// column bodies' accumulators into local memory (732-byte spills).
struct ParamSrc {
    const float *T_;
    const float2 *integ_;
    const float *tabs_, *proj_;
    int view0_, nviews_;
    float scale_;
    int vstep_ = 1;   // view vi of the call is view0 + vi * vstep (integ: slot vi)
    __device__ __forceinline__ const float *T() const { return T_; }
    __device__ __forceinline__ const float2 *integ() const { return integ_; }
    __device__ __forceinline__ const float *tabs() const { return tabs_; }
    __device__ __forceinline__ const float *proj() const { return proj_; }
    __device__ __forceinline__ int view0() const { return view0_; }
    __device__ __forceinline__ int nviews() const { return nviews_; }
    __device__ __forceinline__ float scale() const { return scale_; }
    __device__ __forceinline__ int vstep() const { return vstep_; }
};

__device__ __forceinline__ unsigned long long ld_volatile_u64(const void *p) {
    unsigned long long v;
    asm volatile("ld.global.nc.b64 %0, [%1];" : "=l"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ unsigned ld_volatile_u32(const void *p) {
    unsigned v;
    asm volatile("ld.global.nc.b32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

template <class Job>
struct JobSrc {
    const Job *jp;
    __device__ __forceinline__ const float *T() const { return reinterpret_cast<const float *>(ld_volatile_u64(&jp->T)); }
    __device__ __forceinline__ const float2 *integ() const {
        return reinterpret_cast<const float2 *>(ld_volatile_u64(&jp->integ));
    }
    __device__ __forceinline__ const float *tabs() const {
        return reinterpret_cast<const float *>(ld_volatile_u64(&jp->tabs));
    }
    __device__ __forceinline__ const float *proj() const {
        return reinterpret_cast<const float *>(ld_volatile_u64(&jp->proj));
    }
    __device__ __forceinline__ int view0() const { return (int)ld_volatile_u32(&jp->view0); }
    __device__ __forceinline__ int nviews() const { return (int)ld_volatile_u32(&jp->nviews); }
    __device__ __forceinline__ float scale() const { return __uint_as_float(ld_volatile_u32(&jp->scale)); }
    __device__ __forceinline__ int vstep() const { return 1; }
};

// CTA (bx, by, bz) of the FDK backprojection over integrated projections:
// the body of the single-scan and the batched kernels.  store(i, b) writes
// the result b of volume index i (a plain store, or an iterate's update); it
// fetches its own operands, so nothing it needs is held in registers across
// the view loop.
template <bool CURVED, class Src, class Store>
__device__ __forceinline__ void bp_fdk_column(const Src &src, int bx, int by, int bz, Store store) {
    const float *__restrict__ T0 = src.T();
    const TableHeader &h0 = header(T0);
    const int ix = bx * kBiTX + threadIdx.x;
    const int iy = by * kBiTY + threadIdx.y;
    const int z0 = bz * kBiZ;
    const bool live = ix < h0.nx && iy < h0.ny;
    const int nxh = h0.nx, nyh = h0.ny;
    const int ixc = min(ix, h0.nx - 1), iyc = min(iy, h0.ny - 1);
    const int nu = h0.nu, nv = h0.nv, nz = h0.nz;
#define T T0
#define h h0
    const float *__restrict__ ki = T + h.off_ki;
    const float *__restrict__ pp = T + h.off_pp;
    const float xx = T[h.off_xpix + ixc], yy = T[h.off_ypix + iyc];
    const float hx = h.dx * 0.5f, hy = h.dy * 0.5f, hz = h.dz * 0.5f, dzs = h.dz;
    const float du = h.du_bp, dv = h.dv_bp, inv_du = 1.0f / du, inv_dv = 1.0f / dv;
    const float ki0 = ki[0], pp0 = pp[0];
    const float Sx = h.src0x, Sy = h.src0y, Dy = h.det0y, R = h.sad;
    const float eps = h.eps_bp;
    const float zfirst = T[h.off_zpix + min(z0, nz - 1)];
    const int zlast = min(z0 + kBiZ, nz) - 1 - z0;
    const float zend = zfirst + (float)zlast * dzs;
    const float inv_zlast = zlast > 0 ? 1.0f / (float)zlast : 0.0f;
#undef T
#undef h
    float acc[kBiZ];
#pragma unroll
    for (int j = 0; j < kBiZ; ++j) acc[j] = 0.0f;

    for (int vi = 0; vi < src.nviews(); ++vi) {
        const float *__restrict__ T = src.T();
        const TableHeader &h = header(T);
        const float *__restrict__ ki = T + h.off_ki;
        const float *__restrict__ pp = T + h.off_pp;
        const float *__restrict__ V = T + h.off_views + (long long)(src.view0() + vi) * h.view_stride;
        const float cs = V[VF_COS], sn = V[VF_SIN], Sz = V[VF_BPSZ];
        const float2 *__restrict__ IQ = src.integ() + (long long)vi * (nv + 1) * nu;
        const float scale = src.scale();
        const float yc = yy * cs - xx * sn;
        float umin = INFINITY, umax = -INFINITY, imin = INFINITY, imax = -INFINITY;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float cx = xx + ((q & 1) ? hx : -hx), cy = yy + ((q & 2) ? hy : -hy);
            const float xr = cx * cs + cy * sn, yr = cy * cs - cx * sn;
            const float inv = fast_rcp(Sy - yr);
            const float su = (Sx - xr) * inv;
            umin = fminf(umin, su); umax = fmaxf(umax, su);
            imin = fminf(imin, inv); imax = fmaxf(imax, inv);
        }
        float cu1, cu2;
        if (CURVED) { cu1 = -atanf(umin); cu2 = -atanf(umax); }
        else { cu1 = fmaf(umin, Dy - Sy, Sx); cu2 = fmaf(umax, Dy - Sy, Sx); }
        const float ua = (cu1 - ki0) * inv_du, ub = (cu2 - ki0) * inv_du;
        const float ulo = fminf(ua, ub), uhi = fmaxf(ua, ub);
        float fl0;
        const int l0 = floor_split(ulo, &fl0);
        const float uw = uhi - ulo;
        const float Rd = R - yc;
        float wscale = scale * (R * R) * fast_rcp(Rd * Rd);
        float ov[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int l = l0 + t;
            const float o = fmaxf(0.0f, fminf(fl0 + (float)(t + 1), uhi) - fmaxf(fl0 + (float)t, ulo));
            ov[t] = (l >= 0 && l < nu) ? o : 0.0f;   // cells off the detector add nothing
        }
        if (uw > 1e-6f) wscale *= fast_rcp(uw);
        else { ov[0] = (l0 >= 0 && l0 < nu) ? 1.0f : 0.0f; ov[1] = ov[2] = ov[3] = 0.0f; }
        // Tap base inside the detector row; weights re-aligned only for the
        // (rare) columns whose footprint touches a detector edge.
        const bool inner = l0 >= 0 && l0 + 4 <= nu;
        const int lbase = inner ? l0 : min(max(l0, 0), max(nu - 4, 0));
        float ovb[4];
        if (__all_sync(0xffffffffu, inner)) {
#pragma unroll
            for (int t = 0; t < 4; ++t) ovb[t] = ov[t];
        } else {
            const int shift = lbase - l0;
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const int src = t + shift;
                float w = 0.0f;
#pragma unroll
                for (int k = 0; k < 4; ++k) w = (src == k) ? ov[k] : w;
                ovb[t] = w;
            }
        }
        int ntl = 1;
#pragma unroll
        for (int t = 1; t < 4; ++t) ntl = (ovb[t] > 0.0f) ? t + 1 : ntl;
        float ovw[4];   // tap weights times the distance weight
#pragma unroll
        for (int t = 0; t < 4; ++t) ovw[t] = ovb[t] * wscale;
        const float Mv = (Dy - Sy) * inv_dv, Av = (Sz - pp0) * inv_dv;
        // Linear z regime: neither z end of any voxel in the chunk crosses S_z.
        const float ztop = fmaxf(zfirst, zend) + fabsf(hz), zbot = fminf(zfirst, zend) - fabsf(hz);
        const bool linear = (Sz - ztop > 0.0f) || (Sz - zbot < 0.0f);
        float lo0, hi0, loN, hiN;
        v_footprint(zfirst, hz, Sz, imin, imax, Mv, Av, &lo0, &hi0);
        v_footprint(zend, hz, Sz, imin, imax, Mv, Av, &loN, &hiN);
        const float dlo = (loN - lo0) * inv_zlast, dhi = (hiN - hi0) * inv_zlast;
        const bool ok = live && imin > 0.0f && (uhi - fl0) <= 4.0f && nu >= 4 &&
                        fminf(hi0 - lo0, hiN - loN) > 1e-4f;
        const int nt = __reduce_max_sync(0xffffffffu, ok ? ntl : 1);
        const float fnv = (float)nv;
        const bool inside = fminf(fminf(lo0, loN), fminf(hi0, hiN)) >= 0.0f &&
                            fmaxf(fmaxf(lo0, loN), fmaxf(hi0, hiN)) <= fnv;
        // Clamped reads also for a partial last chunk, whose extrapolated
        // voxels (beyond nz) must still address rows inside [0, nv].
        const bool clamp = !__all_sync(0xffffffffu, inside || !ok) || zlast < kBiZ - 1;
        if (ok) {
            if (linear) {
                if (nt <= 2)
                    integ_dispatch<2, true>(clamp, IQ, nu, nv, lbase, ovw, lo0, hi0, dlo, dhi, zfirst, dzs, hz, Sz,
                                            imin, imax, Mv, Av, acc);
                else if (nt == 3)
                    integ_dispatch<3, true>(clamp, IQ, nu, nv, lbase, ovw, lo0, hi0, dlo, dhi, zfirst, dzs, hz, Sz,
                                            imin, imax, Mv, Av, acc);
                else
                    integ_dispatch<4, true>(clamp, IQ, nu, nv, lbase, ovw, lo0, hi0, dlo, dhi, zfirst, dzs, hz, Sz,
                                            imin, imax, Mv, Av, acc);
            } else {
                integ_voxels<4, false, true>(IQ, nu, nv, lbase, ovw, lo0, hi0, dlo, dhi, zfirst, dzs, hz, Sz, imin,
                                             imax, Mv, Av, acc);
            }
        } else if (live) {
            // Reference weight calculators on the raw values (Q = the float2's y).
            const Span us = make_span(cu1, cu2, ki0, inv_du);
            const int c0 = max(us.s, 0), c1 = min(us.e, nu - 1);
            const float abs_du = fabsf(du), abs_dv = fabsf(dv);
            const float Wd = scale * (R * R) / (Rd * Rd);
#pragma unroll
            for (int j = 0; j < kBiZ; ++j) {
                if (j > zlast) break;
                const float zc = zfirst + (float)j * dzs;
                const float nlo = Sz - (zc - hz), nhi = Sz - (zc + hz);
                const float a0 = nlo * imin, a1 = nlo * imax, a2 = nhi * imin, a3 = nhi * imax;
                const float vmn = fminf(fminf(a0, a1), fminf(a2, a3));
                const float vmx = fmaxf(fmaxf(a0, a1), fmaxf(a2, a3));
                const float cv1 = fmaf(vmn, Dy - Sy, Sz), cv2 = fmaf(vmx, Dy - Sy, Sz);
                const Span vs = make_span(cv1, cv2, pp0, inv_dv);
                const int k0 = max(vs.s, 0), k1 = min(vs.e, nv - 1);
                float sum = 0.0f;
                for (int k = k0; k <= k1; ++k) {
                    const float w1 = span_weight<true>(vs, k, pp[k], pp[k + 1], abs_dv, eps);
                    const float2 *__restrict__ qrow = IQ + (long long)k * nu;
                    float part = 0.0f;
                    for (int l = c0; l <= c1; ++l)
                        part += __ldg(qrow + l).y * span_weight<false>(us, l, ki[l], ki[l + 1], abs_du, eps);
                    sum += part * w1;
                }
                acc[j] = fmaf(sum, Wd, acc[j]);
            }
        }
    }
    if (!live) return;
#pragma unroll
    for (int j = 0; j < kBiZ; ++j) {
        const int iz = z0 + j;
        if (iz < nz) store(((long long)iz * nyh + iy) * nxh + ix, acc[j]);
    }
}

template <bool CURVED>
__global__ void __launch_bounds__(kBiTX * kBiTY, kBiBlocks)
bp_fdk_integ_kernel(const float *__restrict__ T, const float2 *__restrict__ integ, float *__restrict__ vol,
                    int view0, int nviews, float scale, int accumulate) {
    const ParamSrc src = {T, integ, nullptr, nullptr, view0, nviews, scale};
    bp_fdk_column<CURVED>(src, blockIdx.x, blockIdx.y, blockIdx.z,
                          [=](long long i, float b) { vol[i] = accumulate ? __fadd_rn(vol[i], b) : b; });
}

// ---------------------------------------------------------------------------
// FDK-weighted DD backprojection by a row walk over the raw projections.
//
// Per (voxel column, view) the u footprint's taps (columns lbase + t, overlap
// weights w_t with the distance weight folded in) hold for every voxel of the
// column, so detector row r contributes one value R(r) = sum_t w_t p[r][lbase
// + t].  The column's voxel footprints [lo, hi] (row units) move
// monotonically with z and consecutive ones overlap by less than a row, so
// the thread walks up the rows once per (column, view), keeping the R of the
// rows at the walk front in registers.  With G(r) = sum_{r' < r} R(r') and
// G(v) = G(floor v) + R(floor v) frac(v), a voxel's footprint integral
// G(hi) - G(lo), divided by the footprint's width, is the reference's
// weight_calculator1 sum over rows; the walk forms it locally, as the rows
// the voxel crosses plus the partial rows at its two ends, so no running sum
// (and no cancellation between two large ones) is involved.  Each detector row under
// the column is read once per view (NT 4-byte loads) instead of two 8-byte
// running-sum lookups per tap and voxel, and no integrated copy of the
// projections is made.
//
// Four-fold symmetry (NC = 4).  On a full circular orbit whose view count is
// a multiple of 4, with a square grid centred on the rotation axis, the
// column (x, y) at angle theta and the column (-y, x) at theta + pi/2 have the
// same rotated corners, hence the same taps and voxel footprints.  A thread
// then owns the four columns of one rotation orbit (indices (i, j), (j, n-1-i),
// (n-1-i, n-1-j), (n-1-j, i)): every (column, view) set-up and every voxel's
// footprint is computed once and serves four column-views, whose rows are
// walked side by side.
constexpr int kWkTX = 4, kWkTY = 32, kWkThreads = kWkTX * kWkTY;   // 4 x 32 columns per CTA, 4 x 8 per warp
// Z voxels per column chunk, resident CTAs per SM and the voxel loop's unroll
// factor.  The voxel sums live in shared memory (Z * NC floats per thread,
// each thread its own slots), so the voxel loop need not be unrolled: with
// the sums in registers and the loop fully unrolled, the code outgrew the
// instruction cache (stalls on instruction fetch were the largest stall
// reason) and 96 registers still spilled.
template <int NC> struct WalkShape;
template <> struct WalkShape<1> { static constexpr int Z = 16, MINB = 8, UNROLL = 1; };
template <> struct WalkShape<2> { static constexpr int Z = 16, MINB = 8, UNROLL = 1; };
// Quarter-turn orbits: at 512^3 / 720 views, with the columns paired into
// f32x2 lanes, the local voxel integrals and the row steps written out,
// Z = 14 at 7 CTAs per SM takes 106.9 ms (Z = 16 at 6: 111.2; Z = 12 at 8:
// 107.6; Z = 13 or 15 at 7: 107.8, 107.4; Z = 20 at 5: 120.3), and with the
// voxel loop unrolled by 2 104.5 ms (by 7: 111.1; by 14 it spills: 191.9).
// A longer chunk shares each (column, view) set-up between more voxels,
// fewer resident warps hide less of the row loads' latency.  (The
// running-sum walk with a counted step loop: Z = 16 at 6 121.0 ms.)
#ifndef CTGB_WALK_Z4
#define CTGB_WALK_Z4 14
#endif
#ifndef CTGB_WALK_B4
#define CTGB_WALK_B4 7
#endif
#ifndef CTGB_WALK_U4
#define CTGB_WALK_U4 2
#endif
template <> struct WalkShape<4> { static constexpr int Z = CTGB_WALK_Z4, MINB = CTGB_WALK_B4, UNROLL = CTGB_WALK_U4; };

// Walk rows upwards through one chunk of Z voxels for NC column-views.
// vb[k]: view k's projections at column lbase, row 0.  Voxel j's footprint
// comes from the linear model (lin) or from v_footprint.  CLAMP: rows outside
// [0, nv) read as zero.  The caller has checked that the footprints' rows
// grow with j, that footprints are at most 2.5 rows wide, advance at most 2.5
// rows per voxel and overlap their predecessor by under one row, so three row
// steps per voxel always suffice.  (With the source at +y and the detector
// at -y, as in every reference script, rows grow with the voxel index: row
// coordinates run opposite to z on both axes.)  Voxel j of column k adds
// into sacc[j * NC * kWkThreads + k] (sacc: this thread's slots).
template <int NC, int Z, int NT, bool CLAMP>
__device__ __forceinline__ void walk_rows(const float *const (&vb)[NC], int nu, int nv, const float (&ov)[4],
                                          bool lin, float lo0, float hi0, float dlo, float dhi,
                                          float zfirst, float dzs, float hz, float Sz, float imin, float imax,
                                          float Mv, float Av, float *sacc) {
    auto pos = [&](int j) {
        if (lin) return __ffma2_rn(make_float2((float)j, (float)j), make_float2(dlo, dhi), make_float2(lo0, hi0));
        float a, b;
        v_footprint(zfirst + (float)j * dzs, hz, Sz, imin, imax, Mv, Av, &a, &b);
        return make_float2(a, b);
    };
    // R of row r for each view; rows outside the detector read row 0 and count zero
    auto rows = [&](int r, int roff, float (&out)[NC]) {
        const bool in = !CLAMP || (unsigned)r < (unsigned)nv;
        const int off = in ? roff : 0;
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            const float *__restrict__ q = vb[k] + off;
            float t0 = 0.0f;
#pragma unroll
            for (int t = 0; t < NT; ++t) t0 = fmaf(ov[t], __ldg(q + t), t0);
            out[k] = in ? t0 : 0.0f;
        }
    };
    const float2 p0 = pos(0);
    float curf;
    int cur = floor_split(p0.x, &curf);
    int roff = cur * nu;
    // R(cur), R(cur + 1), D = R(cur) - R(cur - 1), and the voxel's integral so far
    float Rc[NC], Rn[NC], D[NC], A[NC];
    rows(cur, roff, Rc);
    rows(cur + 1, roff + nu, Rn);
#pragma unroll
    for (int k = 0; k < NC; ++k) D[k] = 0.0f;
    auto advance = [&]() {
        cur += 1;
        roff += nu;
        curf += 1.0f;
#pragma unroll
        for (int k = 0; k < NC; ++k) {
            A[k] += Rc[k];
            D[k] = Rn[k] - Rc[k];
            Rc[k] = Rn[k];
        }
        rows(cur + 1, roff + nu, Rn);
    };
#pragma unroll (WalkShape<NC>::UNROLL)
    for (int j = 0; j < Z; ++j) {
        const float2 p = pos(j);
        const float rw = fast_rcp(p.y - p.x);
        // lo lies in row cur or cur - 1: G(lo) - G(cur) = R(cur) dl - D m, with
        // dl = lo - cur and m = max(-dl, 0) (zero in row cur)
        const float dl = p.x - curf, m = __saturatef(-dl);
#pragma unroll
        for (int k = 0; k < NC; ++k) A[k] = fmaf(Rc[k], -dl, D[k] * -m);
        // at most three rows per voxel, the steps written out (111.2 against
        // 115.5 ms with a counted loop for the second and third)
        if (p.y - curf >= 1.0f) {
            advance();
            if (p.y - curf >= 1.0f) {
                advance();
                if (p.y - curf >= 1.0f) advance();
            }
        }
        const float dh = p.y - curf;
        float *__restrict__ sa = sacc + j * NC * kWkThreads;
#pragma unroll
        for (int k = 0; k < NC; ++k) sa[k] += fmaf(Rc[k], dh, A[k]) * rw;
    }
}

// The same walk for NC = 2 or 4 columns, the columns' values paired into
// float2 lanes (columns 2p and 2p + 1) so that the row sums, the running G
// and the voxel ends take one packed f32x2 operation per pair; the voxel's
// NC sums are adjacent in shared memory (one 8- or 16-byte access).
template <int NC, int Z, int NT, bool CLAMP, bool LIN>
__device__ __forceinline__ void walk_rows_packed(const float *__restrict__ proj, const int (&vb)[NC], int nu, int nv,
                                                 const float (&ov)[4], float lo0, float hi0, float dlo,
                                                 float dhi, float zfirst, float dzs, float hz, float Sz, float imin,
                                                 float imax, float Mv, float Av, float *sacc) {
    constexpr int NP = NC / 2;
    auto pos = [&](int j) {
        if (LIN) return __ffma2_rn(make_float2((float)j, (float)j), make_float2(dlo, dhi), make_float2(lo0, hi0));
        float a, b;
        v_footprint(zfirst + (float)j * dzs, hz, Sz, imin, imax, Mv, Av, &a, &b);
        return make_float2(a, b);
    };
    auto rows = [&](int r, int roff, float2 (&out)[NP]) {
        const bool in = !CLAMP || (unsigned)r < (unsigned)nv;
        const int off = in ? roff : 0;
#pragma unroll
        for (int q = 0; q < NP; ++q) {
            const float *__restrict__ a = proj + (vb[2 * q] + off);
            const float *__restrict__ b = proj + (vb[2 * q + 1] + off);
            float2 t2 = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int t = 0; t < NT; ++t)
                t2 = __ffma2_rn(make_float2(ov[t], ov[t]), make_float2(__ldg(a + t), __ldg(b + t)), t2);
            out[q] = in ? t2 : make_float2(0.0f, 0.0f);
        }
    };
    const float2 p0 = pos(0);
    float curf;
    int cur = floor_split(p0.x, &curf);
    int roff = cur * nu;
    float2 Rc[NP], Rn[NP], D[NP], A[NP];   // as in walk_rows, column pairs
    rows(cur, roff, Rc);
    rows(cur + 1, roff + nu, Rn);
#pragma unroll
    for (int q = 0; q < NP; ++q) D[q] = make_float2(0.0f, 0.0f);
    auto advance = [&]() {
        cur += 1;
        roff += nu;
        curf += 1.0f;
#pragma unroll
        for (int q = 0; q < NP; ++q) {
            A[q] = __fadd2_rn(A[q], Rc[q]);
            D[q] = __fadd2_rn(Rn[q], make_float2(-Rc[q].x, -Rc[q].y));
            Rc[q] = Rn[q];
        }
        rows(cur + 1, roff + nu, Rn);
    };
#pragma unroll (WalkShape<NC>::UNROLL)
    for (int j = 0; j < Z; ++j) {
        const float2 p = pos(j);
        const float rw = fast_rcp(p.y - p.x);
        const float dl = p.x - curf, m = __saturatef(-dl);
        const float2 ndl2 = make_float2(-dl, -dl), nm2 = make_float2(-m, -m);
#pragma unroll
        for (int q = 0; q < NP; ++q) A[q] = __ffma2_rn(Rc[q], ndl2, __fmul2_rn(D[q], nm2));
        if (p.y - curf >= 1.0f) {
            advance();
            if (p.y - curf >= 1.0f) {
                advance();
                if (p.y - curf >= 1.0f) advance();
            }
        }
        const float dh = p.y - curf;
        const float2 dh2 = make_float2(dh, dh), rw2 = make_float2(rw, rw);
        float2 v[NP];
#pragma unroll
        for (int q = 0; q < NP; ++q) v[q] = __fmul2_rn(__ffma2_rn(Rc[q], dh2, A[q]), rw2);
        float *__restrict__ sa = sacc + j * NC * kWkThreads;
        if (NC == 4) {
            float4 *a4 = reinterpret_cast<float4 *>(sa);
            float4 a = *a4;
            const float2 lo2 = __fadd2_rn(make_float2(a.x, a.y), v[0]);
            const float2 hi2 = __fadd2_rn(make_float2(a.z, a.w), v[NP - 1]);
            *a4 = make_float4(lo2.x, lo2.y, hi2.x, hi2.y);
        } else {
            float2 *a2 = reinterpret_cast<float2 *>(sa);
            *a2 = __fadd2_rn(*a2, v[0]);
        }
    }
}

// NC = 1: views [view0, view0 + nviews) of the scan, proj holding them.
// NC = 2 or 4: base views w in [view0, view0 + nviews) within the first 1/NC
// of the orbit; each w takes set-up views w + d Q (d < NC, Q = views / NC) and
// column k of the orbit reads view (w + (d + k) Q) mod views; proj holds
// every view of the scan.  The grid covers the columns (NC = 1), the lower
// half of the rows (NC = 2) or one quadrant (NC = 4).
template <bool CURVED, int NC>
__global__ void __launch_bounds__(kWkThreads, WalkShape<NC>::MINB)
bp_fdk_walk_kernel(const float *__restrict__ T, const float *__restrict__ proj, float *__restrict__ vol, int view0,
                   int nviews, float scale, int accumulate) {
    constexpr int Z = WalkShape<NC>::Z;
    // voxel j of orbit column k at sacc[j * NC * kWkThreads + k] (this thread's NC sums adjacent)
    __shared__ __align__(16) float sacc_all[Z * NC * kWkThreads];
    const int tid = threadIdx.y * kWkTX + threadIdx.x;
    float *sacc = sacc_all + tid * NC;
#pragma unroll 1
    for (int j = 0; j < Z; ++j)
#pragma unroll
        for (int k = 0; k < NC; ++k) sacc[j * NC * kWkThreads + k] = 0.0f;
    const TableHeader &h = header(T);
    const int nu = h.nu, nv = h.nv, nz = h.nz, nxh = h.nx, nyh = h.ny;
    const int ix = blockIdx.x * kWkTX + threadIdx.x;
    const int iy = blockIdx.y * kWkTY + threadIdx.y;
    const bool live = NC == 1 ? (ix < nxh && iy < nyh)
                    : NC == 2 ? (ix < nxh && iy < nyh / 2) : (ix < nxh / 2 && iy < nxh / 2);
    const int ixc = min(ix, nxh - 1), iyc = min(iy, nyh - 1);
    const int z0 = blockIdx.z * Z;
    const float *__restrict__ ki = T + h.off_ki;
    const float *__restrict__ pp = T + h.off_pp;
    const float xx = T[h.off_xpix + ixc], yy = T[h.off_ypix + iyc];
    const float hx = h.dx * 0.5f, hy = h.dy * 0.5f, hz = h.dz * 0.5f, dzs = h.dz;
    const float du = h.du_bp, dv = h.dv_bp, inv_du = 1.0f / du, inv_dv = 1.0f / dv;
    const float ki0 = ki[0], pp0 = pp[0];
    const float Sx = h.src0x, Sy = h.src0y, Dy = h.det0y, R = h.sad;
    const float eps = h.eps_bp;
    const float zfirst = T[h.off_zpix + min(z0, nz - 1)];
    const int zlast = min(z0 + Z, nz) - 1 - z0;
    const float inv_zlast = zlast > 0 ? 1.0f / (float)zlast : 0.0f;
    const int nall = h.nviews, Q = nall / NC;   // views per 1/NC turn
    const long long vstride = (long long)nu * nv;
    const float Mv = (Dy - Sy) * inv_dv;
    const float smax_base = fabsf(dzs * Mv);

    const int nsetup = NC * nviews;
#pragma unroll 1
    for (int it = 0; it < nsetup; ++it) {
        int sview;
        int pv[NC];
        if (NC == 1) {
            sview = view0 + it;
            pv[0] = it;
        } else {
            sview = view0 + it / NC + (it % NC) * Q;
#pragma unroll
            for (int k = 0; k < NC; ++k) {
                const int v = sview + k * Q;
                pv[k] = v < nall ? v : v - nall;
            }
        }
        const float *__restrict__ V = T + h.off_views + (long long)sview * h.view_stride;
        const float cs = V[VF_COS], sn = V[VF_SIN], Sz = V[VF_BPSZ];
        const float yc = yy * cs - xx * sn;
        float umin = INFINITY, umax = -INFINITY, imin = INFINITY, imax = -INFINITY;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float cxq = xx + ((q & 1) ? hx : -hx), cyq = yy + ((q & 2) ? hy : -hy);
            const float xr = cxq * cs + cyq * sn, yr = cyq * cs - cxq * sn;
            const float inv = fast_rcp(Sy - yr);
            const float su = (Sx - xr) * inv;
            umin = fminf(umin, su); umax = fmaxf(umax, su);
            imin = fminf(imin, inv); imax = fmaxf(imax, inv);
        }
        float cu1, cu2;
        if (CURVED) { cu1 = -atanf(umin); cu2 = -atanf(umax); }
        else { cu1 = fmaf(umin, Dy - Sy, Sx); cu2 = fmaf(umax, Dy - Sy, Sx); }
        const float ua = (cu1 - ki0) * inv_du, ub = (cu2 - ki0) * inv_du;
        const float ulo = fminf(ua, ub), uhi = fmaxf(ua, ub);
        float fl0;
        const int l0 = floor_split(ulo, &fl0);
        const float uw = uhi - ulo;
        const float Rd = R - yc;
        float wscale = scale * (R * R) * fast_rcp(Rd * Rd);
        float ovr[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int l = l0 + t;
            const float o = fmaxf(0.0f, fminf(fl0 + (float)(t + 1), uhi) - fmaxf(fl0 + (float)t, ulo));
            ovr[t] = (l >= 0 && l < nu) ? o : 0.0f;   // cells off the detector add nothing
        }
        if (uw > 1e-6f) wscale *= fast_rcp(uw);
        else { ovr[0] = (l0 >= 0 && l0 < nu) ? 1.0f : 0.0f; ovr[1] = ovr[2] = ovr[3] = 0.0f; }
        const bool inner = l0 >= 0 && l0 + 4 <= nu;
        const int lbase = inner ? l0 : min(max(l0, 0), max(nu - 4, 0));
        float ov[4];
        if (__all_sync(0xffffffffu, inner)) {
#pragma unroll
            for (int t = 0; t < 4; ++t) ov[t] = ovr[t] * wscale;
        } else {
            const int shift = lbase - l0;
#pragma unroll
            for (int t = 0; t < 4; ++t) {
                const int src = t + shift;
                float w = 0.0f;
#pragma unroll
                for (int k = 0; k < 4; ++k) w = (src == k) ? ovr[k] : w;
                ov[t] = w * wscale;
            }
        }
        int ntl = 1;
#pragma unroll
        for (int t = 1; t < 4; ++t) ntl = (ov[t] != 0.0f) ? t + 1 : ntl;
        const float Av = (Sz - pp0) * inv_dv;
        const float zend = zfirst + (float)zlast * dzs;
        const float ztop = fmaxf(zfirst, zfirst + (float)(Z - 1) * dzs) + fabsf(hz);
        const float zbot = fminf(zfirst, zfirst + (float)(Z - 1) * dzs) - fabsf(hz);
        const bool linear = (Sz - ztop > 0.0f) || (Sz - zbot < 0.0f);
        float lo0, hi0, loN, hiN;
        v_footprint(zfirst, hz, Sz, imin, imax, Mv, Av, &lo0, &hi0);
        v_footprint(zend, hz, Sz, imin, imax, Mv, Av, &loN, &hiN);
        const float dlo = (loN - lo0) * inv_zlast, dhi = (hiN - hi0) * inv_zlast;
        // Footprints of the first two and last two voxels: linear model, or
        // exact where the chunk straddles the source height.
        auto posx = [&](int j) {
            if (linear) return make_float2(fmaf((float)j, dlo, lo0), fmaf((float)j, dhi, hi0));
            float a, b;
            v_footprint(zfirst + (float)j * dzs, hz, Sz, imin, imax, Mv, Av, &a, &b);
            return make_float2(a, b);
        };
        const float2 fa = posx(0), fb = posx(1), fc = posx(Z - 2), fd = posx(Z - 1);
        const float wa = fa.y - fa.x, wd = fd.y - fd.x;
        const bool ok = live && imin > 0.0f && (uhi - fl0) <= 4.0f && nu >= 4 &&
                        smax_base * imax <= 2.5f && wa >= 1e-4f && wa <= 2.5f && wd >= 1e-4f && wd <= 2.5f &&
                        fa.y - fb.x < 0.999f && fc.y - fd.x < 0.999f && fb.y >= fa.y && fd.y >= fc.y &&
                        fa.x > -1e6f && fd.y < 1e6f;
        const int nt = __reduce_max_sync(0xffffffffu, ok ? ntl : 1);
        const bool inside = fa.x >= 0.0f && fd.y < (float)(nv - 1);
        const bool clamp = !__all_sync(0xffffffffu, inside || !ok);
        const bool lin = __all_sync(0xffffffffu, linear || !ok);
        if (ok) {
            const float *vb[NC];
            int vo[NC];   // element offsets of the views' column lbase (< 2^31, checked by the host)
#pragma unroll
            for (int k = 0; k < NC; ++k) {
                vb[k] = proj + (long long)pv[k] * vstride + lbase;
                vo[k] = pv[k] * (int)vstride + lbase;
            }
#define CTGB_WALK(NTV, C)                                                                                      \
    do {                                                                                                       \
        if constexpr (NC == 1)                                                                                 \
            walk_rows<NC, Z, NTV, C>(vb, nu, nv, ov, lin, lo0, hi0, dlo, dhi, zfirst, dzs, hz, Sz, imin, imax, Mv, \
                                     Av, sacc);                                                                \
        else if (lin)                                                                                          \
            walk_rows_packed<NC, Z, NTV, C, true>(proj, vo, nu, nv, ov, lo0, hi0, dlo, dhi, zfirst, dzs, hz, Sz,  \
                                                  imin, imax, Mv, Av, sacc);                                   \
        else                                                                                                   \
            walk_rows_packed<NC, Z, NTV, C, false>(proj, vo, nu, nv, ov, lo0, hi0, dlo, dhi, zfirst, dzs, hz, Sz, \
                                                   imin, imax, Mv, Av, sacc);                                  \
    } while (0)
            if (!clamp) {
                if (nt <= 2) CTGB_WALK(2, false);
                else if (nt == 3) CTGB_WALK(3, false);
                else CTGB_WALK(4, false);
            } else {
                if (nt <= 2) CTGB_WALK(2, true);
                else if (nt == 3) CTGB_WALK(3, true);
                else CTGB_WALK(4, true);
            }
#undef CTGB_WALK
        } else if (live) {
            // Reference weight calculators on the raw values.
            const Span us = make_span(cu1, cu2, ki0, inv_du);
            const int c0 = max(us.s, 0), c1 = min(us.e, nu - 1);
            const float abs_du = fabsf(du), abs_dv = fabsf(dv);
            const float Wd = scale * (R * R) / (Rd * Rd);
#pragma unroll 1
            for (int j = 0; j <= zlast; ++j) {
                const float zc = zfirst + (float)j * dzs;
                const float nlo = Sz - (zc - hz), nhi = Sz - (zc + hz);
                const float a0 = nlo * imin, a1 = nlo * imax, a2 = nhi * imin, a3 = nhi * imax;
                const float vmn = fminf(fminf(a0, a1), fminf(a2, a3));
                const float vmx = fmaxf(fmaxf(a0, a1), fmaxf(a2, a3));
                const float cv1 = fmaf(vmn, Dy - Sy, Sz), cv2 = fmaf(vmx, Dy - Sy, Sz);
                const Span vs = make_span(cv1, cv2, pp0, inv_dv);
                const int k0 = max(vs.s, 0), k1 = min(vs.e, nv - 1);
#pragma unroll
                for (int k = 0; k < NC; ++k) {
                    const float *__restrict__ Qv = proj + (long long)pv[k] * vstride;
                    float sum = 0.0f;
                    for (int r = k0; r <= k1; ++r) {
                        const float w1 = span_weight<true>(vs, r, pp[r], pp[r + 1], abs_dv, eps);
                        const float *__restrict__ qrow = Qv + (long long)r * nu;
                        float part = 0.0f;
                        for (int l = c0; l <= c1; ++l)
                            part += __ldg(qrow + l) * span_weight<false>(us, l, ki[l], ki[l + 1], abs_du, eps);
                        sum += part * w1;
                    }
                    sacc[j * NC * kWkThreads + k] += sum * Wd;
                }
            }
        }
    }
    if (!live) return;
    const int n1 = nxh - 1;
#pragma unroll
    for (int k = 0; k < NC; ++k) {
        // column k of the orbit: (i, j), (j, n-1-i), (n-1-i, n-1-j), (n-1-j, i)
        // for quarter turns, (i, j), (nx-1-i, ny-1-j) for half turns
        int cx, cy;
        if (NC == 2) {
            cx = k == 0 ? ix : n1 - ix;
            cy = k == 0 ? iy : nyh - 1 - iy;
        } else {
            cx = k == 0 ? ix : k == 1 ? iy : k == 2 ? n1 - ix : n1 - iy;
            cy = k == 0 ? iy : k == 1 ? n1 - ix : k == 2 ? n1 - iy : ix;
        }
#pragma unroll 1
        for (int j = 0; j < Z; ++j) {
            const int iz = z0 + j;
            if (iz < nz) {
                float *dst = vol + ((long long)iz * nyh + cy) * nxh + cx;
                const float b = sacc[j * NC * kWkThreads + k];
                *dst = accumulate ? __fadd_rn(*dst, b) : b;
            }
        }
    }
}

// ---- matched (adjoint) backprojector ---------------------------------------

template <int A>
__device__ __noinline__ float matched_voxel_view(const TableHeader &h, const float *__restrict__ T,
                                                const float *__restrict__ V, const ViewOffsets &vo,
                                                const float *__restrict__ Q, int ix, int iy, int iz) {
    constexpr int B1 = Axes<A>::B1, B2 = Axes<A>::B2;
    const float d[3] = {h.dx, h.dy, h.dz};
    const float *planes[3] = {T + h.off_xplane, T + h.off_yplane, T + h.off_zplane};
    const int idx[3] = {ix, iy, iz};
    const int s = idx[A], k = idx[B1], l = idx[B2];
    const float *__restrict__ pa = planes[A];
    const float *__restrict__ pb1 = planes[B1];
    const float *__restrict__ pb2 = planes[B2];
    const float pc = pa[s] + d[A] * 0.5f;
    // Candidate pixels: project the voxel's cross-section on its slice centre plane.
    float cmin = INFINITY, cmax = -INFINITY, rmin = INFINITY, rmax = -INFINITY;
    const float zb0 = V[vo.bz], dvz = V[vo.bz] - V[vo.bz + 1];   // row-boundary z step (> 0)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        float P[3];
        P[A] = pc;
        P[B1] = (q & 1) ? pb1[k + 1] : pb1[k];
        P[B2] = (q & 2) ? pb2[l + 1] : pb2[l];
        // Inverse of the forward's detector construction: detector u (flat:
        // distance along eu at depth SDD; arc: angle) and the z where the ray
        // through P meets the detector.
        const float dxs = P[0] - V[VF_SX], dys = P[1] - V[VF_SY];
        const float a = dxs * V[VF_EUX] + dys * V[VF_EUY], b = dxs * V[VF_EWX] + dys * V[VF_EWY];
        const float lam = h.curved ? h.sdd / sqrtf(a * a + b * b) : h.sdd / b;
        const float u = h.curved ? atan2f(a, b) : lam * a;
        const float cu = (u - h.u0_fwd) / h.du_fwd;
        const float zdet = V[VF_SZ] + lam * (P[2] - V[VF_SZ]);
        const float rr = (zb0 - zdet) / dvz;
        cmin = fminf(cmin, cu); cmax = fmaxf(cmax, cu);
        rmin = fminf(rmin, rr); rmax = fmaxf(rmax, rr);
    }
    const int c0 = max((int)floorf(cmin) - 1, 0), c1 = min((int)floorf(cmax) + 1, h.nu - 1);
    const int r0 = max((int)floorf(rmin) - 1, 0), r1 = min((int)floorf(rmax) + 1, h.nv - 1);
    const float p0b1 = pb1[0], p0b2 = pb2[0];
    const float inv_db1 = 1.0f / d[B1], inv_db2 = 1.0f / d[B2];
    const float abs_db1 = fabsf(d[B1]), abs_db2 = fabsf(d[B2]);
    const float eps = h.eps_fwd;
    float acc = 0.0f;
    for (int r = r0; r <= r1; ++r) {
        for (int c = c0; c <= c1; ++c) {
            const PixelLines ln = pixel_lines<A>(V, vo, r, c, fabsf(d[A]));
            const Span u = make_span(ln.sU1 * pc + ln.iU1, ln.sU2 * pc + ln.iU2, p0b1, inv_db1);
            const Span v = make_span(ln.sV1 * pc + ln.iV1, ln.sV2 * pc + ln.iV2, p0b2, inv_db2);
            if (k < u.s || k > u.e || l < v.s || l > v.e) continue;
            const float w1 = (B1 == 0) ? span_weight<false>(u, k, pb1[k], pb1[k + 1], abs_db1, eps)
                                       : span_weight<true>(u, k, pb1[k], pb1[k + 1], abs_db1, eps);
            const float w2 = (B2 == 0) ? span_weight<false>(v, l, pb2[l], pb2[l + 1], abs_db2, eps)
                                       : span_weight<true>(v, l, pb2[l], pb2[l + 1], abs_db2, eps);
            acc += __ldg(Q + (long long)r * h.nu + c) * (w1 * w2) * ln.L;
        }
    }
    return acc;
}

// Matched backprojection, sweep form, for views whose dominant axis is x or y:
// the exact transpose of dd_forward_tma_kernel's arithmetic.  A voxel column
// (ix, iy) lies in one slice s of such a view at one transverse index k, so
// the detector columns whose footprint overlaps it, and their overlaps
// ov_x, are z-independent.  For each such column the rows' z intervals
// [z'_r, z'_{r+1}] tile the z axis; spreading v_r = y[r][c] * K_rc * ov_x * g
// uniformly over row r's interval and integrating over each voxel [l, l+1]
// gives voxel l = R(l+1) - R(l) with R the running integral, evaluated by a
// merge of row boundaries and voxel boundaries.
constexpr int kMZ = 16;

__global__ void __launch_bounds__(kBpTileX * kBpTileY, 6)
bp_matched_sweep_kernel(const float *__restrict__ T, const float *__restrict__ proj, float *__restrict__ vol,
                        int view0, int nviews, float scale, int accumulate) {
    const TableHeader &h = header(T);
    const int ix = blockIdx.x * kBpTileX + threadIdx.x;
    const int iy = blockIdx.y * kBpTileY + threadIdx.y;
    const int l0 = blockIdx.z * kMZ;
    if (ix >= h.nx || iy >= h.ny) return;
    const int nu = h.nu, nv = h.nv, nz = h.nz;
    const ViewOffsets vo = view_offsets(nu, nv);
    const float *__restrict__ pzp = T + h.off_zplane;
    const float inv_dz = 1.0f / h.dz;
    float acc[kMZ];
#pragma unroll
    for (int j = 0; j < kMZ; ++j) acc[j] = 0.0f;

    for (int vi = 0; vi < nviews; ++vi) {
        const float *__restrict__ V = T + h.off_views + (long long)(view0 + vi) * h.view_stride;
        const float *__restrict__ Q = proj + (long long)vi * nu * nv;
        const int axis = (int)V[VF_AXIS];
        if (axis == 2) {
#pragma unroll
            for (int j = 0; j < kMZ; ++j)
                if (l0 + j < nz) acc[j] += matched_voxel_view<2>(h, T, V, vo, Q, ix, iy, l0 + j);
            continue;
        }
        const bool xd = axis == 0;
        const int s = xd ? ix : iy, k = xd ? iy : ix;
        const float *__restrict__ pa = T + (xd ? h.off_xplane : h.off_yplane);
        const float *__restrict__ pb = T + (xd ? h.off_yplane : h.off_xplane);
        const float da = xd ? h.dx : h.dy, db = xd ? h.dy : h.dx;
        const float Sa = xd ? V[VF_SX] : V[VF_SY], Sb = xd ? V[VF_SY] : V[VF_SX], Sz = V[VF_SZ];
        const float *__restrict__ Ba = V + (xd ? vo.bx : vo.by);
        const float *__restrict__ Bb = V + (xd ? vo.by : vo.bx);
        const float *__restrict__ Pa = V + (xd ? vo.px : vo.py);
        const float *__restrict__ Pb = V + (xd ? vo.py : vo.px);
        const float *__restrict__ Pzr = V + vo.pz;
        const float inv_db = 1.0f / db;
        const float Cb = (Sb - pb[0]) * inv_db;
        const float A = (Sz - pzp[0]) * inv_dz;
        const float B0 = V[VF_B0], dB = V[VF_DB];
        const float q = pa[s] + 0.5f * da - Sa;
        const float g = 1.0f / (q * q);
        // Candidate columns: project the voxel's b1 edges on the slice centre plane.
        float cmin = INFINITY, cmax = -INFINITY;
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const float bw = pb[k + e];
            const float ddx = (xd ? pa[s] + 0.5f * da : bw) - V[VF_SX];
            const float ddy = (xd ? bw : pa[s] + 0.5f * da) - V[VF_SY];
            const float aa = ddx * V[VF_EUX] + ddy * V[VF_EUY], bb = ddx * V[VF_EWX] + ddy * V[VF_EWY];
            const float u = h.curved ? atan2f(aa, bb) : h.sdd * aa / bb;
            const float cu = (u - h.u0_fwd) / h.du_fwd;
            cmin = fminf(cmin, cu); cmax = fmaxf(cmax, cu);
        }
        const int cA = max((int)floorf(cmin) - 1, 0), cB = min((int)floorf(cmax) + 1, nu - 1);
        const float kf = (float)k;
        for (int c = cA; c <= cB; ++c) {
            const float Eb0 = (Sb - Bb[c]) / (Sa - Ba[c]) * inv_db;
            const float Eb1 = (Sb - Bb[c + 1]) / (Sa - Ba[c + 1]) * inv_db;
            const float xa = fmaf(Eb0, q, Cb), xb = fmaf(Eb1, q, Cb);
            const float lo = fminf(xa, xb), hi = fmaxf(xa, xb);
            const float ovx = fminf(kf + 1.0f, hi) - fmaxf(kf, lo);
            if (!(ovx > 0.0f)) continue;
            const float invD = 1.0f / (Sa - Pa[c]);
            const float t1 = (Sb - Pb[c]) * invD;
            const float tau = q * invD;
            const float base = fabsf(da) * sqrtf(1.0f + t1 * t1) / (fabsf(Eb1 - Eb0) * fabsf(invD));
            const float vscale = ovx * g * base;
            // First row whose lower boundary lies above voxel boundary l0.
            const int rs = min(max((int)floorf(((float)l0 - A) / (tau * dB) - B0 / dB) - 1, 0), nv);
            // Rows rs + i in the frame of row rs (local z: the frame's integer
            // part removed), placed as the forward places them.
            const ZFrame zf = row_frame(A, tau, B0, dB, (float)rs);
            int r = rs, i = 0;
            // Row r spans [zr, zr1]; C = running integral up to zr.
            float zr = zf.f;
            float C = 0.0f, vr = 0.0f, zr1 = zr;
            bool have_row = false;
            auto load_row = [&]() {
                if (r < nv) {
                    zr1 = fmaf((float)(i + 1), zf.sg, zf.f);
                    const float t2 = (Sz - Pzr[r]) * invD;
                    const float K = sqrtf(1.0f + t2 * t2) / fabsf(dB);
                    vr = __ldg(Q + (long long)r * nu + c) * K * vscale;
                    have_row = true;
                } else {
                    have_row = false;
                    vr = 0.0f;
                }
            };
            load_row();
            float Rprev = 0.0f;
#pragma unroll
            for (int j = 0; j <= kMZ; ++j) {
                const float lb = (float)(l0 + j) - zf.ibf;   // voxel boundary, local z
                // Advance past rows that end at or below this voxel boundary.
                while (have_row && zr1 <= lb) {
                    C += vr * (zr1 - zr);
                    zr = zr1;
                    ++r;
                    ++i;
                    load_row();
                }
                const float Rb = C + ((have_row && lb > zr) ? vr * (lb - zr) : 0.0f);
                if (j > 0) acc[j - 1] += Rb - Rprev;
                Rprev = Rb;
            }
        }
    }
#pragma unroll
    for (int j = 0; j < kMZ; ++j) {
        const int iz = l0 + j;
        if (iz < nz) {
            float *dst = vol + ((long long)iz * h.ny + iy) * h.nx + ix;
            *dst = accumulate ? *dst + scale * acc[j] : scale * acc[j];
        }
    }
}

// Matched backprojection over prescaled, integrated projections (default when
// the caller supplies a workspace).  For x/y-dominant views the forward gives
// pixel (r, c) the weight K_rc * g_s * ov_x(c; k, s) * ov_z(r; l, s) on voxel
// (k, s, l) with ov_z the overlap, in voxel units, of row r's z interval on
// slice s with [l, l+1].  The rows of column c tile that axis with a pitch of
// |dB * tau_c| voxels, so sum_r y'_r ov_z = |dB tau_c| (C(r_hi) - C(r_lo)),
// C the running sum of y' = y * K down the column and r_lo, r_hi the voxel's
// boundaries in row coordinates.  matched_integrate_kernel writes (C, y') as
// float2; z-dominant views read the raw projections instead.
// Per view, after the chunk's integrated rows: the forward's boundary slopes
// Eb[c] = (Sb - Bb[c]) / (Sa - Ba[c]) / db for c = 0 .. nu and the depth
// factors 1 / (Sa - Pa[c]) for c = 0 .. nu - 1, written once here with the
// forward's expressions so the backprojector's candidate search reads them
// instead of dividing per voxel column (the search was most of its time).
__host__ __device__ __forceinline__ int matched_tab_stride(int nu) { return 2 * nu + 2; }

// The forward's per-pixel factor K = base * sqrt(1 + t2^2) / rowspan of
// column c of view V (dd_forward_tma_kernel's epilogue, same expressions),
// with the view's column table entries written to tab on the way.
struct MatchedColumn {
    int axis;
    float base, invD, Sz, rowspan;
    const float *Pzr;
    __device__ __forceinline__ float K(int r) const {
        const float t2 = (Sz - Pzr[r]) * invD;
        return base * sqrtf(1.0f + t2 * t2) / rowspan;
    }
};

__device__ __forceinline__ MatchedColumn matched_column_setup(const TableHeader &h, const float *__restrict__ V,
                                                              const ViewOffsets &vo, int c, float *__restrict__ tab) {
    const int nu = h.nu;
    MatchedColumn mc;
    mc.axis = (int)V[VF_AXIS];
    mc.base = 0.0f; mc.invD = 0.0f; mc.Sz = 0.0f; mc.rowspan = 1.0f;   // z-dominant: unused, finite
    mc.Pzr = V + vo.pz;
    if (mc.axis == 2) return mc;
    const bool xd = mc.axis == 0;
    const float Sa = xd ? V[VF_SX] : V[VF_SY], Sb = xd ? V[VF_SY] : V[VF_SX];
    const float *__restrict__ Ba = V + (xd ? vo.bx : vo.by);
    const float *__restrict__ Bb = V + (xd ? vo.by : vo.bx);
    const float *__restrict__ Pa = V + (xd ? vo.px : vo.py);
    const float *__restrict__ Pb = V + (xd ? vo.py : vo.px);
    const float da = xd ? h.dx : h.dy, db = xd ? h.dy : h.dx;
    const float inv_db = 1.0f / db;
    const float Eb0 = (Sb - Bb[c]) / (Sa - Ba[c]) * inv_db;
    const float Eb1 = (Sb - Bb[c + 1]) / (Sa - Ba[c + 1]) * inv_db;
    mc.invD = 1.0f / (Sa - Pa[c]);
    tab[c] = Eb0;
    if (c == nu - 1) tab[nu] = Eb1;
    tab[nu + 1 + c] = mc.invD;
    const float t1 = (Sb - Pb[c]) * mc.invD;
    mc.base = fabsf(da) * sqrtf(1.0f + t1 * t1) / (fabsf(Eb1 - Eb0) * fabsf(mc.invD));
    mc.rowspan = fabsf(V[VF_DB]);
    mc.Sz = V[VF_SZ];
    return mc;
}

// Column c of the call's view vi (t = vi * nu + c; view view0 + vi * vstep,
// its projections at proj + vi * vstep views, its table at tabs + vi * vstep
// tables, its integrated rows in slot vi of out) of the matched
// backprojector's integration pass.
__device__ __forceinline__ void matched_integrate_one(const float *__restrict__ T, const float *__restrict__ proj,
                                                      float2 *__restrict__ out, float *__restrict__ tabs, int view0,
                                                      int vstep, long long t) {
    const TableHeader &h = header(T);
    const int nu = h.nu, nv = h.nv;
    const int vi = (int)(t / nu), c = (int)(t % nu);
    const ViewOffsets vo = view_offsets(nu, nv);
    const float *__restrict__ V = T + h.off_views + (long long)(view0 + vi * vstep) * h.view_stride;
    const float *__restrict__ q = proj + (long long)vi * vstep * nu * nv + c;
    float2 *__restrict__ o = out + (long long)vi * (nv + 1) * nu + c;
    const MatchedColumn mc =
        matched_column_setup(h, V, vo, c, tabs + (long long)vi * vstep * matched_tab_stride(nu));
    if (mc.axis == 2) {
        for (int r = 0; r < nv; ++r) o[(long long)r * nu] = make_float2(0.0f, __ldg(q + (long long)r * nu));
        o[(long long)nv * nu] = make_float2(0.0f, 0.0f);
        return;
    }
    double run = 0.0;
    for (int r = 0; r < nv; ++r) {
        const float y = __ldg(q + (long long)r * nu) * mc.K(r);
        o[(long long)r * nu] = make_float2((float)run, y);
        run += y;
    }
    o[(long long)nv * nu] = make_float2((float)run, 0.0f);
}

// The integration pass for the quarter-turn orbit kernel: per row boundary
// r, one 32-byte cell {C_0..C_3, y'_0..y'_3} at ((w * (nv + 1) + r) * nu + c)
// holds column c of the four views w + k Q (Q = views / 4), so the orbit
// kernel's four lookups of a row boundary are two adjacent 16-byte loads.
// Thread 4 g + k integrates view w + k Q of cell column g = w * nu + c: the
// four threads of a cell are neighbouring lanes, whose stores fill the same
// sector.  Values and tables as matched_integrate_one (the same expressions
// per view).
__global__ void matched_integrate_orbit_kernel(const float *__restrict__ T, const float *__restrict__ proj,
                                               float *__restrict__ out, float *__restrict__ tabs) {
    const TableHeader &h = header(T);
    const int nu = h.nu, nv = h.nv, Q = h.nviews / 4;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= 4LL * nu * Q) return;
    const int k = (int)(t & 3);
    const long long g = t >> 2;
    const int w = (int)(g / nu), c = (int)(g % nu), v = w + k * Q;
    const ViewOffsets vo = view_offsets(nu, nv);
    const float *__restrict__ V = T + h.off_views + (long long)v * h.view_stride;
    const MatchedColumn mc = matched_column_setup(h, V, vo, c, tabs + (long long)v * matched_tab_stride(nu));
    const float *__restrict__ q = proj + (long long)v * nu * nv + c;
    float *__restrict__ o = out + ((long long)w * (nv + 1) * nu + c) * 8 + k;
    const long long rstride = (long long)nu * 8;
    if (mc.axis == 2) {
        for (int r = 0; r < nv; ++r) {
            o[r * rstride] = 0.0f;
            o[r * rstride + 4] = __ldg(q + (long long)r * nu);
        }
        o[nv * rstride] = 0.0f;
        o[nv * rstride + 4] = 0.0f;
        return;
    }
    double run = 0.0;
    for (int r = 0; r < nv; ++r) {
        const float y = __ldg(q + (long long)r * nu) * mc.K(r);
        o[r * rstride] = (float)run;
        o[r * rstride + 4] = y;
        run += y;
    }
    o[nv * rstride] = (float)run;
    o[nv * rstride + 4] = 0.0f;
}

__global__ void matched_integrate_kernel(const float *__restrict__ T, const float *__restrict__ proj,
                                         float2 *__restrict__ out, float *__restrict__ tabs, int view0,
                                         int nviews, int vstep) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)header(T).nu * nviews) return;
    matched_integrate_one(T, proj, out, tabs, view0, vstep, t);
}

constexpr int kMC = 6;   // detector columns kept per (voxel column, view); more -> per-voxel path

#ifndef CTGB_MI_BLOCKS
#define CTGB_MI_BLOCKS 6
#endif
// CTA shape of bp_matched_integ_kernel (voxel columns in x and y).  At
// 512^3 / 720 views 32 x 4 took 339.7 ms, 8 x 16 339.8, 4 x 32 345.1: the
// shared-boundary lookups do not gain from a compact warp patch.
#ifndef CTGB_MI_TX
#define CTGB_MI_TX 32
#endif
#ifndef CTGB_MI_TY
#define CTGB_MI_TY 4
#endif
constexpr int kMiTX = CTGB_MI_TX, kMiTY = CTGB_MI_TY;
static_assert(kMiTX * kMiTY == 128 && 32 % kMiTX == 0, "bp_matched_integ_kernel: 128-thread CTAs of whole warps");

// CTA (bx, by, bz) of the matched backprojection over prescaled, integrated
// projections: the body of the single-scan and the batched kernels; store as
// for bp_fdk_column (it receives A^T r before the scale).
template <class Src, class Store>
__device__ __forceinline__ void bp_matched_column(const Src &src, int bx, int by, int bz, Store store) {
    const TableHeader &h = header(src.T());
    const int ix = bx * kMiTX + threadIdx.x;
    const int iy = by * kMiTY + threadIdx.y;
    const int l0 = bz * kMZ;
    const bool live = ix < h.nx && iy < h.ny;
    const int ixc = min(ix, h.nx - 1), iyc = min(iy, h.ny - 1);
    const int nu = h.nu, nv = h.nv, nz = h.nz;
    const ViewOffsets vo = view_offsets(nu, nv);
    const float inv_dz = 1.0f / h.dz;
    const float fnv = (float)nv;
    const int nxh = h.nx, nyh = h.ny;
    float acc[kMZ];
#pragma unroll
    for (int j = 0; j < kMZ; ++j) acc[j] = 0.0f;

    for (int vi = 0; vi < src.nviews(); ++vi) {
        const float *__restrict__ T = src.T();
        const TableHeader &h = header(T);
        const float *__restrict__ pzp = T + h.off_zplane;
        const float *__restrict__ V = T + h.off_views + (long long)(src.view0() + vi * src.vstep()) * h.view_stride;
        const float2 *__restrict__ IQ = src.integ() + (long long)vi * (nv + 1) * nu;
        const int axis = (int)V[VF_AXIS];
        const float *__restrict__ Qraw = src.proj() + (long long)vi * src.vstep() * nu * nv;
        if (axis == 2) {
            // z-dominant: per-voxel candidate search on the raw values.
            if (!live) continue;
#pragma unroll
            for (int j = 0; j < kMZ; ++j)
                if (l0 + j < nz) acc[j] += matched_voxel_view<2>(h, T, V, vo, Qraw, ixc, iyc, l0 + j);
            continue;
        }
        const bool xd = axis == 0;
        const int s = xd ? ixc : iyc, k = xd ? iyc : ixc;
        const float *__restrict__ pa = T + (xd ? h.off_xplane : h.off_yplane);
        const float *__restrict__ pb = T + (xd ? h.off_yplane : h.off_xplane);
        const float da = xd ? h.dx : h.dy, db = xd ? h.dy : h.dx;
        const float Sa = xd ? V[VF_SX] : V[VF_SY], Sb = xd ? V[VF_SY] : V[VF_SX], Sz = V[VF_SZ];
        const float inv_db = 1.0f / db;
        const float Cb = (Sb - pb[0]) * inv_db;
        const float A = (Sz - pzp[0]) * inv_dz;
        const float q = pa[s] + 0.5f * da - Sa;
        const float g = 1.0f / (q * q);
        const float B0 = V[VF_B0], dB = V[VF_DB];                     // row boundary r: B0 + r dB
        // Candidate columns: project the voxel's transverse edges on the slice centre plane.
        float cmin = INFINITY, cmax = -INFINITY;
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const float bw = pb[k + e];
            const float pcw = pa[s] + 0.5f * da;
            const float ddx = (xd ? pcw : bw) - V[VF_SX];
            const float ddy = (xd ? bw : pcw) - V[VF_SY];
            const float aa = ddx * V[VF_EUX] + ddy * V[VF_EUY], bb = ddx * V[VF_EWX] + ddy * V[VF_EWY];
            const float u = h.curved ? atan2f(aa, bb) : h.sdd * aa / bb;
            const float cu = (u - h.u0_fwd) / h.du_fwd;
            cmin = fminf(cmin, cu); cmax = fmaxf(cmax, cu);
        }
        const int cA = max((int)floorf(cmin) - 1, 0), cB = min((int)floorf(cmax) + 1, nu - 1);
        const float kf = (float)k;
        // Up to kMC columns with ov_x > 0 (the same x' expressions as the forward).
        const float *__restrict__ EbT = src.tabs() + (long long)vi * src.vstep() * matched_tab_stride(nu);
        const float *__restrict__ IPT = EbT + nu + 1;
        int ncol = 0;
        int cc[kMC];
        float wcol[kMC], tw[kMC], be[kMC];
#pragma unroll
        for (int m = 0; m < kMC; ++m) { cc[m] = 0; wcol[m] = 0.0f; tw[m] = 0.0f; be[m] = 0.0f; }
        bool overflow = false;
        for (int c = cA; c <= cB; ++c) {
            const float Eb0 = __ldg(EbT + c), Eb1 = __ldg(EbT + c + 1);
            const float xa = fmaf(Eb0, q, Cb), xb = fmaf(Eb1, q, Cb);
            const float ovx = fminf(kf + 1.0f, fmaxf(xa, xb)) - fmaxf(kf, fminf(xa, xb));
            if (!(ovx > 0.0f)) continue;
            const float tau = q * __ldg(IPT + c);
            // voxel boundary z' -> row coordinate: r = ((z' - A) / tau - B0) / dB
            const float inv = 1.0f / (tau * dB);
            const float wz = fabsf(dB * tau);
            if (ncol < kMC) {
#pragma unroll
                for (int m = 0; m < kMC; ++m)
                    if (m == ncol) { cc[m] = c; wcol[m] = ovx * g * wz; tw[m] = tau; be[m] = inv; }
                ++ncol;
            } else {
                overflow = true;
            }
        }
        if (overflow) {
            // Detector columns much narrower than a voxel: per-voxel search.
            if (!live) continue;
#pragma unroll
            for (int j = 0; j < kMZ; ++j) {
                if (l0 + j >= nz) continue;
                acc[j] += xd ? matched_voxel_view<0>(h, T, V, vo, Qraw, ixc, iyc, l0 + j)
                             : matched_voxel_view<1>(h, T, V, vo, Qraw, ixc, iyc, l0 + j);
            }
            continue;
        }
        if (!live) continue;
        // Voxel j spans row coordinates [r_j, r_{j+1}]: consecutive voxels
        // share a boundary, so each of the kMZ + 1 boundaries is clamped to
        // [0, nv] and looked up once, and voxel j takes e(r_{j+1}) - e(r_j)
        // with e(r) = C + frac * y', signed by the orientation of be.  The
        // row coordinate of boundary l is found in the frame of row R near
        // the chunk (row_frame: the forward's row placement, exact to ~1e-6
        // voxel): r = R + ((l - ibf) - f) / (tau dB), so rows are placed as
        // the forward places them and the weights agree to float rounding
        // of small local coordinates.
        const float b0r = B0 / dB;
#pragma unroll
        for (int m = 0; m < kMC; ++m) {
            if (m >= ncol) break;
            const float2 *__restrict__ colp = IQ + cc[m];
            const float w = be[m] > 0.0f ? wcol[m] : -wcol[m];
            const int R = min(max((int)floorf(fmaf((float)l0 - A, be[m], -b0r)), 0), nv);
            const ZFrame zf = row_frame(A, tw[m], B0, dB, (float)R);
            const float d0 = ((float)l0 - zf.ibf) - zf.f;                 // local z of boundary l0
            const float rlo = -(float)R, rhi = fnv - (float)R;          // rows 0 and nv, relative to R
            float eprev = 0.0f;
#pragma unroll
            for (int j = 0; j <= kMZ; ++j) {
                const float rr = fminf(fmaxf((d0 + (float)j) * be[m], rlo), rhi);   // rows past R
                float fr;
                const int mr = R + floor_split(rr, &fr);
                const float2 a = __ldg(colp + (long long)mr * nu);
                const float e = fmaf(a.y, rr - fr, a.x);
                if (j > 0) acc[j - 1] = fmaf(e - eprev, w, acc[j - 1]);
                eprev = e;
            }
        }
    }
    if (!live) return;
#pragma unroll
    for (int j = 0; j < kMZ; ++j) {
        const int iz = l0 + j;
        if (iz < nz) store(((long long)iz * nyh + iy) * nxh + ix, acc[j]);
    }
}

__global__ void __launch_bounds__(kMiTX * kMiTY, CTGB_MI_BLOCKS)
bp_matched_integ_kernel(const float *__restrict__ T, const float2 *__restrict__ integ,
                        const float *__restrict__ tabs, const float *__restrict__ proj, float *__restrict__ vol,
                        int view0, int nviews, float scale, int accumulate, int vstep) {
    const ParamSrc src = {T, integ, tabs, proj, view0, nviews, scale, vstep};
    bp_matched_column(src, blockIdx.x, blockIdx.y, blockIdx.z,
                      [=](long long i, float a) {
                          const float b = __fmul_rn(scale, a);
                          vol[i] = accumulate ? __fadd_rn(vol[i], b) : b;
                      });
}

// ---------------------------------------------------------------------------
// Matched backprojection over a quarter-turn-symmetric orbit.
//
// With a square grid centred on the rotation axis, forward planes centred
// there too and a full circular orbit whose view count is a multiple of 4
// (the conditions of the FDK walk's orbits), the forward projector's
// geometry of column (x, y) at view v is that of column (-y, x) at view
// v + Q (Q = views / 4): the same slice distance, candidate detector columns,
// transverse overlaps and row placement (to float rounding of the table's
// per-view values, which a quarter turn maps onto each other).  A thread
// owns the four columns of one rotation orbit (the grid covers a quadrant):
// per set-up view it searches the candidate columns and places their rows
// once, and per z boundary it computes the row coordinate, floor and
// fraction once; only the four (C, y') values and sums are per column.
// matched_integrate_orbit_kernel stores the four views w + t Q of a base
// view w side by side per cell, so a boundary's four lookups are two
// adjacent 16-byte loads and the columns' sums run in f32x2 pairs (183.5
// -> 162.9 ms per call at 512^3 / 720 views against four 8-byte lookups in
// four views' separate rows).  Set-up view w + s4 Q reads slot (s4 + k) & 3
// for orbit column k, so the sums are kept in slot order and rotate by one
// slot between quarter turns.
// At 512^3 / 720 views (four 8-byte lookups): 12 voxels per chunk at 4 CTAs
// per SM (128 registers) 137.9 ms for the kernel; 8 at 5 155.1, 8 at 6
// 260.1 and 12 at 5 288.0 (both spill in the lookup loop), 16 at 4 296.8.
#ifndef CTGB_MO_Z
#define CTGB_MO_Z 12
#endif
#ifndef CTGB_MO_B
#define CTGB_MO_B 4
#endif
constexpr int kMoZ = CTGB_MO_Z;

__global__ void __launch_bounds__(kMiTX * kMiTY, CTGB_MO_B)
bp_matched_orbit_kernel(const float *__restrict__ T, const float4 *__restrict__ integ,
                        const float *__restrict__ tabs, const float *__restrict__ proj, float *__restrict__ vol,
                        float scale, int accumulate) {
    // Candidate columns of the current set-up view, per thread (registers
    // held them across the lookup loop at the cost of spills).
    __shared__ float cand[7][kMC][kMiTX * kMiTY];   // column, 4 weights (slot order), tau, 1 / (tau dB)
    const int tid = threadIdx.y * kMiTX + threadIdx.x;
    const TableHeader &h = header(T);
    const int n = h.nx, hn = n / 2, n1 = n - 1;
    const int ix = blockIdx.x * kMiTX + threadIdx.x;
    const int iy = blockIdx.y * kMiTY + threadIdx.y;
    const int l0 = blockIdx.z * kMoZ;
    const bool live = ix < hn && iy < hn;
    const int ixc = min(ix, n1), iyc = min(iy, n1);
    const int nu = h.nu, nv = h.nv, nz = h.nz, nall = h.nviews, Q = nall / 4;
    const ViewOffsets vo = view_offsets(nu, nv);
    const float inv_dz = 1.0f / h.dz;
    const float fnv = (float)nv;
    const int cstride = (nv + 1) * nu;   // cells per base view
    // orbit columns: (i, j), (j, n-1-i), (n-1-i, n-1-j), (n-1-j, i)
    auto ocx = [&](int k) { return k == 0 ? ixc : k == 1 ? iyc : k == 2 ? n1 - ixc : n1 - iyc; };
    auto ocy = [&](int k) { return k == 0 ? iyc : k == 1 ? n1 - ixc : k == 2 ? n1 - iyc : ixc; };
    // Sums in slot order: in quarter turn s4 of the set-up views, slot t
    // (view w + t Q of a cell) belongs to orbit column (t - s4) & 3; the slots
    // rotate by one between quarter turns, and after the fourth slot k holds
    // column k.  accp[0][j] = slots 0, 1 of voxel j; accp[1][j] = slots 2, 3.
    float2 accp[2][kMoZ];
#pragma unroll
    for (int j = 0; j < kMoZ; ++j) accp[0][j] = accp[1][j] = make_float2(0.0f, 0.0f);
    int s4 = 0;
    // column k's value v into voxel j (k and j known at compile time)
    auto addcol = [&](int k, int j, float v) {
        const int t = (s4 + k) & 3;
        accp[0][j].x += t == 0 ? v : 0.0f;
        accp[0][j].y += t == 1 ? v : 0.0f;
        accp[1][j].x += t == 2 ? v : 0.0f;
        accp[1][j].y += t == 3 ? v : 0.0f;
    };

#pragma unroll 1
    for (int sv = 0; sv < nall; ++sv) {
        if (sv > 0 && sv % Q == 0) {
            // next quarter turn: slot t takes the sums of slot t - 1
#pragma unroll
            for (int j = 0; j < kMoZ; ++j) {
                const float2 a = accp[0][j], b = accp[1][j];
                accp[0][j] = make_float2(b.y, a.x);
                accp[1][j] = make_float2(a.y, b.x);
            }
            ++s4;
        }
        const int w = sv - s4 * Q;   // base view: the cell of views w + t Q
        int pv[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) pv[k] = w + ((s4 + k) & 3) * Q;
        const float *__restrict__ pzp = T + h.off_zplane;
        const float *__restrict__ V = T + h.off_views + (long long)sv * h.view_stride;
        const int axis = (int)V[VF_AXIS];
        // A group whose dominant axis does not alternate (45-degree ties) is
        // backprojected view by view by the host's follow-up launches.
        bool group_ok = true;
#pragma unroll
        for (int k = 1; k < 4; ++k)
            group_ok = group_ok && (int)T[h.off_views + (long long)pv[k] * h.view_stride + VF_AXIS] == (axis ^ (k & 1));
        if (!group_ok) continue;
        if (axis == 2) {
            // z-dominant (not on a circular orbit): per-voxel search per column
            if (!live) continue;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float *__restrict__ Vk = T + h.off_views + (long long)pv[k] * h.view_stride;
                const float *__restrict__ Qk = proj + (long long)pv[k] * nu * nv;
                const int ak = (int)Vk[VF_AXIS];
#pragma unroll
                for (int j = 0; j < kMoZ; ++j) {
                    if (l0 + j >= nz) continue;
                    addcol(k, j, ak == 0 ? matched_voxel_view<0>(h, T, Vk, vo, Qk, ocx(k), ocy(k), l0 + j)
                               : ak == 1 ? matched_voxel_view<1>(h, T, Vk, vo, Qk, ocx(k), ocy(k), l0 + j)
                                         : matched_voxel_view<2>(h, T, Vk, vo, Qk, ocx(k), ocy(k), l0 + j));
                }
            }
            continue;
        }
        const bool xd = axis == 0;
        const int s = xd ? ixc : iyc, kk = xd ? iyc : ixc;
        const float *__restrict__ pa = T + (xd ? h.off_xplane : h.off_yplane);
        const float *__restrict__ pb = T + (xd ? h.off_yplane : h.off_xplane);
        const float da = xd ? h.dx : h.dy;
        const float Sz = V[VF_SZ];
        const float A = (Sz - pzp[0]) * inv_dz;
        const float q = pa[s] + 0.5f * da - (xd ? V[VF_SX] : V[VF_SY]);
        const float B0 = V[VF_B0], dB = V[VF_DB];
        // Per orbit column k (view sv + k Q, dominant axis alternating): the
        // forward's own transverse frame.  The slice distance is +-q exactly
        // (the host checks the slice centres' antisymmetry), so 1/q^2, the
        // depth factor tau and the row placement are shared; the transverse
        // coordinate x = Eb q + Cb and its overlap with cell kk are evaluated
        // per column with that view's expressions (as mirror images they
        // round differently).
        float qk[4], cbk[4], kfk[4], gk[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const bool xdk = (axis ^ (k & 1)) == 0;
            const float *__restrict__ Vk = T + h.off_views + (long long)pv[k] * h.view_stride;
            const int cxk = ocx(k), cyk = ocy(k);
            const int sk = xdk ? cxk : cyk;
            const float *__restrict__ pak = T + (xdk ? h.off_xplane : h.off_yplane);
            const float *__restrict__ pbk = T + (xdk ? h.off_yplane : h.off_xplane);
            const float dak = xdk ? h.dx : h.dy, dbk = xdk ? h.dy : h.dx;
            const float Sak = xdk ? Vk[VF_SX] : Vk[VF_SY], Sbk = xdk ? Vk[VF_SY] : Vk[VF_SX];
            qk[k] = pak[sk] + 0.5f * dak - Sak;
            cbk[k] = (Sbk - pbk[0]) * (1.0f / dbk);
            kfk[k] = (float)(xdk ? cyk : cxk);
            gk[k] = 1.0f / (qk[k] * qk[k]);
        }
        float cmin = INFINITY, cmax = -INFINITY;
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const float bw = pb[kk + e];
            const float pcw = pa[s] + 0.5f * da;
            const float ddx = (xd ? pcw : bw) - V[VF_SX];
            const float ddy = (xd ? bw : pcw) - V[VF_SY];
            const float aa = ddx * V[VF_EUX] + ddy * V[VF_EUY], bb = ddx * V[VF_EWX] + ddy * V[VF_EWY];
            const float u = h.curved ? atan2f(aa, bb) : h.sdd * aa / bb;
            const float cu = (u - h.u0_fwd) / h.du_fwd;
            cmin = fminf(cmin, cu); cmax = fmaxf(cmax, cu);
        }
        const int cA = max((int)floorf(cmin) - 1, 0), cB = min((int)floorf(cmax) + 1, nu - 1);
        const float *__restrict__ EbT = tabs + (long long)sv * matched_tab_stride(nu);
        const float *__restrict__ IPT = EbT + nu + 1;
        int ncol = 0;
        bool overflow = false;
        for (int c = cA; c <= cB; ++c) {
            const float Eb0 = __ldg(EbT + c), Eb1 = __ldg(EbT + c + 1);
            float ovk[4];
            bool any = false;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float xa = fmaf(Eb0, qk[k], cbk[k]), xb = fmaf(Eb1, qk[k], cbk[k]);
                const float o = fminf(kfk[k] + 1.0f, fmaxf(xa, xb)) - fmaxf(kfk[k], fminf(xa, xb));
                ovk[k] = o > 0.0f ? o : 0.0f;
                any = any || o > 0.0f;
            }
            if (!any) continue;
            const float tau = q * __ldg(IPT + c);
            const float inv = 1.0f / (tau * dB);
            const float wz = fabsf(dB * tau);
            if (ncol < kMC) {
                cand[0][ncol][tid] = __int_as_float(c);
#pragma unroll
                for (int k = 0; k < 4; ++k) cand[1 + ((s4 + k) & 3)][ncol][tid] = ovk[k] * gk[k] * wz;
                cand[5][ncol][tid] = tau;
                cand[6][ncol][tid] = inv;
                ++ncol;
            } else {
                overflow = true;
            }
        }
        if (!live) continue;
        if (overflow) {
            // Detector columns much narrower than a voxel: per-voxel search per column.
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float *__restrict__ Vk = T + h.off_views + (long long)pv[k] * h.view_stride;
                const float *__restrict__ Qk = proj + (long long)pv[k] * nu * nv;
                const int ak = (int)Vk[VF_AXIS];
#pragma unroll
                for (int j = 0; j < kMoZ; ++j) {
                    if (l0 + j >= nz) continue;
                    addcol(k, j, ak == 0 ? matched_voxel_view<0>(h, T, Vk, vo, Qk, ocx(k), ocy(k), l0 + j)
                                         : matched_voxel_view<1>(h, T, Vk, vo, Qk, ocx(k), ocy(k), l0 + j));
                }
            }
            continue;
        }
        const float b0r = B0 / dB;
#pragma unroll 1
        for (int m = 0; m < ncol; ++m) {
            // candidate m: the same row placement as bp_matched_column
            const int cm = __float_as_int(cand[0][m][tid]);
            const float tm = cand[5][m][tid], bm = cand[6][m][tid];
            const float sgn = bm > 0.0f ? 1.0f : -1.0f;
            const float2 w01 = make_float2(sgn * cand[1][m][tid], sgn * cand[2][m][tid]);
            const float2 w23 = make_float2(sgn * cand[3][m][tid], sgn * cand[4][m][tid]);
            const int R = min(max((int)floorf(fmaf((float)l0 - A, bm, -b0r)), 0), nv);
            const ZFrame zf = row_frame(A, tm, B0, dB, (float)R);
            const float d0 = ((float)l0 - zf.ibf) - zf.f;
            const float rlo = -(float)R, rhi = fnv - (float)R;
            // float4 offset of base view w's cell (row R, column cm) (< 2^31, checked by the host)
            const int coff = (w * cstride + R * nu + cm) * 2;
            float2 ep01, ep23;
#pragma unroll
            for (int j = 0; j <= kMoZ; ++j) {
                const float rr = fminf(fmaxf((d0 + (float)j) * bm, rlo), rhi);
                float fr;
                const int mr = floor_split(rr, &fr);
                const float fx = rr - fr;
                const float4 *cell = integ + (coff + mr * nu * 2);
                const float4 C = __ldg(cell), Y = __ldg(cell + 1);
                const float2 fx2 = make_float2(fx, fx);
                const float2 e01 = __ffma2_rn(make_float2(Y.x, Y.y), fx2, make_float2(C.x, C.y));
                const float2 e23 = __ffma2_rn(make_float2(Y.z, Y.w), fx2, make_float2(C.z, C.w));
                if (j > 0) {
                    accp[0][j - 1] = __ffma2_rn(__fadd2_rn(e01, make_float2(-ep01.x, -ep01.y)), w01, accp[0][j - 1]);
                    accp[1][j - 1] = __ffma2_rn(__fadd2_rn(e23, make_float2(-ep23.x, -ep23.y)), w23, accp[1][j - 1]);
                }
                ep01 = e01;
                ep23 = e23;
            }
        }
    }
    // the fourth quarter turn's rotation: slot k holds column k
#pragma unroll
    for (int j = 0; j < kMoZ; ++j) {
        const float2 a = accp[0][j], b = accp[1][j];
        accp[0][j] = make_float2(b.y, a.x);
        accp[1][j] = make_float2(a.y, b.x);
    }
    if (!live) return;
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int j = 0; j < kMoZ; ++j) {
            const int iz = l0 + j;
            if (iz < nz) {
                float *dst = vol + ((long long)iz * n + ocy(k)) * n + ocx(k);
                const float a = k == 0 ? accp[0][j].x : k == 1 ? accp[0][j].y : k == 2 ? accp[1][j].x : accp[1][j].y;
                const float b = __fmul_rn(scale, a);
                *dst = accumulate ? __fadd_rn(*dst, b) : b;
            }
        }
}

// ---- batched backprojection (many scans per launch) --------------------------
// Job j covers the CTA items [item0, item0 + gx * gy * gz) of its scan's grid
// (x fastest); the integration pass covers threads [t0, t0 + nu * nviews).
struct BpJob {
    const float *T;
    const float2 *integ;        // integrated projections of the job's views
    const float *tabs;          // matched: the per-view column tables after them
    const float *proj;          // raw projections (matched: z-dominant views and wide footprints)
    float *vol;
    int view0, nviews;
    float scale;
    int accumulate;
    int gx, gy, gz, item0;
    BpEpi epi;
};

struct IntegJob {
    const float *T;
    const float *proj;
    float2 *out;
    float *tabs;
    int view0, nu, nv, pad;
    long long t0;
};

// The batched bodies need more registers than the single-scan ones (at eight
// or six CTAs per SM they spilled 700 and 270 bytes): four CTAs per SM.
#ifndef CTGB_BATCH_BP_BLOCKS
#define CTGB_BATCH_BP_BLOCKS 4
#endif
constexpr int kBatchBpBlocks = CTGB_BATCH_BP_BLOCKS;

template <bool CURVED>
__global__ void __launch_bounds__(kBiTX * kBiTY, kBatchBpBlocks)
bp_fdk_batch_kernel(const BpJob *__restrict__ jobs, int njobs, int nitems) {
    int j = 0;
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        while (j + 1 < njobs && it >= jobs[j + 1].item0) ++j;
        const BpJob &jb = jobs[j];
        const int local = it - jb.item0, gxy = jb.gx * jb.gy;
        const int bz = local / gxy, r = local - bz * gxy;
        const BpJob *jp = jobs + j;
        const JobSrc<BpJob> src = {jp};
        bp_fdk_column<CURVED>(src, r % jb.gx, r / jb.gx, bz,
                              [=](long long i, float b) { bp_epilogue(jp->epi, jp->vol, i, b, jp->accumulate); });
    }
}

__global__ void __launch_bounds__(kMiTX * kMiTY, kBatchBpBlocks)
bp_matched_batch_kernel(const BpJob *__restrict__ jobs, int njobs, int nitems) {
    int j = 0;
    for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
        while (j + 1 < njobs && it >= jobs[j + 1].item0) ++j;
        const BpJob &jb = jobs[j];
        const int local = it - jb.item0, gxy = jb.gx * jb.gy;
        const int bz = local / gxy, r = local - bz * gxy;
        const BpJob *jp = jobs + j;
        const JobSrc<BpJob> src = {jp};
        bp_matched_column(src, r % jb.gx, r / jb.gx, bz,
                          [=](long long i, float a) {
                              bp_epilogue(jp->epi, jp->vol, i, __fmul_rn(jp->scale, a), jp->accumulate);
                          });
    }
}

template <bool MATCHED>
__global__ void integrate_batch_kernel(const IntegJob *__restrict__ jobs, int njobs, long long nthreads) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nthreads;
         t += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = njobs - 1;   // last job with t0 <= t
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (jobs[mid].t0 <= t) lo = mid;
            else hi = mid - 1;
        }
        const IntegJob &jb = jobs[lo];
        if (MATCHED) matched_integrate_one(jb.T, jb.proj, jb.out, jb.tabs, jb.view0, 1, t - jb.t0);
        else integrate_rows_one(jb.proj, jb.out, jb.nu, jb.nv, t - jb.t0);
    }
}

__global__ void __launch_bounds__(kBpTileX * kBpTileY)
bp_matched_kernel(const float *__restrict__ T, const float *__restrict__ proj, float *__restrict__ vol, int view0,
                  int nviews, float scale, int accumulate) {
    const TableHeader &h = header(T);
    const int ix = blockIdx.x * kBpTileX + threadIdx.x;
    const int iy = blockIdx.y * kBpTileY + threadIdx.y;
    const int iz = blockIdx.z;
    if (ix >= h.nx || iy >= h.ny) return;
    const ViewOffsets vo = view_offsets(h.nu, h.nv);
    float acc = 0.0f;
    for (int vi = 0; vi < nviews; ++vi) {
        const float *__restrict__ V = T + h.off_views + (long long)(view0 + vi) * h.view_stride;
        const float *__restrict__ Q = proj + (long long)vi * h.nu * h.nv;
        const int axis = (int)V[VF_AXIS];
        if (axis == 1) acc += matched_voxel_view<1>(h, T, V, vo, Q, ix, iy, iz);
        else if (axis == 0) acc += matched_voxel_view<0>(h, T, V, vo, Q, ix, iy, iz);
        else acc += matched_voxel_view<2>(h, T, V, vo, Q, ix, iy, iz);
    }
    float *dst = vol + ((long long)iz * h.ny + iy) * h.nx + ix;
    *dst = accumulate ? *dst + scale * acc : scale * acc;
}

}  // namespace ctgb

using namespace ctgb;

static int bp_args(const ctgb_params *p, const void *t, const float *q, float *v, int view0, int nviews,
                   const char *who) {
    // projections may be absent (an empty tensor) when no view is read
    if (!p || !t || !v || (!q && nviews > 0)) return set_error(CTGB_ERR_ARG, "%s: NULL argument", who);
    if (view0 < 0 || nviews < 0 || view0 + nviews > p->nviews)
        return set_error(CTGB_ERR_ARG, "%s: view range [%d,%d) outside [0,%d)", who, view0, view0 + nviews,
                         p->nviews);
    return CTGB_OK;
}

// One launch of the integrated FDK backprojector over nviews views.
static int launch_bp_integ(const ctgb_params *p, const float *T, const float2 *ws, float *d_vol, int view0,
                           int nviews, float scale, int accumulate, cudaStream_t s) {
    dim3 block(kBiTX, kBiTY);
    dim3 grid((p->nx + kBiTX - 1) / kBiTX, (p->ny + kBiTY - 1) / kBiTY, (p->nz + kBiZ - 1) / kBiZ);
    if (p->curved)
        bp_fdk_integ_kernel<true><<<grid, block, 0, s>>>(T, ws, d_vol, view0, nviews, scale, accumulate);
    else
        bp_fdk_integ_kernel<false><<<grid, block, 0, s>>>(T, ws, d_vol, view0, nviews, scale, accumulate);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "bp_fdk_integ_kernel: %s", cudaGetErrorString(e));
    return CTGB_OK;
}

// Largest rotation-orbit size the FDK walk uses (1, 2 or 4).
#ifndef CTGB_WALK_NC
#define CTGB_WALK_NC 4
#endif

// Half-turn symmetry of a scan for bp_fdk_walk_kernel<.., 2, ..>: a grid of
// even height centred on the rotation axis (voxel centres i and n-1-i exact
// negatives of each other in x and in y), no helical pitch, and an even view
// count whose float32 cosines and sines change sign every half of the views.
static bool fdk_twofold(const ctgb_params *p) {
    if ((p->ny & 1) || p->ny < 2) return false;
    if (p->recon_center[0] != 0.0 || p->recon_center[1] != 0.0 || p->pitch != 0.0) return false;
    const int n = p->nviews, q = n / 2;
    if (n < 2 || n % 2) return false;
    const double step = (p->end_angle - p->start_angle) / n;
    for (int v = 0; v < n; ++v) {
        const double a = v * step + p->start_angle, b = ((v + q) % n) * step + p->start_angle;
        const float ca = (float)std::cos(a), sa = (float)std::sin(a), cb = (float)std::cos(b), sb = (float)std::sin(b);
        if (std::fabs(cb + ca) > 2.4e-7f || std::fabs(sb + sa) > 2.4e-7f) return false;
    }
    return true;
}

// Four-fold symmetry of a scan for bp_fdk_walk_kernel<.., 4, ..>: a square
// grid of even side centred on the rotation axis (x and y voxel centres exact
// negatives of each other in the table), no helical pitch, and a view count
// divisible by 4 whose float32 cosines and sines repeat, rotated by a quarter
// turn, every quarter of the views (a full circular orbit).
static bool fdk_fourfold(const ctgb_params *p) {
    if (p->nx != p->ny || (p->nx & 1) || p->nx < 2 || p->dx != p->dy) return false;
    if (p->recon_center[0] != 0.0 || p->recon_center[1] != 0.0 || p->pitch != 0.0) return false;
    const int n = p->nviews, q = n / 4;
    if (n < 4 || n % 4) return false;
    const double step = (p->end_angle - p->start_angle) / n;
    for (int v = 0; v < n; ++v) {
        const double a = v * step + p->start_angle, b = ((v + q) % n) * step + p->start_angle;
        const float ca = (float)std::cos(a), sa = (float)std::sin(a), cb = (float)std::cos(b), sb = (float)std::sin(b);
        if (std::fabs(cb + sa) > 2.4e-7f || std::fabs(sb - ca) > 2.4e-7f) return false;
    }
    return true;
}

template <int NC>
static void launch_walk(bool curved, dim3 grid, cudaStream_t s, const float *T, const float *proj, float *vol,
                        int view0, int nviews, float scale, int accumulate) {
    dim3 block(kWkTX, kWkTY);
    if (curved)
        bp_fdk_walk_kernel<true, NC><<<grid, block, 0, s>>>(T, proj, vol, view0, nviews, scale, accumulate);
    else
        bp_fdk_walk_kernel<false, NC><<<grid, block, 0, s>>>(T, proj, vol, view0, nviews, scale, accumulate);
}

// The paired (2- and 4-column) walks address the projections with 32-bit
// element offsets.
static bool walk_offsets_fit(const ctgb_params *p) {
    return (long long)p->nviews * p->nu * p->nv < (1LL << 31);
}

static int fdk_orbit(const ctgb_params *p) {
    if (!walk_offsets_fit(p)) return 1;
    if (CTGB_WALK_NC >= 4 && fdk_fourfold(p)) return 4;
    if (CTGB_WALK_NC >= 2 && fdk_twofold(p)) return 2;
    return 1;
}

extern "C" int ctgb_backproject_fdk_orbit_size(const ctgb_params *p, int32_t *nc) {
    clear_error();
    if (!p || !nc) return set_error(CTGB_ERR_ARG, "ctgb_backproject_fdk_orbit_size: NULL argument");
    *nc = fdk_orbit(p);
    return CTGB_OK;
}

extern "C" int ctgb_backproject_fdk_orbits(const ctgb_params *p, const void *d_table, const float *d_proj,
                                           float *d_vol, int32_t base0, int32_t nbase, float scale,
                                           int32_t accumulate, void *stream) {
    clear_error();
    if (!p || !d_table || !d_vol || (!d_proj && nbase > 0))
        return set_error(CTGB_ERR_ARG, "ctgb_backproject_fdk_orbits: NULL argument");
    const int nc = fdk_orbit(p), period = p->nviews / nc;
    if (base0 < 0 || nbase < 0 || base0 + nbase > period)
        return set_error(CTGB_ERR_ARG, "ctgb_backproject_fdk_orbits: base views [%d,%d) outside [0,%d)", base0,
                         base0 + nbase, period);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (nbase == 0) {
        if (!accumulate) {
            cudaError_t e = cudaMemsetAsync(d_vol, 0, sizeof(float) * (size_t)p->nx * p->ny * p->nz, s);
            if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "memset: %s", cudaGetErrorString(e));
        }
        return CTGB_OK;
    }
    if ((long long)p->nu * (p->nv + 2) >= (1LL << 31))
        return set_error(CTGB_ERR_SIZE, "ctgb_backproject_fdk_orbits: detector of %d x %d pixels too large", p->nu,
                         p->nv);
    const float *T = static_cast<const float *>(d_table);
    if (nc == 4) {
        const int hn = p->nx / 2;
        dim3 grid((hn + kWkTX - 1) / kWkTX, (hn + kWkTY - 1) / kWkTY, (p->nz + WalkShape<4>::Z - 1) / WalkShape<4>::Z);
        launch_walk<4>(p->curved, grid, s, T, d_proj, d_vol, base0, nbase, scale, accumulate);
    } else if (nc == 2) {
        dim3 grid((p->nx + kWkTX - 1) / kWkTX, (p->ny / 2 + kWkTY - 1) / kWkTY,
                  (p->nz + WalkShape<2>::Z - 1) / WalkShape<2>::Z);
        launch_walk<2>(p->curved, grid, s, T, d_proj, d_vol, base0, nbase, scale, accumulate);
    } else {
        dim3 grid((p->nx + kWkTX - 1) / kWkTX, (p->ny + kWkTY - 1) / kWkTY,
                  (p->nz + WalkShape<1>::Z - 1) / WalkShape<1>::Z);
        launch_walk<1>(p->curved, grid, s, T, d_proj + (long long)base0 * p->nu * p->nv, d_vol, base0, nbase, scale,
                       accumulate);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "bp_fdk_walk_kernel: %s", cudaGetErrorString(e));
    return CTGB_OK;
}

extern "C" int ctgb_backproject_fdk(const ctgb_params *p, const void *d_table, const float *d_proj, float *d_vol,
                                    int32_t view0, int32_t nviews, float scale, int32_t accumulate, void *stream) {
    clear_error();
    int st = bp_args(p, d_table, d_proj, d_vol, view0, nviews, "ctgb_backproject_fdk");
    if (st) return st;
    const float *T = static_cast<const float *>(d_table);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (nviews == 0) {
        if (!accumulate) {
            cudaError_t e = cudaMemsetAsync(d_vol, 0, sizeof(float) * (size_t)p->nx * p->ny * p->nz, s);
            if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "memset: %s", cudaGetErrorString(e));
        }
        return CTGB_OK;
    }
    if ((long long)p->nu * (p->nv + 2) >= (1LL << 31))
        return set_error(CTGB_ERR_SIZE, "ctgb_backproject_fdk: detector of %d x %d pixels too large", p->nu, p->nv);
    const bool full = view0 == 0 && nviews == p->nviews;
    const int nc = full ? fdk_orbit(p) : 1;
    if (nc == 4) {
        const int hn = p->nx / 2;
        dim3 grid((hn + kWkTX - 1) / kWkTX, (hn + kWkTY - 1) / kWkTY, (p->nz + WalkShape<4>::Z - 1) / WalkShape<4>::Z);
        launch_walk<4>(p->curved, grid, s, T, d_proj, d_vol, 0, p->nviews / 4, scale, accumulate);
    } else if (nc == 2) {
        dim3 grid((p->nx + kWkTX - 1) / kWkTX, (p->ny / 2 + kWkTY - 1) / kWkTY,
                  (p->nz + WalkShape<2>::Z - 1) / WalkShape<2>::Z);
        launch_walk<2>(p->curved, grid, s, T, d_proj, d_vol, 0, p->nviews / 2, scale, accumulate);
    } else {
        dim3 grid((p->nx + kWkTX - 1) / kWkTX, (p->ny + kWkTY - 1) / kWkTY,
                  (p->nz + WalkShape<1>::Z - 1) / WalkShape<1>::Z);
        launch_walk<1>(p->curved, grid, s, T, d_proj, d_vol, view0, nviews, scale, accumulate);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "bp_fdk_walk_kernel: %s", cudaGetErrorString(e));
    return CTGB_OK;
}

extern "C" int ctgb_backproject_matched(const ctgb_params *p, const void *d_table, const float *d_proj,
                                        float *d_vol, int32_t view0, int32_t nviews, float scale,
                                        int32_t accumulate, void *stream) {
    clear_error();
    int st = bp_args(p, d_table, d_proj, d_vol, view0, nviews, "ctgb_backproject_matched");
    if (st) return st;
    dim3 block(kBpTileX, kBpTileY);
    dim3 grid((p->nx + kBpTileX - 1) / kBpTileX, (p->ny + kBpTileY - 1) / kBpTileY, (p->nz + kMZ - 1) / kMZ);
    bp_matched_sweep_kernel<<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const float *>(d_table), d_proj, d_vol, view0, nviews, scale, accumulate);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "bp_matched_kernel: %s", cudaGetErrorString(e));
    return CTGB_OK;
}

extern "C" int ctgb_backproject_fdk_workspace_bytes(const ctgb_params *p, int32_t nviews, size_t *bytes) {
    clear_error();
    if (!p || !bytes || nviews < 0 || p->nu < 1 || p->nv < 1)
        return set_error(CTGB_ERR_ARG, "ctgb_backproject_fdk_workspace_bytes: bad arguments");
    // integrated rows, plus the matched backprojector's per-view column tables
    *bytes = (size_t)nviews * ((size_t)(p->nv + 1) * (size_t)p->nu * sizeof(float2) +
                               (size_t)(2 * p->nu + 2) * sizeof(float));
    return CTGB_OK;
}

extern "C" int ctgb_backproject_fdk_ws(const ctgb_params *p, const void *d_table, const float *d_proj, float *d_vol,
                                       int32_t view0, int32_t nviews, float scale, int32_t accumulate,
                                       void *d_workspace, size_t workspace_bytes, void *stream) {
    clear_error();
    int st = bp_args(p, d_table, d_proj, d_vol, view0, nviews, "ctgb_backproject_fdk_ws");
    if (st) return st;
    if (!d_workspace) return set_error(CTGB_ERR_ARG, "ctgb_backproject_fdk_ws: NULL workspace");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (nviews == 0) {
        if (!accumulate) {
            cudaError_t e = cudaMemsetAsync(d_vol, 0, sizeof(float) * (size_t)p->nx * p->ny * p->nz, s);
            if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "memset: %s", cudaGetErrorString(e));
        }
        return CTGB_OK;
    }
    // A full orbit with four-fold symmetry runs the row walk over the raw
    // projections (no workspace needed): faster than integrating them.
    if (view0 == 0 && nviews == p->nviews && fdk_orbit(p) == 4)
        return ctgb_backproject_fdk(p, d_table, d_proj, d_vol, view0, nviews, scale, accumulate, stream);
    const size_t per_view = (size_t)(p->nv + 1) * (size_t)p->nu * sizeof(float2);
    const int chunk = (int)(workspace_bytes / per_view);
    if (chunk < 1) return set_error(CTGB_ERR_SIZE, "ctgb_backproject_fdk_ws: workspace below one view");
    const float *T = static_cast<const float *>(d_table);
    float2 *ws = static_cast<float2 *>(d_workspace);
    for (int v = 0; v < nviews; v += chunk) {
        const int n = nviews - v < chunk ? nviews - v : chunk;
        const long long threads = (long long)p->nu * n;
        integrate_rows_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
            d_proj + (long long)v * p->nu * p->nv, ws, p->nu, p->nv, n);
        const int acc = (v > 0) ? 1 : accumulate;
        if (int st2 = launch_bp_integ(p, T, ws, d_vol, view0 + v, n, scale, acc, s)) return st2;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "bp_fdk_integ_kernel: %s", cudaGetErrorString(e));
    return CTGB_OK;
}

extern "C" int ctgb_integrate_projections(const ctgb_params *p, const float *d_proj, int32_t nviews,
                                          void *d_workspace, size_t workspace_bytes, void *stream) {
    clear_error();
    if (!p || !d_proj || !d_workspace) return set_error(CTGB_ERR_ARG, "ctgb_integrate_projections: NULL argument");
    if (nviews < 0 || nviews > p->nviews)
        return set_error(CTGB_ERR_ARG, "ctgb_integrate_projections: view count %d outside [0,%d]", nviews, p->nviews);
    const size_t per_view = (size_t)(p->nv + 1) * (size_t)p->nu * sizeof(float2);
    if (workspace_bytes < per_view * (size_t)nviews)
        return set_error(CTGB_ERR_SIZE, "ctgb_integrate_projections: workspace below nviews views");
    if (nviews == 0) return CTGB_OK;
    const long long threads = (long long)p->nu * nviews;
    integrate_rows_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        d_proj, static_cast<float2 *>(d_workspace), p->nu, p->nv, nviews);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "integrate_rows_kernel: %s", cudaGetErrorString(e));
    return CTGB_OK;
}

extern "C" int ctgb_backproject_fdk_integrated(const ctgb_params *p, const void *d_table, const void *d_integrated,
                                               float *d_vol, int32_t view0, int32_t nviews, float scale,
                                               int32_t accumulate, void *stream) {
    clear_error();
    int st = bp_args(p, d_table, static_cast<const float *>(d_integrated), d_vol, view0, nviews,
                     "ctgb_backproject_fdk_integrated");
    if (st) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (nviews == 0) {
        if (!accumulate) {
            cudaError_t e = cudaMemsetAsync(d_vol, 0, sizeof(float) * (size_t)p->nx * p->ny * p->nz, s);
            if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "memset: %s", cudaGetErrorString(e));
        }
        return CTGB_OK;
    }
    const float *T = static_cast<const float *>(d_table);
    const float2 *ws = static_cast<const float2 *>(d_integrated);
    if (int st2 = launch_bp_integ(p, T, ws, d_vol, view0, nviews, scale, accumulate, s)) return st2;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "bp_fdk_integ_kernel: %s", cudaGetErrorString(e));
    return CTGB_OK;
}

extern "C" int ctgb_backproject_matched_ws(const ctgb_params *p, const void *d_table, const float *d_proj,
                                           float *d_vol, int32_t view0, int32_t nviews, float scale,
                                           int32_t accumulate, void *d_workspace, size_t workspace_bytes,
                                           void *stream) {
    clear_error();
    int st = bp_args(p, d_table, d_proj, d_vol, view0, nviews, "ctgb_backproject_matched_ws");
    if (st) return st;
    if (!d_workspace) return set_error(CTGB_ERR_ARG, "ctgb_backproject_matched_ws: NULL workspace");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (nviews == 0) {
        if (!accumulate) {
            cudaError_t e = cudaMemsetAsync(d_vol, 0, sizeof(float) * (size_t)p->nx * p->ny * p->nz, s);
            if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "memset: %s", cudaGetErrorString(e));
        }
        return CTGB_OK;
    }
    const size_t rows_view = (size_t)(p->nv + 1) * (size_t)p->nu * sizeof(float2);
    const size_t per_view = rows_view + (size_t)(2 * p->nu + 2) * sizeof(float);
    const int chunk = (int)(workspace_bytes / per_view);
    if (chunk < 1) return set_error(CTGB_ERR_SIZE, "ctgb_backproject_matched_ws: workspace below one view");
    const float *T = static_cast<const float *>(d_table);
    float2 *ws = static_cast<float2 *>(d_workspace);
    dim3 block(kMiTX, kMiTY);
    // A full quarter-turn-symmetric orbit whose integrated views all fit the
    // workspace: one integration pass, then the orbit kernel.
    // Needs the table's exactly rotated view records (quarter_turn_views) and
    // a square grid of even side whose forward planes are centred on the axis.
    const double *cf = p->flavour == CTGB_FLAVOUR_PYCUDA ? p->recon_center : p->phantom_center;
    const bool square = p->nx == p->ny && !(p->nx & 1) && p->dx == p->dy && cf[0] == 0.0 && cf[1] == 0.0 &&
                        slice_centres_antisymmetric(p);
    std::vector<int> broken;
    if (CTGB_WALK_NC >= 4 && view0 == 0 && nviews == p->nviews && chunk >= nviews && square &&
        (long long)p->nviews * (p->nv + 1) * p->nu < (1LL << 31) && quarter_turn_views(p, &broken)) {
        // the four views of each base view interleaved per cell (the same
        // bytes as nviews views of (C, y') pairs), the column tables after them
        const int q = nviews / 4;
        const long long threads = 4LL * p->nu * q;
        float *tabs = reinterpret_cast<float *>(ws + (size_t)nviews * (p->nv + 1) * p->nu);
        matched_integrate_orbit_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
            T, d_proj, reinterpret_cast<float *>(ws), tabs);
        const int hn = p->nx / 2;
        dim3 ogrid((hn + kMiTX - 1) / kMiTX, (hn + kMiTY - 1) / kMiTY, (p->nz + kMoZ - 1) / kMoZ);
        bp_matched_orbit_kernel<<<ogrid, block, 0, s>>>(T, reinterpret_cast<const float4 *>(ws), tabs, d_proj, d_vol,
                                                         scale, accumulate);
        // the groups the orbit kernel skipped: the four views g + k q of each
        // integrated again, as (C, y') pairs, into the workspace's start (the
        // orbit kernel has read it by then: same stream), then backprojected
        // by one launch (view step q)
        dim3 grid1((p->nx + kMiTX - 1) / kMiTX, (p->ny + kMiTY - 1) / kMiTY, (p->nz + kMZ - 1) / kMZ);
        for (int g : broken) {
            const float *pg = d_proj + (long long)g * p->nu * p->nv;
            float *tab_g = tabs + (size_t)g * matched_tab_stride(p->nu);
            matched_integrate_kernel<<<(unsigned)((4 * p->nu + 255) / 256), 256, 0, s>>>(T, pg, ws, tab_g, g, 4, q);
            bp_matched_integ_kernel<<<grid1, block, 0, s>>>(T, ws, tab_g, pg, d_vol, g, 4, scale, 1, q);
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "bp_matched_orbit_kernel: %s", cudaGetErrorString(e));
        return CTGB_OK;
    }
    dim3 grid((p->nx + kMiTX - 1) / kMiTX, (p->ny + kMiTY - 1) / kMiTY, (p->nz + kMZ - 1) / kMZ);
    for (int v = 0; v < nviews; v += chunk) {
        const int n = nviews - v < chunk ? nviews - v : chunk;
        const long long threads = (long long)p->nu * n;
        const float *pv = d_proj + (long long)v * p->nu * p->nv;
        // the chunk's n views of integrated rows, then their column tables
        float *tabs = reinterpret_cast<float *>(ws + (size_t)n * (p->nv + 1) * p->nu);
        matched_integrate_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(T, pv, ws, tabs, view0 + v, n, 1);
        const int acc = (v > 0) ? 1 : accumulate;
        bp_matched_integ_kernel<<<grid, block, 0, s>>>(T, ws, tabs, pv, d_vol, view0 + v, n, scale, acc, 1);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "bp_matched_integ_kernel: %s", cudaGetErrorString(e));
    return CTGB_OK;
}

namespace {

constexpr uint32_t kBpPlanMagic = 0x31425042u;

// Host and device copies of a plan are the same bytes: this head, the BpJob
// array, the IntegJob array.
struct BpPlanHead {
    uint32_t magic;
    int32_t matched, curved, njobs;
    int32_t nitems, pad;
    int64_t nthreads, off_jobs, off_integ, total;
};

size_t bp_align(size_t v) { return (v + 127) / 128 * 128; }

int build_bp_plan(const ctgb_bp_job *jobs, int njobs, int matched, unsigned char *out, size_t bytes, size_t *need) {
    if (!jobs || njobs < 1) return set_error(CTGB_ERR_ARG, "batched backprojection: no jobs");
    int curved = -1;
    long long items = 0, threads = 0;
    for (int i = 0; i < njobs; ++i) {
        const ctgb_bp_job &jb = jobs[i];
        const ctgb_params *p = jb.params;
        if (!p || !jb.table || !jb.workspace || (!jb.proj && jb.nviews > 0))
            return set_error(CTGB_ERR_ARG, "batched backprojection: job %d has a NULL argument", i);
        if (jb.view0 < 0 || jb.nviews < 0 || jb.view0 + jb.nviews > p->nviews)
            return set_error(CTGB_ERR_ARG, "batched backprojection: job %d view range outside the scan", i);
        if (jb.epilogue < CTGB_BP_STORE || jb.epilogue > CTGB_BP_POCS_UPDATE)
            return set_error(CTGB_ERR_ARG, "batched backprojection: job %d unknown epilogue %d", i, jb.epilogue);
        if (jb.epilogue == CTGB_BP_STORE ? !jb.vol : (!jb.x || !jb.n1))
            return set_error(CTGB_ERR_ARG, "batched backprojection: job %d epilogue output missing", i);
        if (!matched && p->nu < 4)
            return set_error(CTGB_ERR_ARG, "batched backprojection: job %d has fewer than 4 detector columns", i);
        size_t ws = 0;
        if (int st = ctgb_backproject_fdk_workspace_bytes(p, jb.nviews, &ws)) return st;
        if (jb.workspace_bytes < ws)
            return set_error(CTGB_ERR_SIZE, "batched backprojection: job %d workspace of %zu bytes below %zu", i,
                             jb.workspace_bytes, ws);
        if (!matched) {
            if (curved >= 0 && curved != (p->curved ? 1 : 0))
                return set_error(CTGB_ERR_ARG, "batched backprojection: flat and curved detectors in one plan");
            curved = p->curved ? 1 : 0;
        }
        const int tx = matched ? kMiTX : kBiTX, ty = matched ? kMiTY : kBiTY, tz = matched ? kMZ : kBiZ;
        items += (long long)((p->nx + tx - 1) / tx) * ((p->ny + ty - 1) / ty) * ((p->nz + tz - 1) / tz);
        threads += (long long)p->nu * jb.nviews;
    }
    if (items > 0x7fffffffLL) return set_error(CTGB_ERR_SIZE, "batched backprojection: too many blocks");
    BpPlanHead head;
    std::memset(&head, 0, sizeof head);
    head.magic = kBpPlanMagic;
    head.matched = matched ? 1 : 0;
    head.curved = curved > 0 ? 1 : 0;
    head.njobs = njobs;
    head.nitems = (int32_t)items;
    head.nthreads = threads;
    head.off_jobs = (int64_t)bp_align(sizeof head);
    head.off_integ = (int64_t)bp_align(head.off_jobs + sizeof(BpJob) * njobs);
    head.total = (int64_t)bp_align(head.off_integ + sizeof(IntegJob) * njobs);
    *need = (size_t)head.total;
    if (!out) return CTGB_OK;
    if (bytes < *need)
        return set_error(CTGB_ERR_SIZE, "batched backprojection: plan buffer of %zu bytes below %zu", bytes, *need);
    std::memset(out, 0, *need);
    std::memcpy(out, &head, sizeof head);
    BpJob *bj = reinterpret_cast<BpJob *>(out + head.off_jobs);
    IntegJob *ij = reinterpret_cast<IntegJob *>(out + head.off_integ);
    int item = 0;
    long long t0 = 0;
    for (int i = 0; i < njobs; ++i) {
        const ctgb_bp_job &jb = jobs[i];
        const ctgb_params *p = jb.params;
        float2 *ws = static_cast<float2 *>(jb.workspace);
        float *tabs = reinterpret_cast<float *>(ws + (size_t)jb.nviews * (p->nv + 1) * p->nu);
        BpJob &b = bj[i];
        b.T = static_cast<const float *>(jb.table);
        b.integ = ws;
        b.tabs = tabs;
        b.proj = jb.proj;
        b.vol = jb.vol;
        b.view0 = jb.view0;
        b.nviews = jb.nviews;
        b.scale = jb.scale;
        b.accumulate = jb.accumulate ? 1 : 0;
        const int tx = matched ? kMiTX : kBiTX, ty = matched ? kMiTY : kBiTY, tz = matched ? kMZ : kBiZ;
        b.gx = (p->nx + tx - 1) / tx;
        b.gy = (p->ny + ty - 1) / ty;
        b.gz = (p->nz + tz - 1) / tz;
        b.item0 = item;
        item += b.gx * b.gy * b.gz;
        b.epi.mode = jb.epilogue;
        b.epi.coef = jb.coef;
        b.epi.eps = jb.eps;
        b.epi.x = jb.x;
        b.epi.n1 = jb.n1;
        IntegJob &g = ij[i];
        g.T = b.T;
        g.proj = jb.proj;
        g.out = ws;
        g.tabs = tabs;
        g.view0 = jb.view0;
        g.nu = p->nu;
        g.nv = p->nv;
        g.t0 = t0;
        t0 += (long long)p->nu * jb.nviews;
    }
    return CTGB_OK;
}

}  // namespace

extern "C" int ctgb_batch_backproject_plan_bytes(const ctgb_bp_job *jobs, int32_t njobs, size_t *bytes) {
    clear_error();
    if (!bytes) return set_error(CTGB_ERR_ARG, "ctgb_batch_backproject_plan_bytes: NULL argument");
    // the layout does not depend on the backprojector kind
    return build_bp_plan(jobs, njobs, 1, nullptr, 0, bytes);
}

extern "C" int ctgb_batch_backproject_plan(const ctgb_bp_job *jobs, int32_t njobs, int32_t matched, void *host_plan,
                                           size_t bytes) {
    clear_error();
    if (!host_plan) return set_error(CTGB_ERR_ARG, "ctgb_batch_backproject_plan: NULL plan");
    size_t need = 0;
    return build_bp_plan(jobs, njobs, matched, static_cast<unsigned char *>(host_plan), bytes, &need);
}

extern "C" int ctgb_batch_backproject(const void *host_plan, const void *d_plan, int32_t ctas_per_sm, void *stream) {
    clear_error();
    if (!host_plan || !d_plan || ctas_per_sm < 1)
        return set_error(CTGB_ERR_ARG, "ctgb_batch_backproject: bad arguments");
    const BpPlanHead &head = *static_cast<const BpPlanHead *>(host_plan);
    if (head.magic != kBpPlanMagic) return set_error(CTGB_ERR_ARG, "ctgb_batch_backproject: not a backprojection plan");
    if (reinterpret_cast<uintptr_t>(d_plan) % 128)
        return set_error(CTGB_ERR_ARG, "ctgb_batch_backproject: device plan must be 128-byte aligned");
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "ctgb_batch_backproject: %s", cudaGetErrorString(e));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const unsigned char *dp = static_cast<const unsigned char *>(d_plan);
    const IntegJob *ij = reinterpret_cast<const IntegJob *>(dp + head.off_integ);
    const BpJob *bj = reinterpret_cast<const BpJob *>(dp + head.off_jobs);
    if (head.nthreads > 0) {
        const long long blocks = std::min<long long>((head.nthreads + 255) / 256, (long long)sms * 8);
        if (head.matched) integrate_batch_kernel<true><<<(unsigned)blocks, 256, 0, st>>>(ij, head.njobs, head.nthreads);
        else integrate_batch_kernel<false><<<(unsigned)blocks, 256, 0, st>>>(ij, head.njobs, head.nthreads);
    }
    if (head.nitems > 0) {
        const int grid = (int)std::min<long long>(head.nitems, (long long)sms * ctas_per_sm);
        if (head.matched)
            bp_matched_batch_kernel<<<grid, dim3(kMiTX, kMiTY), 0, st>>>(bj, head.njobs, head.nitems);
        else if (head.curved)
            bp_fdk_batch_kernel<true><<<grid, dim3(kBiTX, kBiTY), 0, st>>>(bj, head.njobs, head.nitems);
        else
            bp_fdk_batch_kernel<false><<<grid, dim3(kBiTX, kBiTY), 0, st>>>(bj, head.njobs, head.nitems);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "batched backprojection: %s", cudaGetErrorString(e));
    return CTGB_OK;
}
