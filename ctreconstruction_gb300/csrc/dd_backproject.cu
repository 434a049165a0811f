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
//    GB300 layout: one thread owns a column of kZc voxels (fixed x, y) and
//    keeps their sums in registers across all views (no atomics; the reference
//    launches one kernel per view and atomically adds).  Everything that does
//    not depend on z — the four rotated xy corners, the u footprint, the
//    distance weight — is computed once per (column, view); per voxel only the
//    v footprint (two products and a min/max per z end) is new.  With
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

#include "dd_common.cuh"
#include "status.h"

namespace ctgb {

constexpr int kBpTileX = 32, kBpTileY = 4, kZc = 8;

template <bool CURVED>
__global__ void __launch_bounds__(kBpTileX * kBpTileY)
bp_fdk_kernel(const float *__restrict__ T, const float *__restrict__ proj, float *__restrict__ vol, int view0,
              int nviews, float scale, int accumulate) {
    const TableHeader &h = header(T);
    const int ix = blockIdx.x * kBpTileX + threadIdx.x;
    const int iy = blockIdx.y * kBpTileY + threadIdx.y;
    const int z0 = blockIdx.z * kZc;
    if (ix >= h.nx || iy >= h.ny) return;
    const float *__restrict__ xpix = T + h.off_xpix;
    const float *__restrict__ ypix = T + h.off_ypix;
    const float *__restrict__ zpix = T + h.off_zpix;
    const float *__restrict__ ki = T + h.off_ki;
    const float *__restrict__ pp = T + h.off_pp;
    const int nu = h.nu, nv = h.nv;
    const float xx = xpix[ix], yy = ypix[iy];
    const float hx = h.dx * 0.5f, hy = h.dy * 0.5f, hz = h.dz * 0.5f;
    const float du = h.du_bp, dv = h.dv_bp, inv_du = 1.0f / du, inv_dv = 1.0f / dv;
    const float abs_du = fabsf(du), abs_dv = fabsf(dv);
    const float ki0 = ki[0], pp0 = pp[0];
    const float Sx = h.src0x, Sy = h.src0y, Dy = h.det0y, R = h.sad;
    const float eps = h.eps_bp;
    float zz[kZc];
    float acc[kZc];
#pragma unroll
    for (int j = 0; j < kZc; ++j) {
        zz[j] = (z0 + j < h.nz) ? zpix[z0 + j] : 0.0f;
        acc[j] = 0.0f;
    }
    for (int vi = 0; vi < nviews; ++vi) {
        const float *__restrict__ V = T + h.off_views + (long long)(view0 + vi) * h.view_stride;
        const float cs = V[VF_COS], sn = V[VF_SIN], Sz = V[VF_BPSZ];
        const float yc = yy * cs - xx * sn;
        float umin = INFINITY, umax = -INFINITY, imin = INFINITY, imax = -INFINITY;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float cx = xx + ((q & 1) ? hx : -hx), cy = yy + ((q & 2) ? hy : -hy);
            const float xr = cx * cs + cy * sn, yr = cy * cs - cx * sn;
            const float su = (Sx - xr) / (Sy - yr);
            const float inv = 1.0f / (Sy - yr);
            umin = fminf(umin, su); umax = fmaxf(umax, su);
            imin = fminf(imin, inv); imax = fmaxf(imax, inv);
        }
        float cu1, cu2;
        if (CURVED) { cu1 = -atanf(umin); cu2 = -atanf(umax); }
        else { cu1 = umin * Dy + (Sx - umin * Sy); cu2 = umax * Dy + (Sx - umax * Sy); }
        const Span us = make_span(cu1, cu2, ki0, inv_du);
        const int l0 = max(us.s, 0), l1 = min(us.e, nu - 1);
        const float W = scale * (R * R) / ((R - yc) * (R - yc));
        const float *__restrict__ Q = proj + (long long)vi * nu * nv;
#pragma unroll
        for (int j = 0; j < kZc; ++j) {
            const float nlo = Sz - (zz[j] - hz), nhi = Sz - (zz[j] + hz);
            const float a0 = nlo * imin, a1 = nlo * imax, a2 = nhi * imin, a3 = nhi * imax;
            const float vmin = fminf(fminf(a0, a1), fminf(a2, a3));
            const float vmax = fmaxf(fmaxf(a0, a1), fmaxf(a2, a3));
            const float cv1 = vmin * Dy + (Sz - vmin * Sy), cv2 = vmax * Dy + (Sz - vmax * Sy);
            const Span vs = make_span(cv1, cv2, pp0, inv_dv);
            const int k0 = max(vs.s, 0), k1 = min(vs.e, nv - 1);
            float sum = 0.0f;
            for (int k = k0; k <= k1; ++k) {
                const float w1 = span_weight<true>(vs, k, pp[k], pp[k + 1], abs_dv, eps);
                const float *__restrict__ qrow = Q + (long long)k * nu;
                float part = 0.0f;
                for (int l = l0; l <= l1; ++l) {
                    const float w2 = span_weight<false>(us, l, ki[l], ki[l + 1], abs_du, eps);
                    part += __ldg(qrow + l) * w2;
                }
                sum += part * w1;
            }
            acc[j] += sum * W;
        }
    }
#pragma unroll
    for (int j = 0; j < kZc; ++j) {
        const int iz = z0 + j;
        if (iz < h.nz) {
            float *dst = vol + ((long long)iz * h.ny + iy) * h.nx + ix;
            *dst = accumulate ? *dst + acc[j] : acc[j];
        }
    }
}

// ---- matched (adjoint) backprojector ---------------------------------------

template <int A>
__device__ float matched_voxel_view(const TableHeader &h, const float *__restrict__ T, const float *__restrict__ V,
                                    const ViewOffsets &vo, const float *__restrict__ Q, int ix, int iy, int iz) {
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
    if (!p || !t || !q || !v) return set_error(CTGB_ERR_ARG, "%s: NULL argument", who);
    if (view0 < 0 || nviews < 0 || view0 + nviews > p->nviews)
        return set_error(CTGB_ERR_ARG, "%s: view range [%d,%d) outside [0,%d)", who, view0, view0 + nviews,
                         p->nviews);
    return CTGB_OK;
}

extern "C" int ctgb_backproject_fdk(const ctgb_params *p, const void *d_table, const float *d_proj, float *d_vol,
                                    int32_t view0, int32_t nviews, float scale, int32_t accumulate, void *stream) {
    clear_error();
    int st = bp_args(p, d_table, d_proj, d_vol, view0, nviews, "ctgb_backproject_fdk");
    if (st) return st;
    dim3 block(kBpTileX, kBpTileY);
    dim3 grid((p->nx + kBpTileX - 1) / kBpTileX, (p->ny + kBpTileY - 1) / kBpTileY, (p->nz + kZc - 1) / kZc);
    const float *T = static_cast<const float *>(d_table);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (p->curved) bp_fdk_kernel<true><<<grid, block, 0, s>>>(T, d_proj, d_vol, view0, nviews, scale, accumulate);
    else bp_fdk_kernel<false><<<grid, block, 0, s>>>(T, d_proj, d_vol, view0, nviews, scale, accumulate);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "bp_fdk_kernel: %s", cudaGetErrorString(e));
    return CTGB_OK;
}

extern "C" int ctgb_backproject_matched(const ctgb_params *p, const void *d_table, const float *d_proj,
                                        float *d_vol, int32_t view0, int32_t nviews, float scale,
                                        int32_t accumulate, void *stream) {
    clear_error();
    int st = bp_args(p, d_table, d_proj, d_vol, view0, nviews, "ctgb_backproject_matched");
    if (st) return st;
    if (p->nz > 65535) return set_error(CTGB_ERR_SIZE, "ctgb_backproject_matched: nz above 65535");
    dim3 block(kBpTileX, kBpTileY);
    dim3 grid((p->nx + kBpTileX - 1) / kBpTileX, (p->ny + kBpTileY - 1) / kBpTileY, p->nz);
    bp_matched_kernel<<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const float *>(d_table), d_proj, d_vol, view0, nviews, scale, accumulate);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "bp_matched_kernel: %s", cudaGetErrorString(e));
    return CTGB_OK;
}
