// Ray-driven (Siddon) projector and its transpose.
//
// Semantics: matlab/RayDrivenProjection3DSiddon.m:55-180 (Siddon's method:
// the ray from the source to a detector pixel centre is cut by every voxel
// plane; between consecutive crossings lies one voxel, which contributes
// segment length x value), on the geometry of the Python class's
// `Method: 'Ray'` branch (python/Reconstruction_numba.py:788-789, a stub
// there): the same source positions, pixel centres (FlatDetectorConstruction
// / CurvedDetectorConstruction) and voxel planes as the DD forward.
//
// GB300 layout: one thread per ray (pixel x view), 32 x 4 pixel tiles so a
// warp's rays are neighbours.  The crossings are visited in order by an
// incremental 3-D traversal instead of Siddon's sort-and-merge: each axis
// keeps the index of its next plane, and the next crossing is the smallest
// of the three, computed from the plane index (no accumulated increments),
// so each segment's alpha interval equals the merged list's.  The transpose
// scatters segment x value with atomicAdd (order-dependent rounding only).
#include <cuda_runtime.h>

#include <cmath>

#include "../../include/ctgb.h"
#include "dd_common.cuh"
#include "status.h"

namespace ctgb {

constexpr int kRayTX = 32, kRayTY = 4;

template <bool SCATTER>
__global__ void __launch_bounds__(kRayTX * kRayTY)
ray_kernel(const float *__restrict__ T, const float *__restrict__ vol, const float *__restrict__ proj_in,
           float *__restrict__ out, int view0, float scale) {
    const TableHeader &h = header(T);
    const int c = blockIdx.x * kRayTX + threadIdx.x;
    const int r = blockIdx.y * kRayTY + threadIdx.y;
    const int vi = blockIdx.z;
    if (c >= h.nu || r >= h.nv) return;
    const ViewOffsets vo = view_offsets(h.nu, h.nv);
    const float *__restrict__ V = T + h.off_views + (long long)(view0 + vi) * h.view_stride;
    const long long pix = ((long long)vi * h.nv + r) * h.nu + c;
    float val = 0.0f;
    if (SCATTER) {
        val = proj_in[pix] * scale;
        if (val == 0.0f) return;
    }
    const float S[3] = {V[VF_SX], V[VF_SY], V[VF_SZ]};
    const float P[3] = {V[vo.px + c], V[vo.py + c], V[vo.pz + r]};
    const float p0[3] = {T[h.off_xplane], T[h.off_yplane], T[h.off_zplane]};
    const float d[3] = {h.dx, h.dy, h.dz};
    const int n[3] = {h.nx, h.ny, h.nz};
    float dir[3], inv[3], base[3];
    float amin = 0.0f, amax = 1.0f;
    const float tol = 1e-6f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        dir[a] = P[a] - S[a];
        base[a] = p0[a] - S[a];                 // alpha of plane k: (base + k d) / dir
        if (fabsf(dir[a]) < tol) {
            inv[a] = 0.0f;
            const float lo = fminf(p0[a], p0[a] + n[a] * d[a]), hi = fmaxf(p0[a], p0[a] + n[a] * d[a]);
            if (S[a] < lo || S[a] > hi) amax = -1.0f;       // parallel and outside: no intersection
        } else {
            inv[a] = 1.0f / dir[a];
            const float a0 = base[a] * inv[a], a1 = (base[a] + n[a] * d[a]) * inv[a];
            amin = fmaxf(amin, fminf(a0, a1));
            amax = fminf(amax, fmaxf(a0, a1));
        }
    }
    float acc = 0.0f;
    if (amin < amax && amax - amin >= tol) {
        const float L = sqrtf(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
        // First voxel: the one holding a point just past the entry.
        const float probe = amin + 1e-4f * (amax - amin);
        int idx[3], step[3];
        float anext[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float f = (S[a] + probe * dir[a] - p0[a]) / d[a];
            idx[a] = min(max((int)floorf(f), 0), n[a] - 1);
            if (inv[a] == 0.0f) {
                step[a] = 0;
                anext[a] = INFINITY;
            } else {
                step[a] = (dir[a] * d[a] > 0.0f) ? 1 : -1;      // index direction along the ray
                anext[a] = (base[a] + (float)(idx[a] + (step[a] > 0 ? 1 : 0)) * d[a]) * inv[a];
            }
        }
        float alpha = amin;
        const int max_steps = n[0] + n[1] + n[2] + 3;
        for (int it = 0; it < max_steps; ++it) {
            const float an = fminf(fminf(anext[0], anext[1]), fminf(anext[2], amax));
            const float seg = an - alpha;
            const long long vox = ((long long)idx[2] * h.ny + idx[1]) * h.nx + idx[0];
            if (seg > 0.0f) {
                if (SCATTER) atomicAdd(out + vox, seg * L * val);
                else acc = fmaf(seg, __ldg(vol + vox), acc);
            }
            if (an >= amax) break;
            bool inside = true;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                if (anext[a] <= an) {
                    idx[a] += step[a];
                    inside = inside && idx[a] >= 0 && idx[a] < n[a];
                    anext[a] = (base[a] + (float)(idx[a] + (step[a] > 0 ? 1 : 0)) * d[a]) * inv[a];
                }
            }
            if (!inside) break;
            alpha = an;
        }
        acc *= L;
    }
    if (!SCATTER) out[pix] = acc;
}

}  // namespace ctgb

using namespace ctgb;

static int ray_args(const ctgb_params *p, const void *t, const void *a, const void *b, int view0, int nviews,
                    const char *who) {
    if (!p || !t || !a || !b) return set_error(CTGB_ERR_ARG, "%s: NULL argument", who);
    if (view0 < 0 || nviews < 0 || view0 + nviews > p->nviews || nviews > 65535)
        return set_error(CTGB_ERR_ARG, "%s: view range [%d,%d) outside [0,%d)", who, view0, view0 + nviews,
                         p->nviews);
    return CTGB_OK;
}

extern "C" int ctgb_ray_forward(const ctgb_params *p, const void *d_table, const float *d_vol, float *d_proj,
                                int32_t view0, int32_t nviews, void *stream) {
    clear_error();
    if (int st = ray_args(p, d_table, d_vol, d_proj, view0, nviews, "ctgb_ray_forward")) return st;
    if (nviews == 0) return CTGB_OK;
    dim3 block(kRayTX, kRayTY), grid((p->nu + kRayTX - 1) / kRayTX, (p->nv + kRayTY - 1) / kRayTY, nviews);
    ray_kernel<false><<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const float *>(d_table), d_vol, nullptr, d_proj, view0, 1.0f);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "ray_kernel: %s", cudaGetErrorString(e));
    return CTGB_OK;
}

extern "C" int ctgb_ray_backproject(const ctgb_params *p, const void *d_table, const float *d_proj, float *d_vol,
                                    int32_t view0, int32_t nviews, float scale, int32_t accumulate, void *stream) {
    clear_error();
    if (int st = ray_args(p, d_table, d_proj, d_vol, view0, nviews, "ctgb_ray_backproject")) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (!accumulate) {
        cudaError_t e = cudaMemsetAsync(d_vol, 0, sizeof(float) * (size_t)p->nx * p->ny * p->nz, s);
        if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "memset: %s", cudaGetErrorString(e));
    }
    if (nviews == 0) return CTGB_OK;
    dim3 block(kRayTX, kRayTY), grid((p->nu + kRayTX - 1) / kRayTX, (p->nv + kRayTY - 1) / kRayTY, nviews);
    ray_kernel<true><<<grid, block, 0, s>>>(static_cast<const float *>(d_table), nullptr, d_proj, d_vol, view0,
                                            scale);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "ray_kernel: %s", cudaGetErrorString(e));
    return CTGB_OK;
}
