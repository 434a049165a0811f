// Voxel-driven FDK of the standalone cone-beam reconstructor
// (python/ConeBeamGPU.py:161-321; CPU twin python/ConeBeam.py:86-167), and
// the 2-D fan-beam FBP backprojection (python/FanBeam.py:82-138 equispaced
// "line" detector; matlab/FanBeamReconArc.m:20-47 equiangular "arc").
//
// Cone beam (ConeBeamGPU.Reconstruction with its kernels CalculateInterpolGrid
// and Interpol2dLineargpu, python/GPUFuncs_pycuda.py:40-102):
//   per voxel (x, y, z) and view theta:  t = x cos + y sin,  s = -x sin + y cos,
//   U = R t / (R - s),  V = R z / (R - s),  W = R^2 / (R - s)^2,
//   recon += dtheta * W * bilinear(Q, U, V)  on the iso-scaled detector grid,
//   nothing where (U, V) falls outside the grid (fill value 0).
// GB300 layout: one thread per (x, y) column with kCbZ voxels of z in
// registers and all views in one launch (the reference launches two kernels
// per view and re-uploads the grid); U, W and the u interpolation weights are
// z-independent and computed once per (column, view).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/ctgb.h"
#include "status.h"

namespace ctgb {

struct CbHeader {
    int32_t X, Y, Z, nx, ny, nviews;
    float R, dtheta;
    float u0, du, v0, dv;          // iso-scaled detector grid: first sample and spacing
    int32_t pad[4];
    int64_t off_x, off_y, off_z, off_cos, off_sin, off_ki, off_p, total;
};

// CTAs of 4 x 32 voxel columns, so each warp is a 4 x 8 patch that samples
// nearby detector rows and columns at every view angle (15.1 ms against
// 15.3 ms for 32 x 4 at 256^3 / 360 views: this kernel waits mostly on its
// dependent grid and sample loads, not on their spread).
#ifndef CTGB_CB_TX
#define CTGB_CB_TX 4
#endif
constexpr int kCbZ = 16, kCbTX = CTGB_CB_TX, kCbTY = 128 / CTGB_CB_TX;

__device__ __forceinline__ void lin_weights(float xq, float x0, float inv_dx, const float *__restrict__ grid, int n,
                                            int *lo, int *hi, float *a, float *b, bool *ok) {
    // GFp Interpol2dLineargpu: XLow = floor, XHigh = ceil, w1 = x - grid[lo],
    // w2 = grid[hi] - x, (w1, w2 ~ 0) -> w1 = 1; weights w2/(w1+w2), w1/(w1+w2).
    const float f = (xq - x0) * inv_dx;
    const int l = (int)floorf(f), h = (int)ceilf(f);
    *ok = (h < n) && (l >= 0);
    const int lc = min(max(l, 0), n - 1), hc = min(max(h, 0), n - 1);
    float w1 = xq - grid[lc], w2 = grid[hc] - xq;
    if (fabsf(w1) < 1e-4f && fabsf(w2) < 1e-4f) w1 = 1.0f;
    // fast reciprocal (a few ulp; w1 + w2 is the grid pitch or 1 + w2)
    const float inv = __fdividef(1.0f, w1 + w2);
    *lo = lc; *hi = hc;
    *a = w2 * inv; *b = w1 * inv;
}

__global__ void __launch_bounds__(kCbTX * kCbTY)
conebeam_bp_kernel(const float *__restrict__ T, const float *__restrict__ Q, float *__restrict__ recon, int view0,
                   int nviews, int accumulate) {
    const CbHeader &h = *reinterpret_cast<const CbHeader *>(T);
    const int tx = blockIdx.x * kCbTX + threadIdx.x;
    const int ty = blockIdx.y * kCbTY + threadIdx.y;
    const int z0 = blockIdx.z * kCbZ;
    if (tx >= h.X || ty >= h.Y) return;
    const float xx = T[h.off_x + tx], yy = T[h.off_y + ty];
    const float *__restrict__ zs = T + h.off_z;
    const float *__restrict__ ki = T + h.off_ki;
    const float *__restrict__ pg = T + h.off_p;
    const int nx = h.nx, ny = h.ny;
    const float R = h.R, dth = h.dtheta;
    const float inv_du = 1.0f / h.du, inv_dv = 1.0f / h.dv;
    float acc[kCbZ];
#pragma unroll
    for (int j = 0; j < kCbZ; ++j) acc[j] = 0.0f;
    for (int vi = 0; vi < nviews; ++vi) {
        const int v = view0 + vi;
        const float c = T[h.off_cos + v], s_ = T[h.off_sin + v];
        const float t = xx * c + yy * s_;
        const float s = -xx * s_ + yy * c;
        const float rs = R - s;
        const float U = (R * t) / rs;
        const float W = (R * R) / (rs * rs) * dth;
        int ulo, uhi;
        float ua, ub;
        bool uok;
        lin_weights(U, h.u0, inv_du, ki, nx, &ulo, &uhi, &ua, &ub, &uok);
        if (!uok) continue;
        const float *__restrict__ q = Q + (long long)vi * nx * ny;
        const float Rz = R / rs;
#pragma unroll
        for (int j = 0; j < kCbZ; ++j) {
            const int iz = min(z0 + j, h.Z - 1);
            const float V = Rz * zs[iz];
            int vlo, vhi;
            float va, vb;
            bool vok;
            lin_weights(V, h.v0, inv_dv, pg, ny, &vlo, &vhi, &va, &vb, &vok);
            if (vok) {
                const float *r0 = q + (long long)vlo * nx, *r1 = q + (long long)vhi * nx;
                const float M = ua * __ldg(r0 + ulo) + ub * __ldg(r0 + uhi);
                const float N = ua * __ldg(r1 + ulo) + ub * __ldg(r1 + uhi);
                acc[j] = fmaf(va * M + vb * N, W, acc[j]);
            }
        }
    }
#pragma unroll
    for (int j = 0; j < kCbZ; ++j) {
        const int iz = z0 + j;
        if (iz < h.Z) {
            float *d = recon + ((long long)iz * h.Y + ty) * h.X + tx;
            *d = accumulate ? *d + acc[j] : acc[j];
        }
    }
}

}  // namespace ctgb

using namespace ctgb;

static bool cb_valid(const ctgb_conebeam_params *p) {
    return p && p->source_to_axis > 0 && p->source_to_detector > p->source_to_axis && p->pixel_width > 0 &&
           p->pixel_height > 0 && p->det_width >= 2 && p->det_height >= 2 && p->nviews >= 1 && p->recon_x >= 1 &&
           p->recon_y >= 1 && p->recon_z >= 1;
}

static CbHeader cb_layout(const ctgb_conebeam_params *p) {
    CbHeader h;
    std::memset(&h, 0, sizeof h);
    h.X = p->recon_x; h.Y = p->recon_y; h.Z = p->recon_z;
    h.nx = p->det_width; h.ny = p->det_height; h.nviews = p->nviews;
    int64_t off = (sizeof(CbHeader) + 127) / 128 * 32;
    auto take = [&](int64_t n) { int64_t o = off; off += (n + 31) / 32 * 32; return o; };
    h.off_x = take(h.X);
    h.off_y = take(h.Y);
    h.off_z = take(h.Z);
    h.off_cos = take(h.nviews);
    h.off_sin = take(h.nviews);
    h.off_ki = take(h.nx);
    h.off_p = take(h.ny);
    h.total = off;
    return h;
}

extern "C" int ctgb_conebeam_table_bytes(const ctgb_conebeam_params *p, size_t *bytes) {
    clear_error();
    if (!cb_valid(p) || !bytes) return set_error(CTGB_ERR_ARG, "ctgb_conebeam_table_bytes: bad geometry");
    *bytes = (size_t)cb_layout(p).total * sizeof(float);
    return CTGB_OK;
}

// ConeBeamGPU.py:205-248: fov from the detector size, voxel grids by
// linspace(-fov/2, fov/2, n), view angles linspace(0, coverage, ns+1)[:-1],
// iso-scaled detector grids ki, p.
extern "C" int ctgb_conebeam_table_build(const ctgb_conebeam_params *p, void *host, size_t bytes) {
    size_t need = 0;
    int st = ctgb_conebeam_table_bytes(p, &need);
    if (st) return st;
    if (!host || bytes < need) return set_error(CTGB_ERR_SIZE, "ctgb_conebeam_table_build: buffer too small");
    std::memset(host, 0, need);
    CbHeader h = cb_layout(p);
    float *T = static_cast<float *>(host);
    const double R = p->source_to_axis, D = p->source_to_detector - R;
    const double fov = 2 * R * std::sin(std::atan(p->det_width * p->pixel_width / 2 / (D + R)));
    const double fovz = 2 * R * std::sin(std::atan(p->det_height * p->pixel_height / 2 / (D + R)));
    auto linspace = [](double a, double b, int n, float *out) {
        if (n == 1) { out[0] = (float)a; return; }
        const double step = (b - a) / (n - 1);
        for (int i = 0; i < n; ++i) out[i] = (float)(a + i * step);
        out[n - 1] = (float)b;
    };
    linspace(-fov / 2, fov / 2, h.X, T + h.off_x);
    linspace(-fov / 2, fov / 2, h.Y, T + h.off_y);
    linspace(-fovz / 2, fovz / 2, h.Z, T + h.off_z);
    const double step = p->angle_coverage / p->nviews;
    for (int v = 0; v < h.nviews; ++v) {
        const double a = v * step;
        T[h.off_cos + v] = (float)std::cos(a);
        T[h.off_sin + v] = (float)std::sin(a);
    }
    h.dtheta = (float)(h.nviews > 1 ? step : 0.0);
    h.R = (float)R;
    for (int i = 0; i < h.nx; ++i) T[h.off_ki + i] = (float)((i - (h.nx - 1) / 2.0) * p->pixel_width * R / (R + D));
    for (int i = 0; i < h.ny; ++i) T[h.off_p + i] = (float)((i - (h.ny - 1) / 2.0) * p->pixel_height * R / (R + D));
    h.u0 = T[h.off_ki];
    h.du = T[h.off_ki + 1] - T[h.off_ki];
    h.v0 = T[h.off_p];
    h.dv = T[h.off_p + 1] - T[h.off_p];
    std::memcpy(host, &h, sizeof h);
    return CTGB_OK;
}

extern "C" int ctgb_conebeam_backproject(const ctgb_conebeam_params *p, const void *d_table, const float *d_q,
                                         float *d_recon, int32_t view0, int32_t nviews, int32_t accumulate,
                                         void *stream) {
    clear_error();
    if (!cb_valid(p) || !d_table || !d_q || !d_recon)
        return set_error(CTGB_ERR_ARG, "ctgb_conebeam_backproject: bad arguments");
    if (view0 < 0 || nviews < 0 || view0 + nviews > p->nviews)
        return set_error(CTGB_ERR_ARG, "ctgb_conebeam_backproject: view range outside the scan");
    dim3 block(kCbTX, kCbTY);
    dim3 grid((p->recon_x + kCbTX - 1) / kCbTX, (p->recon_y + kCbTY - 1) / kCbTY, (p->recon_z + kCbZ - 1) / kCbZ);
    conebeam_bp_kernel<<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const float *>(d_table), d_q, d_recon, view0, nviews, accumulate);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "conebeam_bp_kernel: %s", cudaGetErrorString(e));
    return CTGB_OK;
}

// ---------------------------------------------------------------------------
// Batched fan-beam backprojection (persistent work list).
namespace ctgb {

struct FanBatchHeader {
    int32_t nslices, nitems, tile_x, tile_y, max_views, pad[3];
    int64_t off_slices, off_items;     // in 4-byte words from the base
};

// Linear interpolation of one sinogram row at channel position f
// (interp1d(kind='linear', bounds_error=False, fill_value=0)).
__device__ __forceinline__ float fan_sample(const float *__restrict__ row, float f, float last, int nch) {
    if (!(f >= 0.0f && f <= last)) return 0.0f;
    const int k = min((int)f, nch - 2);
    const float fr = f - (float)k;
    const float a = __ldg(row + k), b = __ldg(row + k + 1);
    return fmaf(fr, b - a, a);
}

// Each thread owns two pixels of an item's tile, rows j and j + blockDim.y
// of the same column, so the per-view geometry of both (t, s, the
// interpolation position and the distance weight) runs on packed f32x2
// operations; the launch uses tile_y / 2 thread rows for a tile_y-row tile.
__global__ void fan_bp_kernel(const int *__restrict__ B, const float *__restrict__ sino, float *__restrict__ images,
                              int accumulate) {
    extern __shared__ float2 cs[];     // (cos, sin) per view of the current item's slice
    const FanBatchHeader &h = *reinterpret_cast<const FanBatchHeader *>(B);
    const ctgb_fan_slice *S = reinterpret_cast<const ctgb_fan_slice *>(B + h.off_slices);
    const int4 *items = reinterpret_cast<const int4 *>(B + h.off_items);
    const int tid = threadIdx.y * blockDim.x + threadIdx.x, nthr = blockDim.x * blockDim.y;
    for (int it = blockIdx.x; it < h.nitems; it += gridDim.x) {
        const int4 w = items[it];       // (slice, tile x0, tile y0, 0)
        const ctgb_fan_slice sl = S[w.x];
        __syncthreads();                // previous item's table no longer read
        for (int v = tid; v < sl.nviews; v += nthr) {
            float sv, cv;
            sincosf(sl.theta0 + v * sl.dtheta, &sv, &cv);
            cs[v] = make_float2(cv, sv);
        }
        __syncthreads();
        const int i = w.y + threadIdx.x, j0 = w.z + threadIdx.y, j1 = j0 + blockDim.y;
        // the second row only inside this item's tile (odd tile heights)
        const bool in0 = i < sl.nx && j0 < sl.ny;
        const bool in1 = i < sl.nx && j1 < sl.ny && (int)(threadIdx.y + blockDim.y) < h.tile_y;
        if (!in0) continue;             // row j1 > j0: nothing in this thread's column either
        const float x = sl.x0 + i * sl.dx;
        const float2 y2 = make_float2(sl.y0 + j0 * sl.dy, sl.y0 + j1 * sl.dy);
        const float *__restrict__ q = sino + sl.sino_offset;
        const float inv_dg = 1.0f / sl.dg, inv_D = 1.0f / sl.D;
        const float last = (float)(sl.nch - 1);
        const float2 R2 = make_float2(sl.R, sl.R), m1 = make_float2(-1.0f, -1.0f);
        float acc0 = 0.0f, acc1 = 0.0f;
        // Fast reciprocals (a few ulp) instead of IEEE divides: well inside
        // the 1e-4 agreement with the FP64 restatement.
        for (int v = 0; v < sl.nviews; ++v) {
            const float2 c = cs[v];
            // t = x cos + y sin, s = -x sin + y cos for both pixels
            const float2 t2 = __ffma2_rn(y2, make_float2(c.y, c.y), make_float2(x * c.x, x * c.x));
            const float2 s2 = __ffma2_rn(y2, make_float2(c.x, c.x), make_float2(-x * c.y, -x * c.y));
            const float2 den = __ffma2_rn(s2, m1, R2);
            float2 f, wgt;
            if (sl.arc) {
                // matlab/FanBeamReconArc.m:37-44: gamma' = atan(t / (R - s)), 1 / L^2.
                f = make_float2((atan2f(t2.x, den.x) - sl.g0) * inv_dg, (atan2f(t2.y, den.y) - sl.g0) * inv_dg);
                const float2 L2 = __ffma2_rn(den, den, __fmul2_rn(t2, t2));
                wgt = make_float2(__fdividef(1.0f, L2.x), __fdividef(1.0f, L2.y));
            } else {
                // FanBeam.py:123-129: InterpX = R t / (R - s); U = (D - s) / D.
                const float2 rden = make_float2(__fdividef(1.0f, den.x), __fdividef(1.0f, den.y));
                f = __fmul2_rn(__ffma2_rn(__fmul2_rn(R2, t2), rden, make_float2(-sl.g0, -sl.g0)),
                               make_float2(inv_dg, inv_dg));
                const float2 U = __fmul2_rn(__ffma2_rn(s2, m1, make_float2(sl.D, sl.D)), make_float2(inv_D, inv_D));
                const float2 UU = __fmul2_rn(U, U);
                wgt = make_float2(__fdividef(1.0f, UU.x), __fdividef(1.0f, UU.y));
            }
            const float *__restrict__ row = q + (long long)v * sl.nch;
            acc0 = fmaf(fan_sample(row, f.x, last, sl.nch), wgt.x, acc0);
            if (in1) acc1 = fmaf(fan_sample(row, f.y, last, sl.nch), wgt.y, acc1);
        }
        float *dst = images + sl.image_offset + (long long)j0 * sl.nx + i;
        const float val0 = acc0 * sl.dtheta;
        *dst = accumulate ? *dst + val0 : val0;
        if (in1) {
            float *dst1 = images + sl.image_offset + (long long)j1 * sl.nx + i;
            const float val1 = acc1 * sl.dtheta;
            *dst1 = accumulate ? *dst1 + val1 : val1;
        }
    }
}

}  // namespace ctgb

static bool fan_valid(const ctgb_fan_slice *s, int n, int tx, int ty) {
    if (!s || n < 1 || tx < 1 || ty < 1 || tx * ty > 1024) return false;
    for (int i = 0; i < n; ++i)
        if (s[i].nx < 1 || s[i].ny < 1 || s[i].nch < 2 || s[i].nviews < 1 || !(s[i].dg != 0.0f) ||
            s[i].sino_offset < 0 || s[i].image_offset < 0 || s[i].nviews > 8192)
            return false;
    return true;
}

static long long fan_items(const ctgb_fan_slice *s, int n, int tx, int ty) {
    long long c = 0;
    for (int i = 0; i < n; ++i) c += (long long)((s[i].nx + tx - 1) / tx) * ((s[i].ny + ty - 1) / ty);
    return c;
}

extern "C" int ctgb_fan_batch_bytes(const ctgb_fan_slice *slices, int32_t nslices, int32_t tile_x, int32_t tile_y,
                                    size_t *bytes) {
    clear_error();
    if (!fan_valid(slices, nslices, tile_x, tile_y) || !bytes)
        return set_error(CTGB_ERR_ARG, "ctgb_fan_batch_bytes: bad slices or tile");
    const long long items = fan_items(slices, nslices, tile_x, tile_y);
    if (items > 0x7fffffffLL) return set_error(CTGB_ERR_SIZE, "ctgb_fan_batch_bytes: too many tiles");
    const size_t hdr = (sizeof(FanBatchHeader) + 15) / 16 * 16;
    *bytes = hdr + sizeof(ctgb_fan_slice) * nslices + 16 * (size_t)items;
    return CTGB_OK;
}

extern "C" int ctgb_fan_batch_build(const ctgb_fan_slice *slices, int32_t nslices, int32_t tile_x, int32_t tile_y,
                                    void *host_buf, size_t bytes) {
    size_t need = 0;
    int st = ctgb_fan_batch_bytes(slices, nslices, tile_x, tile_y, &need);
    if (st) return st;
    if (!host_buf || bytes < need) return set_error(CTGB_ERR_SIZE, "ctgb_fan_batch_build: buffer too small");
    std::memset(host_buf, 0, need);
    FanBatchHeader h;
    std::memset(&h, 0, sizeof h);
    const size_t hdr = (sizeof(FanBatchHeader) + 15) / 16 * 16;
    h.nslices = nslices;
    h.tile_x = tile_x;
    h.tile_y = tile_y;
    h.off_slices = (int64_t)(hdr / 4);
    h.off_items = (int64_t)((hdr + sizeof(ctgb_fan_slice) * nslices) / 4);
    unsigned char *base = static_cast<unsigned char *>(host_buf);
    std::memcpy(base + hdr, slices, sizeof(ctgb_fan_slice) * nslices);
    int *items = reinterpret_cast<int *>(base + h.off_items * 4);
    long long c = 0;
    for (int i = 0; i < nslices; ++i) {
        h.max_views = std::max(h.max_views, slices[i].nviews);
        for (int y0 = 0; y0 < slices[i].ny; y0 += tile_y)
            for (int x0 = 0; x0 < slices[i].nx; x0 += tile_x) {
                items[4 * c + 0] = i; items[4 * c + 1] = x0; items[4 * c + 2] = y0; items[4 * c + 3] = 0;
                ++c;
            }
    }
    h.nitems = (int32_t)c;
    std::memcpy(host_buf, &h, sizeof h);
    return CTGB_OK;
}

extern "C" int ctgb_fan_backproject(const void *d_batch, int32_t max_views, const float *d_sino, float *d_images,
                                    int32_t tile_x, int32_t tile_y, int32_t grid_blocks, int32_t accumulate,
                                    void *stream) {
    clear_error();
    if (!d_batch || !d_sino || !d_images || tile_x < 1 || tile_y < 1 || tile_x * tile_y > 1024 || grid_blocks < 1 ||
        max_views < 1 || max_views > 8192)
        return set_error(CTGB_ERR_ARG, "ctgb_fan_backproject: bad arguments");
    const size_t smem = (size_t)max_views * sizeof(float2);
    static std::atomic<unsigned long long> attr{0};
    cudaError_t ea = smem_limit_once((const void *)fan_bp_kernel, (int)(8192 * sizeof(float2)), attr);
    if (ea != cudaSuccess) return set_error(CTGB_ERR_CUDA, "fan_bp smem: %s", cudaGetErrorString(ea));
    // two pixel rows per thread: tile_y / 2 thread rows (a tile of one row
    // keeps one thread row and its second pixel falls outside the tile)
    const int rows = tile_y > 1 ? (tile_y + 1) / 2 : 1;
    fan_bp_kernel<<<grid_blocks, dim3(tile_x, rows), smem, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const int *>(d_batch), d_sino, d_images, accumulate);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "fan_bp_kernel: %s", cudaGetErrorString(e));
    return CTGB_OK;
}
