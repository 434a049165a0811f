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

#include "dd_common.cuh"
#include "status.h"

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

__global__ void transpose_xy_kernel(const float *__restrict__ in, float *__restrict__ out, int nx, int ny) {
    __shared__ float tile[32][33];
    const int z = blockIdx.z;
    const int x0 = blockIdx.x * 32, y0 = blockIdx.y * 32;
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

}  // namespace ctgb

using namespace ctgb;

static int check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return CTGB_OK;
}

extern "C" int ctgb_forward(const ctgb_params *p, const void *d_table, const float *d_vol, const float *d_vol_xzy,
                            float *d_proj, int32_t view0, int32_t nviews, void *stream) {
    clear_error();
    if (!p || !d_table || !d_vol || !d_proj) return set_error(CTGB_ERR_ARG, "ctgb_forward: NULL argument");
    if (view0 < 0 || nviews < 0 || view0 + nviews > p->nviews)
        return set_error(CTGB_ERR_ARG, "ctgb_forward: view range [%d,%d) outside [0,%d)", view0, view0 + nviews,
                         p->nviews);
    if (nviews == 0) return CTGB_OK;
    dim3 block(kFwdTileU, kFwdTileV);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    for (int v = 0; v < nviews; v += 65535) {
        int nv_chunk = nviews - v < 65535 ? nviews - v : 65535;
        dim3 grid((p->nu + kFwdTileU - 1) / kFwdTileU, (p->nv + kFwdTileV - 1) / kFwdTileV, nv_chunk);
        dd_forward_kernel<<<grid, block, 0, st>>>(static_cast<const float *>(d_table), d_vol, d_vol_xzy,
                                                  d_proj + (long long)v * p->nu * p->nv, view0 + v);
    }
    return check_launch("dd_forward_kernel");
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
