// Element-wise and stencil kernels of the iterative drivers.
//
// Each kernel restates one update line of the reference scripts in float32
// (the reference works on float32 NumPy arrays):
//   SART      python/SART.py:51,55
//   MLEM      python/EM.py:36-42
//   ASD-POCS  python/ASD_POCS.py:174-179 (POCS), :55-77 (tv_grad), :183,189 (norms)
// The update passes may run in place (x_prev == x: each element is read, then
// written, by the same thread), so those two pointers are not __restrict__.
// All are HBM-bound streaming passes (grid-stride loops over 4-float
// vectors where the arrays allow it).  Reductions are deterministic: each
// block writes one double partial sum, and the consumer sums the partials in
// a fixed order.
#include <cuda_runtime.h>

#include "../../include/ctgb.h"
#include "status.h"
#include "updates.cuh"

namespace ctgb {

constexpr int kEwThreads = 256;

static int ew_blocks(long long n) {
    long long b = (n + kEwThreads * 4 - 1) / (kEwThreads * 4);
    if (b < 1) b = 1;
    if (b > 152 * 16) b = 152 * 16;
    return (int)b;
}

// SART.py:51  r = (Ax - p0) / (A1 + eps)
__global__ void sart_residual_kernel(const float *__restrict__ ax, const float *__restrict__ p0,
                                     const float *__restrict__ a1, float eps, float *__restrict__ out, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = sart_residual(ax[i], p0[i], a1[i], eps);
}

// SART.py:55  x = x_prev - alpha * (bp / norm1 + eps)   (eps added after the division, as written)
__global__ void sart_update_kernel(const float *xp, const float *__restrict__ bp,
                                   const float *__restrict__ n1, float alpha, float eps, float *x,
                                   long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] = sart_update(xp[i], bp[i], n1[i], alpha, eps);
}

// EM.py:36-39  p0[Ax == 0] = 0 (in place: the script's proj0 aliases the
// measured data); Ax[Ax == 0] = eps; r = p0 / Ax
__global__ void em_ratio_kernel(float *__restrict__ p0, const float *__restrict__ ax, float eps,
                                float *__restrict__ out, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        out[i] = em_ratio(p0 + i, ax[i], eps);
    }
}

// EM.py:41-42  x = x_prev * (bp / norm)
__global__ void em_update_kernel(const float *xp, const float *__restrict__ bp,
                                 const float *__restrict__ nrm, float *x, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] = em_update(xp[i], bp[i], nrm[i]);
}

// ASD_POCS.py:174-175  r = (p0 - Ax) / (A1 + eps); r[A1 == 0] = 0
__global__ void pocs_residual_kernel(const float *__restrict__ p0, const float *__restrict__ ax,
                                     const float *__restrict__ a1, float eps, float *__restrict__ out, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        out[i] = pocs_residual(p0[i], ax[i], a1[i], eps);
    }
}

// ASD_POCS.py:177-179  bp[norm1 == 0] = 0; x = x_prev + beta * bp / (norm1 + eps); x[x < 0] = 0
__global__ void pocs_update_kernel(const float *xp, const float *__restrict__ bp,
                                   const float *__restrict__ n1, float beta, float eps, float *x,
                                   long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        x[i] = pocs_update(xp[i], bp[i], n1[i], beta, eps);
    }
}

// tv_grad (ASD_POCS.py:55-77) at interior voxel (i, j, k) of a [n0][n1][n2]
// array: the sum of the four one-sided terms, before normalisation.  Each
// term is w * rsqrtf(eps + |w|^2) rather than an IEEE square root and
// division: the four IEEE pairs made this pass instruction-bound (246 us
// per TV step at 256^3), and the step only uses dtv / ||dtv|| scaled by a
// small step, so the few-ulp difference stays far below float32 noise in x.
__device__ __forceinline__ float tv_term(const float *__restrict__ x, int n1, int n2, int i, int j, int k, float eps) {
    const long long s0 = (long long)n1 * n2, s1 = n2;
    const long long c = i * s0 + j * s1 + k;
    const float v = x[c];
    const float w1 = v - x[c - s0], w2 = v - x[c - s1], w3 = v - x[c - 1];
    const float t1 = (w1 + w2 + w3) * rsqrtf(eps + w1 * w1 + w2 * w2 + w3 * w3);
    const float xi = x[c + s0];
    const float w4 = xi - v, w5 = xi - x[c + s0 - s1], w6 = xi - x[c + s0 - 1];
    const float t2 = -w4 * rsqrtf(eps + w4 * w4 + w5 * w5 + w6 * w6);
    const float xj = x[c + s1];
    const float w7 = xj - x[c - s0 + s1], w8 = xj - v, w9 = xj - x[c + s1 - 1];
    const float t3 = -w8 * rsqrtf(eps + w7 * w7 + w8 * w8 + w9 * w9);
    const float xk = x[c + 1];
    const float w10 = xk - x[c - s0 + 1], w11 = xk - x[c - s1 + 1], w12 = xk - v;
    const float t4 = -w12 * rsqrtf(eps + w10 * w10 + w11 * w11 + w12 * w12);
    return t1 + t2 + t3 + t4;
}

// Pass 1: dtv at every interior voxel, written to y (the output array, used
// as scratch), and per-block partial sums of dtv^2.  Each warp walks whole
// rows (i, j) of the array (rows distributed grid-stride over the block's
// warps), its lanes striding along k, so the only integer division is one
// 32-bit split of the row index per row.
__global__ void tv_norm_kernel(const float *__restrict__ x, float *__restrict__ y, int n0, int n1, int n2, float eps,
                               double *__restrict__ partials) {
    __shared__ double red[kEwThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    const unsigned m1 = (unsigned)(n1 - 2), rows = (unsigned)(n0 - 2) * m1;
    double acc = 0.0;
    for (unsigned r = blockIdx.x * wpb + warp; r < rows; r += gridDim.x * wpb) {
        const int i = (int)(r / m1) + 1, j = (int)(r % m1) + 1;
        float *__restrict__ yrow = y + ((long long)i * n1 + j) * n2;
        float racc = 0.0f;
        for (int k = 1 + lane; k < n2 - 1; k += 32) {
            const float d = tv_term(x, n1, n2, i, j, k, eps);
            yrow[k] = d;
            racc = fmaf(d, d, racc);
        }
        acc += (double)racc;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) red[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < wpb; ++w) s += red[w];
        partials[blockIdx.x] = s;
    }
}

// Pass 1b: partials[0] = sum of partials[0 .. np-1] (one block, fixed order:
// per-thread strided sums, then a tree).
constexpr int kReduceThreads = 1024;

__global__ void __launch_bounds__(kReduceThreads) reduce_partials_kernel(double *partials, int np) {
    __shared__ double red[kReduceThreads];
    double s = 0.0;
    for (int b = threadIdx.x; b < np; b += kReduceThreads) s += partials[b];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = kReduceThreads / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partials[0] = red[0];
}

// Pass 2 (streaming): y = x - step * dtv / ||dtv|| with dtv from pass 1 in y
// (||dtv|| -> 1 when below eps) and ||dtv||^2 in partials[0]; the border of y
// is x's border (tv_grad pads dtv with zeros).
__global__ void tv_step_kernel(const float *__restrict__ x, float *__restrict__ y, int n0, int n1, int n2, float eps,
                               const double *__restrict__ partials, float step) {
    float nrm = (float)sqrt(partials[0]);
    if (fabsf(nrm) < eps) nrm = 1.0f;
    const float inv = 1.0f / nrm;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    const unsigned rows = (unsigned)n0 * (unsigned)n1;
    for (unsigned r = blockIdx.x * wpb + warp; r < rows; r += gridDim.x * wpb) {
        const int i = (int)(r / (unsigned)n1), j = (int)(r % (unsigned)n1);
        const long long base = (long long)r * n2;
        const bool inner_row = i > 0 && i < n0 - 1 && j > 0 && j < n1 - 1;
        for (int k = lane; k < n2; k += 32) {
            float v = x[base + k];
            if (inner_row && k > 0 && k < n2 - 1) v = v - step * (y[base + k] * inv);
            y[base + k] = v;
        }
    }
}

__device__ __forceinline__ double sum_partials(const double *__restrict__ partials, int np) {
    double s = 0.0;
    for (int b = 0; b < np; ++b) s += partials[b];
    return s;
}

// Per-block partial sums of (a - b)^2 (b may be NULL: sum of a^2).
__global__ void sqdist_kernel(const float *__restrict__ a, const float *__restrict__ b, long long n,
                              double *__restrict__ partials) {
    __shared__ double red[kEwThreads / 32];
    double acc = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float d = b ? a[i] - b[i] : a[i];
        acc += (double)d * d;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < kEwThreads / 32; ++w) s += red[w];
        partials[blockIdx.x] = s;
    }
}

// out[0] = sum of partials (one thread).
__global__ void sum_partials_kernel(const double *__restrict__ partials, int np, double *__restrict__ out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) out[0] = sum_partials(partials, np);
}

}  // namespace ctgb

using namespace ctgb;

static int ew_check(const char *who, long long n, const void *a, const void *b) {
    if (n < 0 || !a || !b) return set_error(CTGB_ERR_ARG, "%s: bad arguments", who);
    return CTGB_OK;
}

static int launched(const char *who) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "%s: %s", who, cudaGetErrorString(e));
    return CTGB_OK;
}

#define EW_LAUNCH(kernel, n, stream, ...)                                                                    \
    kernel<<<ew_blocks(n), kEwThreads, 0, static_cast<cudaStream_t>(stream)>>>(__VA_ARGS__)

extern "C" int ctgb_partials_count(int64_t n, int32_t *count) {
    clear_error();
    if (!count || n < 0) return set_error(CTGB_ERR_ARG, "ctgb_partials_count: bad arguments");
    *count = ew_blocks(n);
    return CTGB_OK;
}

extern "C" int ctgb_sart_residual(const float *ax, const float *p0, const float *a1, float eps, float *out, int64_t n,
                                  void *stream) {
    clear_error();
    if (int st = ew_check("ctgb_sart_residual", n, ax, out)) return st;
    if (!p0 || !a1) return set_error(CTGB_ERR_ARG, "ctgb_sart_residual: NULL argument");
    if (n == 0) return CTGB_OK;
    EW_LAUNCH(sart_residual_kernel, n, stream, ax, p0, a1, eps, out, n);
    return launched("ctgb_sart_residual");
}

extern "C" int ctgb_sart_update(const float *x_prev, const float *bp, const float *norm1, float alpha, float eps,
                                float *x, int64_t n, void *stream) {
    clear_error();
    if (int st = ew_check("ctgb_sart_update", n, x_prev, x)) return st;
    if (!bp || !norm1) return set_error(CTGB_ERR_ARG, "ctgb_sart_update: NULL argument");
    if (n == 0) return CTGB_OK;
    EW_LAUNCH(sart_update_kernel, n, stream, x_prev, bp, norm1, alpha, eps, x, n);
    return launched("ctgb_sart_update");
}

extern "C" int ctgb_em_ratio(float *p0, const float *ax, float eps, float *out, int64_t n, void *stream) {
    clear_error();
    if (int st = ew_check("ctgb_em_ratio", n, p0, ax)) return st;
    if (!out) return set_error(CTGB_ERR_ARG, "ctgb_em_ratio: NULL argument");
    if (n == 0) return CTGB_OK;
    EW_LAUNCH(em_ratio_kernel, n, stream, p0, ax, eps, out, n);
    return launched("ctgb_em_ratio");
}

extern "C" int ctgb_em_update(const float *x_prev, const float *bp, const float *norm, float *x, int64_t n,
                              void *stream) {
    clear_error();
    if (int st = ew_check("ctgb_em_update", n, x_prev, x)) return st;
    if (!bp || !norm) return set_error(CTGB_ERR_ARG, "ctgb_em_update: NULL argument");
    if (n == 0) return CTGB_OK;
    EW_LAUNCH(em_update_kernel, n, stream, x_prev, bp, norm, x, n);
    return launched("ctgb_em_update");
}

extern "C" int ctgb_pocs_residual(const float *p0, const float *ax, const float *a1, float eps, float *out,
                                  int64_t n, void *stream) {
    clear_error();
    if (int st = ew_check("ctgb_pocs_residual", n, p0, out)) return st;
    if (!ax || !a1) return set_error(CTGB_ERR_ARG, "ctgb_pocs_residual: NULL argument");
    if (n == 0) return CTGB_OK;
    EW_LAUNCH(pocs_residual_kernel, n, stream, p0, ax, a1, eps, out, n);
    return launched("ctgb_pocs_residual");
}

extern "C" int ctgb_pocs_update(const float *x_prev, const float *bp, const float *norm1, float beta, float eps,
                                float *x, int64_t n, void *stream) {
    clear_error();
    if (int st = ew_check("ctgb_pocs_update", n, x_prev, x)) return st;
    if (!bp || !norm1) return set_error(CTGB_ERR_ARG, "ctgb_pocs_update: NULL argument");
    if (n == 0) return CTGB_OK;
    EW_LAUNCH(pocs_update_kernel, n, stream, x_prev, bp, norm1, beta, eps, x, n);
    return launched("ctgb_pocs_update");
}

extern "C" int ctgb_tv_step(const float *x, float *y, int32_t n0, int32_t n1, int32_t n2, float eps, float step,
                            double *partials, void *stream) {
    clear_error();
    if (!x || !y || !partials || n0 < 1 || n1 < 1 || n2 < 1 || x == y)
        return set_error(CTGB_ERR_ARG, "ctgb_tv_step: bad arguments (x and y must differ)");
    const long long tot = (long long)n0 * n1 * n2;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nb = ew_blocks(tot);
    if (n0 < 3 || n1 < 3 || n2 < 3) {
        cudaError_t e = cudaMemcpyAsync(y, x, sizeof(float) * tot, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "ctgb_tv_step: %s", cudaGetErrorString(e));
        return CTGB_OK;
    }
    tv_norm_kernel<<<nb, kEwThreads, 0, st>>>(x, y, n0, n1, n2, eps, partials);
    reduce_partials_kernel<<<1, kReduceThreads, 0, st>>>(partials, nb);
    tv_step_kernel<<<nb, kEwThreads, 0, st>>>(x, y, n0, n1, n2, eps, partials, step);
    return launched("ctgb_tv_step");
}

extern "C" int ctgb_sqdist(const float *a, const float *b, int64_t n, double *partials, double *out, void *stream) {
    clear_error();
    if (!a || !partials || !out || n < 0) return set_error(CTGB_ERR_ARG, "ctgb_sqdist: bad arguments");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nb = ew_blocks(n);
    sqdist_kernel<<<nb, kEwThreads, 0, st>>>(a, b, n, partials);
    sum_partials_kernel<<<1, 32, 0, st>>>(partials, nb, out);
    return launched("ctgb_sqdist");
}
