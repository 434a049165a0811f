// FDK filtering: cosine pre-weight + zero-padded ramp filter along u, in place.
//
// Restates Reconstruction.Filtering / filter_proj / Filter
// (python/Reconstruction_numba.py:190-259): for each detector row,
//   Q = real(ifft(ifftshift(filter * fftshift(fft(weight * row, zpl)))))[:nu] * deltaS
// with zpl = 2^ceil(log2(2(nu-1))).  For even zpl the shifts cancel into
// ifftshift(filter), a real spectrum; the host folds deltaS and 1/zpl into it
// (geometry.cpp, ctgb_filter_build).
//
// GB300 layout: an in-house shared-memory radix-2 FFT, no cuFFT.  Because the
// spectrum is real, two real rows are filtered at once as the real and
// imaginary parts of one complex row (filtering a real row with a real,
// even-symmetric spectrum keeps it real, so the parts never mix).  One CTA per
// row pair: decimation-in-time forward FFT from bit-reversed loads, spectrum
// multiply, decimation-in-frequency inverse FFT, bit-reversed reads of the
// first nu outputs.  Twiddles come from a float64-built table.
#include <cuda_runtime.h>

#include "status.h"
#include "tma.cuh"

namespace ctgb {

struct FilterHeaderDev {
    int zpl, log2zpl, nu, nv;
    float R;
    int flip, pad[2];
    long long off_h, off_tw, off_kk, off_pp, total;
};

constexpr int kFftThreads = 256;

__device__ __forceinline__ unsigned bitrev(unsigned x, int bits) { return __brev(x) >> (32 - bits); }

// zpl_launch: the row length the launch's dynamic shared memory was sized
// for.  A table built for another length (or a malformed header) is refused:
// the CTA sets kDevErrArg in the device status word and returns before it
// touches shared memory or the rows.
__global__ void __launch_bounds__(kFftThreads)
fdk_filter_kernel(const float *__restrict__ F, float *__restrict__ proj, long long nrows, int zpl_launch,
                  int *status) {
    extern __shared__ float2 sm[];
    const FilterHeaderDev &f = *reinterpret_cast<const FilterHeaderDev *>(F);
    const int N = f.zpl, bits = f.log2zpl, nu = f.nu, nv = f.nv;
    if (N != zpl_launch || bits < 1 || bits > 13 || (1 << bits) != N || nu < 1 || nu > N || nv < 1) {
        if (threadIdx.x == 0 && status) atomicOr(status, kDevErrArg);
        return;
    }
    const float *__restrict__ H = F + f.off_h;
    const float2 *__restrict__ tw = reinterpret_cast<const float2 *>(F + f.off_tw);
    const float *__restrict__ kk = F + f.off_kk;
    const float *__restrict__ pp = F + f.off_pp;
    const float R = f.R;
    const long long ra = 2LL * blockIdx.x, rb = ra + 1;
    const bool has_b = rb < nrows;
    float *rowa = proj + ra * nu;
    float *rowb = proj + rb * nu;
    const float pa = pp[ra % nv], pb = has_b ? pp[rb % nv] : 0.0f;
    // Load weighted rows at bit-reversed positions (zero padding beyond nu).
    const int flip = f.flip;
    for (int n = threadIdx.x; n < N; n += blockDim.x) {
        float2 z = make_float2(0.0f, 0.0f);
        if (n < nu) {
            const float k2 = kk[n] * kk[n];
            const int src = flip ? nu - 1 - n : n;   // ConeBeamGPU.py:298 weights fliplr(proj)
            z.x = rowa[src] * (R * rsqrtf(R * R + k2 + pa * pa));
            if (has_b) z.y = rowb[src] * (R * rsqrtf(R * R + k2 + pb * pb));
        }
        sm[bitrev(n, bits)] = z;
    }
    __syncthreads();
    // Forward FFT, decimation in time: w = exp(-2 pi i j / (2 half)).
    for (int half = 1; half < N; half <<= 1) {
        const int step = N / (2 * half);
        for (int b = threadIdx.x; b < N / 2; b += blockDim.x) {
            const int j = b & (half - 1);
            const int i0 = (b - j) * 2 + j, i1 = i0 + half;
            const float2 w = tw[j * step];
            const float2 x1 = sm[i1], x0 = sm[i0];
            const float tr = x1.x * w.x + x1.y * w.y;     // x1 * conj(w_table) = x1 * exp(-i a)
            const float ti = x1.y * w.x - x1.x * w.y;
            sm[i1] = make_float2(x0.x - tr, x0.y - ti);
            sm[i0] = make_float2(x0.x + tr, x0.y + ti);
        }
        __syncthreads();
    }
    // Real spectrum (deltaS / N folded in).
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
        const float hk = H[k];
        float2 z = sm[k];
        sm[k] = make_float2(z.x * hk, z.y * hk);
    }
    __syncthreads();
    // Inverse FFT, decimation in frequency: w = exp(+2 pi i j / (2 half)).
    for (int half = N / 2; half >= 1; half >>= 1) {
        const int step = N / (2 * half);
        for (int b = threadIdx.x; b < N / 2; b += blockDim.x) {
            const int j = b & (half - 1);
            const int i0 = (b - j) * 2 + j, i1 = i0 + half;
            const float2 w = tw[j * step];
            const float2 x0 = sm[i0], x1 = sm[i1];
            const float dr = x0.x - x1.x, di = x0.y - x1.y;
            sm[i0] = make_float2(x0.x + x1.x, x0.y + x1.y);
            sm[i1] = make_float2(dr * w.x - di * w.y, dr * w.y + di * w.x);
        }
        __syncthreads();
    }
    for (int n = threadIdx.x; n < nu; n += blockDim.x) {
        const float2 z = sm[bitrev(n, bits)];
        rowa[n] = z.x;
        if (has_b) rowb[n] = z.y;
    }
}

}  // namespace ctgb

using namespace ctgb;

extern "C" int ctgb_fdk_filter(const ctgb_params *p, const void *d_filter, float *d_proj, int32_t nviews,
                               void *stream) {
    clear_error();
    if (!p || !d_filter || !d_proj || nviews < 0) return set_error(CTGB_ERR_ARG, "ctgb_fdk_filter: bad arguments");
    size_t need = 0;
    int st = ctgb_filter_bytes(p, &need);
    if (st) return st;
    if (nviews == 0) return CTGB_OK;
    // zpl as ctgb_filter_build computes it.
    int zpl = 1;
    while (zpl < 2 * (p->nu - 1)) zpl <<= 1;
    const long long nrows = (long long)nviews * p->nv;
    const long long nblocks = (nrows + 1) / 2;
    if (nblocks > 0x7fffffffLL) return set_error(CTGB_ERR_SIZE, "ctgb_fdk_filter: too many rows");
    const size_t smem = (size_t)zpl * sizeof(float2);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(fdk_filter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "fdk_filter smem: %s", cudaGetErrorString(e));
    }
    fdk_filter_kernel<<<(unsigned)nblocks, kFftThreads, smem, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const float *>(d_filter), d_proj, nrows, zpl, ctgb_status_ptr());
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "fdk_filter_kernel: %s", cudaGetErrorString(e));
    return CTGB_OK;
}

extern "C" int ctgb_filter_apply(const void *d_filter, int32_t zpl, float *d_rows, int64_t nrows, void *stream) {
    clear_error();
    if (!d_filter || !d_rows || nrows < 0 || zpl < 2 || zpl > 8192 || (zpl & (zpl - 1)))
        return set_error(CTGB_ERR_ARG, "ctgb_filter_apply: bad arguments");
    if (nrows == 0) return CTGB_OK;
    const long long nblocks = (nrows + 1) / 2;
    if (nblocks > 0x7fffffffLL) return set_error(CTGB_ERR_SIZE, "ctgb_filter_apply: too many rows");
    const size_t smem = (size_t)zpl * sizeof(float2);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(fdk_filter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "fdk_filter smem: %s", cudaGetErrorString(e));
    }
    fdk_filter_kernel<<<(unsigned)nblocks, kFftThreads, smem, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const float *>(d_filter), d_rows, nrows, zpl, ctgb_status_ptr());
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "fdk_filter_kernel: %s", cudaGetErrorString(e));
    return CTGB_OK;
}
