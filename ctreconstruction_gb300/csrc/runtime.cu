// Runtime helpers: the device status word, TMA descriptor construction.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <atomic>

#include "status.h"
#include "tma.cuh"

namespace ctgb {
__device__ int g_device_status = 0;
}

// One cached address per device ordinal (atomic: several host threads may
// make their first call on a device at once; all store the same value).
int *ctgb_status_ptr() {
    static std::atomic<int *> ptrs[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    int *cached = ptrs[dev].load(std::memory_order_acquire);
    if (!cached) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, ctgb::g_device_status) != cudaSuccess) return nullptr;
        cached = static_cast<int *>(p);
        ptrs[dev].store(cached, std::memory_order_release);
    }
    return cached;
}

// The driver's tensor-map encoder, looked up once (a function-local static
// is initialised exactly once even when several threads arrive together).
static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() -> PFN_cuTensorMapEncodeTiled_v12000 {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        return nullptr;
    }();
    return fn;
}

bool ctgb_make_tmap_3d(CUtensorMap *map, const float *base, const uint64_t dims[3], const uint32_t box[3]) {
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
    if (!fn) return false;
    cuuint64_t gdim[3] = {dims[0], dims[1], dims[2]};
    cuuint64_t gstride[2] = {dims[0] * 4, dims[0] * dims[1] * 4};
    cuuint32_t bdim[3] = {box[0], box[1], box[2]};
    cuuint32_t estride[3] = {1, 1, 1};
    if ((gstride[0] % 16) || (gstride[1] % 16) || (reinterpret_cast<uintptr_t>(base) % 16)) return false;
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), gdim, gstride, bdim, estride,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

bool ctgb_make_tmap_bf16(CUtensorMap *map, const void *base, int rank, const uint64_t *dims, const uint32_t *box) {
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
    if (!fn || rank < 1 || rank > 5) return false;
    cuuint64_t gdim[5], gstride[4];
    cuuint32_t bdim[5], estride[5];
    uint64_t stride = 2;
    for (int i = 0; i < rank; ++i) {
        gdim[i] = dims[i];
        bdim[i] = box[i];
        estride[i] = 1;
        if (i > 0) gstride[i - 1] = stride;
        stride *= dims[i];
    }
    for (int i = 0; i + 1 < rank; ++i)
        if (gstride[i] % 16) return false;
    if (reinterpret_cast<uintptr_t>(base) % 16) return false;
    const uint32_t inner = box[0] * 2;
    CUtensorMapSwizzle sw;
    if (inner == 16) sw = CU_TENSOR_MAP_SWIZZLE_NONE;
    else if (inner == 32) sw = CU_TENSOR_MAP_SWIZZLE_32B;
    else if (inner == 64) sw = CU_TENSOR_MAP_SWIZZLE_64B;
    else if (inner == 128) sw = CU_TENSOR_MAP_SWIZZLE_128B;
    else return false;
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, (cuuint32_t)rank, const_cast<void *>(base), gdim, gstride,
                    bdim, estride, CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

// Self-test of the bounded device waits: one warp initialises an mbarrier
// that expects one arrival, never arrives, and waits on it with a limit of
// `polls` polls; the wait runs out, records kDevErrTimeout in the status word
// and the kernel returns.  No copy is in flight and nothing else waits.
__global__ void bounded_wait_selftest_kernel(long long polls, int *status) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        ctgb::mbar_init(&bar, 1);
        ctgb::fence_mbar_init();
    }
    __syncwarp();
    ctgb::mbar_wait(&bar, 0, status, polls);
}

extern "C" int ctgb_selftest_bounded_wait(int32_t polls, void *stream) {
    ctgb::clear_error();
    if (polls < 1 || polls > (1 << 20))
        return ctgb::set_error(CTGB_ERR_ARG, "ctgb_selftest_bounded_wait: polls %d outside [1, 2^20]", polls);
    int *status = ctgb_status_ptr();
    if (!status) return ctgb::set_error(CTGB_ERR_CUDA, "ctgb_selftest_bounded_wait: device status word unavailable");
    bounded_wait_selftest_kernel<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(polls, status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return ctgb::set_error(CTGB_ERR_CUDA, "bounded_wait_selftest_kernel: %s", cudaGetErrorString(e));
    return CTGB_OK;
}

// Reads (and optionally clears) the device status word of the current device.
// Synchronises the device.  *out = 0 when no kernel reported a problem.
extern "C" int ctgb_device_status(int32_t *out, int32_t clear) {
    ctgb::clear_error();
    if (!out) return ctgb::set_error(CTGB_ERR_ARG, "ctgb_device_status: out is NULL");
    int v = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, ctgb::g_device_status, sizeof(int));
    if (e != cudaSuccess) return ctgb::set_error(CTGB_ERR_CUDA, "ctgb_device_status: %s", cudaGetErrorString(e));
    if (clear && v) {
        int z = 0;
        e = cudaMemcpyToSymbol(ctgb::g_device_status, &z, sizeof(int));
        if (e != cudaSuccess) return ctgb::set_error(CTGB_ERR_CUDA, "ctgb_device_status: %s", cudaGetErrorString(e));
    }
    *out = v;
    return CTGB_OK;
}
