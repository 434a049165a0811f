// TMA (cp.async.bulk.tensor) and mbarrier helpers for sm_103a, inline PTX.
//
// Every wait on an mbarrier is bounded: after kWaitLimit polls the waiting
// thread records kDevErrTimeout in the device status word and reports
// failure, and the kernel returns instead of hanging the GPU.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace ctgb {

// Status bits (CTGB_DEVERR_* in include/ctgb.h).
constexpr int kDevErrTimeout = 1;
constexpr int kDevErrArg = 2;       // a kernel refused a malformed device-side table

constexpr long long kWaitLimit = 1LL << 26;   // ~ seconds of polling

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// Bounded wait for the phase with the given parity; false on timeout (and
// kDevErrTimeout is or-ed into *status, the library's device status word).
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *status,
                                          long long limit = kWaitLimit) {
    const uint32_t a = smem_addr(bar);
    for (long long i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    atomicOr(status, kDevErrTimeout);
    return false;
}

// 3-D tiled TMA load of one box into shared memory, completing on `bar`.
// c0 (innermost coordinate) must be a multiple of 4 for float32 data.
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *tmap, int c0, int c1, int c2,
                                            uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(tmap)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(bar))
        : "memory");
}

// floor(x) for |x| < 2^22 as (int, float) via a round-down add of 1.5*2^23.
__device__ __forceinline__ int floor_split(float x, float *f) {
    const float t = __fadd_rd(x, 12582912.0f);
    *f = t - 12582912.0f;
    return __float_as_int(t) - 0x4B400000;
}

}  // namespace ctgb

// Host: build a 3-D float32 tiled tensor map (dims/box innermost first).
// Returns false if the driver rejects the description (e.g. unaligned strides).
bool ctgb_make_tmap_3d(CUtensorMap *map, const float *base, const uint64_t dims[3], const uint32_t box[3]);

// Host: a bf16 tiled tensor map of `rank` dims (innermost first, dense
// strides), with the shared-memory swizzle whose span equals the box's inner
// extent in bytes (32, 64 or 128; a 16-byte inner extent is unswizzled).
// Out-of-bounds elements load as zeros.
bool ctgb_make_tmap_bf16(CUtensorMap *map, const void *base, int rank, const uint64_t *dims, const uint32_t *box);

// Host: device address of the library's status word on the current device
// (a file-scope __device__ int in runtime.cu; looked up once per device).
int *ctgb_status_ptr();
