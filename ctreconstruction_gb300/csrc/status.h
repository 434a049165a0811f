// Per-thread last-error state behind ctgb_last_error(), and the per-device
// kernel attribute helper the launchers share.
#pragma once
#include <cuda_runtime.h>

#include <atomic>

#include "../../include/ctgb.h"

namespace ctgb {
int set_error(int status, const char *fmt, ...);   // records the message, returns status
void clear_error();
int last_status();

// Raises `kernel`'s dynamic shared-memory limit to `bytes` on the current
// device, once per device: the attribute belongs to the device's copy of the
// kernel, so a process that drives several GPUs sets it on each (one bit
// per device ordinal in `done`).
inline cudaError_t smem_limit_once(const void *kernel, int bytes, std::atomic<unsigned long long> &done) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = 1ull << (dev & 63);
    if (done.load(std::memory_order_acquire) & bit) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) done.fetch_or(bit, std::memory_order_acq_rel);
    return e;
}
}  // namespace ctgb
