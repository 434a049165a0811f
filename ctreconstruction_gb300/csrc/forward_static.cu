// ctgb_forward_static: DD forward projection that allocates nothing.
//
// ctgb_forward reads x-dominant views from a [nz][nx][ny] copy of the volume
// that the caller allocates (d_vol_xzy).  Some callers cannot allocate device
// memory where they call the projector: an application that hands the whole
// device memory budget to its own pool and gives plugins no allocation
// rights, or a reconstruction loop on a latency budget where cudaMalloc's
// implicit device-wide synchronisation is not acceptable.  For them this entry
// point keeps that copy in a file-scope __device__ array of fixed size
// (CTGB_STATIC_MAX_VOXELS floats, 16 MiB), which every GPU that loads
// libctgb.so holds until the process exits.
//
// Set-up: the first call on each device (with that device current) looks up
// the array's device address with cudaGetSymbolAddress and caches it; make
// that first call before any stream capture.  Each call rewrites the whole
// copy before reading it, so nothing from an earlier call is used, but all
// calls share the one array: calls that overlap on the GPU (other streams,
// other host threads) race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <atomic>

#include "../../include/ctgb.h"
#include "status.h"

namespace ctgb {

static __device__ __align__(256) float g_forward_scratch[CTGB_STATIC_MAX_VOXELS];

// One cached address per device ordinal.  Concurrent first calls from
// several host threads may each look the address up; they store the same
// value, and the atomic makes the stores and loads well defined.
static float *scratch_ptr(int *err) {
    static std::atomic<float *> ptrs[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) {
        *err = set_error(CTGB_ERR_CUDA, "ctgb_forward_static: no current device (%s)", cudaGetErrorString(e));
        return nullptr;
    }
    float *cached = ptrs[dev].load(std::memory_order_acquire);
    if (!cached) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_forward_scratch);
        if (e != cudaSuccess || !p) {
            *err = set_error(CTGB_ERR_CUDA, "ctgb_forward_static: cudaGetSymbolAddress failed (%s)",
                             cudaGetErrorString(e));
            return nullptr;
        }
        cached = static_cast<float *>(p);
        ptrs[dev].store(cached, std::memory_order_release);
    }
    return cached;
}

}  // namespace ctgb

extern "C" int ctgb_forward_static(const ctgb_params *p, const void *d_table, const float *d_vol, float *d_proj,
                                   int32_t view0, int32_t nviews, void *stream) {
    ctgb::clear_error();
    if (!p) return ctgb::set_error(CTGB_ERR_ARG, "ctgb_forward_static: NULL argument");
    if (view0 < 0 || nviews < 0 || view0 + nviews > p->nviews)
        return ctgb::set_error(CTGB_ERR_ARG, "ctgb_forward_static: view range [%d,%d) outside [0,%d)", view0,
                               view0 + nviews, p->nviews);
    if (nviews == 0) return CTGB_OK;
    if (!d_table || !d_vol || !d_proj) return ctgb::set_error(CTGB_ERR_ARG, "ctgb_forward_static: NULL argument");
    if (p->nx < 1 || p->ny < 1 || p->nz < 1) return ctgb::set_error(CTGB_ERR_ARG, "ctgb_forward_static: bad volume size");
    const long long nvox = (long long)p->nx * p->ny * p->nz;
    if (nvox > (long long)CTGB_STATIC_MAX_VOXELS)
        return ctgb::set_error(CTGB_ERR_SIZE,
                               "ctgb_forward_static: volume of %lld voxels exceeds the static scratch of %d voxels "
                               "(use ctgb_forward with a caller-allocated copy)",
                               nvox, (int)CTGB_STATIC_MAX_VOXELS);
    int err = CTGB_OK;
    float *xzy = ctgb::scratch_ptr(&err);
    if (!xzy) return err;
    int st = ctgb_transpose_xy(d_vol, xzy, p->nx, p->ny, p->nz, stream);
    if (st != CTGB_OK) return st;
    return ctgb_forward(p, d_table, d_vol, xzy, d_proj, view0, nviews, stream);
}
