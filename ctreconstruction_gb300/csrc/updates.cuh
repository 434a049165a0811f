// The iterative drivers' element-wise lines, one device function each, shared
// by the stand-alone element-wise kernels (iterative.cu) and the projectors'
// fused epilogues (the forward projector's store of a residual, the
// backprojectors' store of an updated iterate).  The roundings are pinned
// with the _rn intrinsics (no contraction into fused multiply-adds), so a
// fused epilogue stores the same bits as the projector's plain store
// followed by the element-wise kernel.
//
//   SART      python/SART.py:51,55
//   MLEM      python/EM.py:36-42
//   POCS      python/ASD_POCS.py:174-179 (also each OS-SART sub-iteration)
#pragma once
#include <cuda_runtime.h>

namespace ctgb {

// Forward epilogues: what the forward projector stores for y = (A x)[i].
enum FwdEpiMode {
    kFwdStore = 0,      // y
    kFwdSartRes = 1,    // SART.py:51   (y - p0) / (A1 + eps)
    kFwdPocsRes = 2,    // ASD_POCS.py:174-175   (p0 - y) / (A1 + eps), 0 where A1 == 0
    kFwdEmRatio = 3,    // EM.py:36-39  p0 / y with p0 := 0 and y := eps where y == 0 (p0 written back)
};

// Backprojector epilogues: what the backprojector stores for b = (B r)[i].
enum BpEpiMode {
    kBpStore = 0,       // b (or vol + b with accumulate)
    kBpSartUpd = 1,     // SART.py:55   x = x - alpha * (b / n1 + eps)
    kBpEmUpd = 2,       // EM.py:41-42  x = x * (b / n1)
    kBpPocsUpd = 3,     // ASD_POCS.py:177-179   x = max(0, x + beta * b' / (n1 + eps)), b' = 0 where n1 == 0
};

__device__ __forceinline__ float sart_residual(float ax, float p0, float a1, float eps) {
    return __fdiv_rn(__fsub_rn(ax, p0), __fadd_rn(a1, eps));
}

__device__ __forceinline__ float pocs_residual(float p0, float ax, float a1, float eps) {
    return (a1 == 0.0f) ? 0.0f : __fdiv_rn(__fsub_rn(p0, ax), __fadd_rn(a1, eps));
}

// *p0 is the measured value, zeroed in place where ax == 0.
__device__ __forceinline__ float em_ratio(float *p0, float ax, float eps) {
    float p = *p0, a = ax;
    if (a == 0.0f) { p = 0.0f; *p0 = 0.0f; a = eps; }
    return __fdiv_rn(p, a);
}

__device__ __forceinline__ float sart_update(float xp, float b, float n1, float alpha, float eps) {
    return __fsub_rn(xp, __fmul_rn(alpha, __fadd_rn(__fdiv_rn(b, n1), eps)));
}

__device__ __forceinline__ float em_update(float xp, float b, float n1) {
    return __fmul_rn(xp, __fdiv_rn(b, n1));
}

__device__ __forceinline__ float pocs_update(float xp, float b, float n1, float beta, float eps) {
    const float bb = (n1 == 0.0f) ? 0.0f : b;
    const float v = __fadd_rn(xp, __fdiv_rn(__fmul_rn(beta, bb), __fadd_rn(n1, eps)));
    return v < 0.0f ? 0.0f : v;
}

// Forward epilogue parameters (by value in the kernel's parameters).
struct FwdEpi {
    int mode;
    float eps;
    float *p0;          // measured projections, same layout as the output (EM: zeroed in place)
    const float *a1;    // A 1 (SART, POCS)
};

__device__ __forceinline__ float fwd_epilogue(const FwdEpi &e, long long i, float y) {
    switch (e.mode) {
        case kFwdSartRes: return sart_residual(y, e.p0[i], e.a1[i], e.eps);
        case kFwdPocsRes: return pocs_residual(e.p0[i], y, e.a1[i], e.eps);
        case kFwdEmRatio: return em_ratio(e.p0 + i, y, e.eps);
        default: return y;
    }
}

// Backprojector epilogue parameters.
struct BpEpi {
    int mode;
    float coef;         // alpha (SART) or beta / lambda (POCS)
    float eps;
    float *x;           // iterate, updated in place
    const float *n1;    // backprojection normaliser
};

// Store of backprojected value b at volume index i of out (the plain store
// honours accumulate; the updates write the iterate instead).
__device__ __forceinline__ void bp_epilogue(const BpEpi &e, float *out, long long i, float b, int accumulate) {
    switch (e.mode) {
        case kBpSartUpd: e.x[i] = sart_update(e.x[i], b, e.n1[i], e.coef, e.eps); break;
        case kBpEmUpd: e.x[i] = em_update(e.x[i], b, e.n1[i]); break;
        case kBpPocsUpd: e.x[i] = pocs_update(e.x[i], b, e.n1[i], e.coef, e.eps); break;
        default: out[i] = accumulate ? __fadd_rn(out[i], b) : b;
    }
}

}  // namespace ctgb
