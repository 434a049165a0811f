// Packed two-lane float32 arithmetic (PTX add/sub/mul/fma .f32x2, sm_100+).
// Each lane rounds exactly as the scalar instruction with the same rounding
// mode would, so packed and scalar code give the same bits.  A pair lives in
// one 64-bit register pair: lane x in the low half, lane y in the high half,
// the same order as a float2 loaded with one 8-byte load.
#pragma once
#include <cstdint>

namespace ctgb {

typedef unsigned long long f2x;

__device__ __forceinline__ f2x f2_pack(float x, float y) {
    f2x r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(x), "f"(y));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2x r, float &x, float &y) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(x), "=f"(y) : "l"(r));
}
__device__ __forceinline__ f2x f2_fma(f2x a, f2x b, f2x c) {
    f2x d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ f2x f2_mul(f2x a, f2x b) {
    f2x d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2x f2_add_rd(f2x a, f2x b) {
    f2x d;
    asm("add.rm.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2x f2_sub(f2x a, f2x b) {
    f2x d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
// 8-byte read-only load of a float2 straight into a pair.
__device__ __forceinline__ f2x f2_ldg(const float2 *p) {
    f2x r;
    asm("ld.global.nc.b64 %0, [%1];" : "=l"(r) : "l"(p));
    return r;
}

}  // namespace ctgb
