// 5th-generation tensor core (tcgen05) and TMEM helpers for sm_100-family
// GPUs, inline PTX.  Single-CTA forms (cta_group::1) only.
//
// Shared-memory matrix descriptor (64-bit) of a K-major operand tile stored
// in the canonical swizzled layout that a TMA load with the same swizzle
// writes: rows of S bytes (S = 32, 64 or 128, the swizzle span), 8-row
// groups SBO = 8*S bytes apart.  Fields: start address >> 4 (bits 0-13),
// leading-dimension byte offset >> 4 (16-29, unused for these layouts),
// stride-dimension byte offset >> 4 (32-45), descriptor version 1 (46-47),
// base offset (49-51, 0: tiles are aligned to the swizzle repeat), layout
// type (61-63: 2 = 128-byte, 4 = 64-byte, 6 = 32-byte swizzle).
//
// Instruction descriptor of kind::f16 (32-bit): D format f32 (bits 4-5 = 1),
// A and B format bf16 (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 =
// 0), N >> 3 (bits 17-22), M >> 4 (bits 24-28).
#pragma once
#include <stdint.h>

#include "tma.cuh"

namespace ctgb {

__device__ __forceinline__ uint32_t umma_layout_for_row_bytes(uint32_t row_bytes) {
    return row_bytes == 128 ? 2u : (row_bytes == 64 ? 4u : 6u);
}

__device__ __forceinline__ uint64_t umma_smem_desc(uint32_t saddr, uint32_t row_bytes) {
    const uint64_t sbo = (8u * row_bytes) >> 4;
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1u << 16;
    d |= (sbo & 0x3FFFu) << 32;
    d |= (uint64_t)1u << 46;
    d |= (uint64_t)umma_layout_for_row_bytes(row_bytes) << 61;
    return d;
}

// The same descriptor with its start address moved by delta16 * 16 bytes.
// The start field is the low 14 bits and shared memory is below 256 KB, so
// the addition never carries out of the field: a 32-bit add on the low word.
__device__ __forceinline__ uint64_t desc_advance(uint64_t d, uint32_t delta16) {
    return (d & 0xFFFFFFFF00000000ull) | (uint64_t)((uint32_t)d + delta16);
}

// Descriptor of a K-major operand in the unswizzled (interleaved) layout:
// 8 x 16-byte core matrices whose 8 rows are 16 bytes apart, core matrices
// adjacent in K `lbo` bytes apart and 8-row groups `sbo` bytes apart; the
// start address only needs 16-byte alignment, so a tile may begin at any row.
__device__ __forceinline__ uint64_t umma_smem_desc_interleaved(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1u << 46;
    return d;                                   // layout type 0: no swizzle
}

__host__ __device__ constexpr uint32_t umma_idesc_bf16_f32(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void tmem_alloc(uint32_t *smem_slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(smem_slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, one instruction, issued by one thread.
__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrive on an mbarrier once every tcgen05 operation this thread issued so
// far has completed.
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_addr(bar))
                 : "memory");
}

// 32 lanes x 16 consecutive 32-bit columns: thread t of the warp gets lane
// (base lane + t), columns col .. col+15.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
        "%14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tma_load_5d(void *dst, const CUtensorMap *tmap, int c0, int c1, int c2, int c3,
                                            int c4, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(tmap)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *tmap, int c0, int c1, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(tmap)), "r"(c0), "r"(c1), "r"(smem_addr(bar))
        : "memory");
}

}  // namespace ctgb
