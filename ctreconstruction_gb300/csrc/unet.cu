// Learned proximal step: the building blocks of a small 3-D U-Net (no
// reference counterpart; it stands in for ASD-POCS's TV descent,
// python/ASD_POCS.py:186-190).
//
// Activations are bf16 in [N][D][H][W][C] order (channels innermost, C in
// {16, 32, 64}); weights of a 3x3x3 convolution are [27 taps][Cout][Cin]
// (tap = (dz+1)*9 + (dy+1)*3 + (dx+1)); accumulation is fp32.
//
// conv3d_tc_kernel is an implicit GEMM on the 5th-generation tensor cores:
// one CTA computes a tile of M = 128 output voxels x Cout channels.  The K
// loop runs over the 27 taps (x the input segments of a channel concat):
// per step TMA brings the 128 shifted input voxels (a box {C, Wb, R, 1, 1} of
// the 5-D activation tensor; zero fill outside the volume is the conv's zero
// padding) and the tap's [Cout][C] weight block into a ring of 3-8
// shared-memory stages (sized for the layer's widest segment), in the swizzled K-major layout tcgen05 reads; one
// thread issues tcgen05.mma (M = 128, N = Cout, K = 16 per instruction)
// into a TMEM accumulator, and tcgen05.commit releases each stage.  The
// epilogue reads TMEM with tcgen05.ld (one row per thread), adds the bias,
// applies ReLU and stores bf16 — or stores the raw fp32 sums (the data
// gradient, which runs the same kernel on flipped weights).
//
// The remaining passes (input packing, pooling, upsampling, masks, the 1x1
// head, the weight gradient) are CUDA-core kernels.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/ctgb.h"
#include "status.h"
#include "tcgen05.cuh"
#include "tma.cuh"

namespace ctgb {

constexpr int kCvM = 128, kCvThreads = 128;

// Stage buffers sized for the widest input segment (CMAX channels), so that
// narrow layers keep more stages (and more CTAs per SM) in flight.
template <int COUT, int CMAX>
struct ConvCfg {
    static constexpr int kABytes = kCvM * CMAX * 2;                          // 128 rows of CMAX bf16
    static constexpr int kBBytes = ((COUT * CMAX * 2 + 1023) / 1024) * 1024;  // COUT rows of CMAX bf16
    static constexpr int kStage = kABytes + kBBytes;
    static constexpr int kStages = (65536 / kStage) < 3 ? 3 : ((65536 / kStage) > 8 ? 8 : 65536 / kStage);
    static constexpr int kTmemCols = COUT <= 32 ? 32 : (COUT <= 64 ? 64 : 128);
    static constexpr int kSmem = kStages * kStage + 1024 + 256;
};

struct ConvGeom {
    int N, D, H, W, Wb, R, c0, c1, nseg;
};

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t *>(&v);
}

// EPI 0: out bf16 = relu(acc + bias); EPI 1: out fp32 = acc.
template <int COUT, int CMAX, int EPI>
__global__ void __launch_bounds__(kCvThreads, 1)
conv3d_tc_kernel(const __grid_constant__ CUtensorMap ta0, const __grid_constant__ CUtensorMap ta1,
                 const __grid_constant__ CUtensorMap tb0, const __grid_constant__ CUtensorMap tb1, const ConvGeom g,
                 const float *__restrict__ bias, void *__restrict__ out, int *status) {
    using Cfg = ConvCfg<COUT, CMAX>;
    extern __shared__ uint8_t smraw[];
    const uint32_t raw = smem_addr(smraw);
    uint8_t *base = smraw + (((raw + 1023u) & ~1023u) - raw);
    uint64_t *full = reinterpret_cast<uint64_t *>(base + Cfg::kStages * Cfg::kStage);
    uint64_t *empty = full + Cfg::kStages;
    uint64_t *done = empty + Cfg::kStages;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(done + 1);
    volatile int *failed = reinterpret_cast<volatile int *>(tslot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tiles_x = g.W / g.Wb, tiles_h = g.H / g.R;
    int t = blockIdx.x;
    const int tx = t % tiles_x;
    t /= tiles_x;
    const int th = t % tiles_h;
    t /= tiles_h;
    const int d = t % g.D, n = t / g.D;
    const int x0 = tx * g.Wb, h0 = th * g.R;

    if (threadIdx.x == 0) {
        for (int s = 0; s < Cfg::kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        *failed = 0;
        fence_mbar_init();
    }
    if (warp == 0) tmem_alloc(tslot, Cfg::kTmemCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const int nsteps = 27 * g.nseg;

    if (warp == 0 && lane == 0) {
        // TMA producer.
        for (int i = 0; i < nsteps; ++i) {
            const int s = i % Cfg::kStages;
            if (i >= Cfg::kStages && !mbar_wait(&empty[s], ((i / Cfg::kStages) - 1) & 1, status)) {
                *failed = 1;
                break;
            }
            const int tap = i / g.nseg, seg = i - tap * g.nseg;
            const int c = seg ? g.c1 : g.c0;
            uint8_t *A = base + s * Cfg::kStage;
            uint8_t *B = A + Cfg::kABytes;
            mbar_arrive_expect_tx(&full[s], (uint32_t)((kCvM + COUT) * c * 2));
            const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
            tma_load_5d(A, seg ? &ta1 : &ta0, 0, x0 + dx, h0 + dy, d + dz, n, &full[s]);
            tma_load_2d(B, seg ? &tb1 : &tb0, 0, tap * COUT, &full[s]);
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer.
        constexpr uint32_t idesc = umma_idesc_bf16_f32(kCvM, COUT);
        for (int i = 0; i < nsteps; ++i) {
            const int s = i % Cfg::kStages;
            if (!mbar_wait(&full[s], (i / Cfg::kStages) & 1, status)) {
                *failed = 1;
                break;
            }
            tc_fence_after();
            const int seg = i % g.nseg;
            const uint32_t rb = (uint32_t)(seg ? g.c1 : g.c0) * 2u;
            const uint32_t a_addr = smem_addr(base + s * Cfg::kStage), b_addr = a_addr + Cfg::kABytes;
            for (uint32_t k = 0; k < rb / 32u; ++k)
                umma_bf16(tmem, umma_smem_desc(a_addr + 32u * k, rb), umma_smem_desc(b_addr + 32u * k, rb), idesc,
                          (i > 0 || k > 0) ? 1u : 0u);
            umma_commit(&empty[s]);
        }
        umma_commit(done);
    }
    __syncwarp();

    // Epilogue: thread (warp w, lane l) owns tile row 32 w + l.
    const bool got = mbar_wait(done, 0, status);
    tc_fence_after();
    const bool go = __all_sync(0xffffffffu, got && !*failed);
    if (go) {
        const int row = warp * 32 + lane;
        const int hh = h0 + row / g.Wb, xx = x0 + row % g.Wb;
        const long long vox = (((long long)n * g.D + d) * g.H + hh) * g.W + xx;
#pragma unroll
        for (int cb = 0; cb < COUT; cb += 16) {
            float v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cb, v);
            if (EPI == 0) {
                uint32_t p[8];
#pragma unroll
                for (int i = 0; i < 8; ++i)
                    p[i] = pack_bf16x2(fmaxf(v[2 * i] + bias[cb + 2 * i], 0.0f),
                                       fmaxf(v[2 * i + 1] + bias[cb + 2 * i + 1], 0.0f));
                uint4 *o = reinterpret_cast<uint4 *>(static_cast<__nv_bfloat16 *>(out) + vox * COUT + cb);
                o[0] = make_uint4(p[0], p[1], p[2], p[3]);
                o[1] = make_uint4(p[4], p[5], p[6], p[7]);
            } else {
                float4 *o = reinterpret_cast<float4 *>(static_cast<float *>(out) + vox * COUT + cb);
#pragma unroll
                for (int i = 0; i < 4; ++i) o[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, Cfg::kTmemCols);
    }
}

// ---- tap reuse for rows of 128 voxels ------------------------------------------
//
// When W is a multiple of 128 a tile is R runs of 128 voxels along x, in R
// consecutive rows y0 .. y0 + R - 1 (R = 1 or 2 by the layer's channel
// counts; rows past H are computed from zero fill and not stored).  For one
// dz plane, the 9 R (row, dy, dx) products read R + 2 input rows
// (y0 - 1 .. y0 + R), each shifted by one voxel per dx.
// conv3d_tc_dx_kernel loads those rows once per dz and segment — one TMA box
// of (R + 2) x 130 whole voxels (x0 - 1 .. x0 + 128, C channels, 2C-byte
// rows) in the swizzled K-major layout whose span is the row (32/64/128 B) —
// and starts the A operand of output row r, tap (dy, dx) at voxel row
// (r + dy) * 130 + dx of it.  The swizzle is a function of the shared-memory
// address bits (the box starts 1024-byte aligned), so a descriptor may start
// at any row: no copy per tap.  Each output row has its own TMEM
// accumulator; R rows need (R + 2) / (3 R) of the input rows that one row
// per tile would load.  When the layer's weights fit (<= 16 KB) they are
// loaded once per CTA and stay in shared memory; otherwise each stage also
// carries its nine weight blocks.
//
// The kernel is persistent and warp-specialised: warp 0 issues the TMA loads
// of tile after tile into a ring of stages, warp 1 issues the MMAs into one
// of two TMEM accumulators, and warps 2-5 drain the other accumulator
// (tcgen05.ld, bias/ReLU, stores), so a tile's epilogue overlaps the next
// tile's loads and MMAs.
// Sizes of the tap-reuse kernel for (Cout, widest input segment, resident
// weights), shared by the kernel's template and the host's routing.
struct DxSizes {
    int rows;        // output rows per tile (R)
    int abytes;      // input bytes of one stage: R + 2 rows of 130 voxels
    int btap;        // one tap's weight block
    int stage;       // bytes of one stage (input, and nine weight blocks unless resident)
    int stages;
    int acc_cols;    // TMEM columns of one output row's accumulator
    int tmem_cols;   // two tiles' accumulators
    int fixed;       // dynamic shared memory besides the resident weights
};
// Occupancy decides this kernel's speed: each CTA has one MMA-issuing
// thread, and the Cout = 16 layers ran fastest with four CTAs per SM.  At
// 256^3 (one U-Net forward): resident weights only up to 16 KB, two output
// rows per tile for 16- and 32-channel inputs and a 48 KB stage ring gave
// 6.26 ms; four rows, 64 KB resident weights and a 96 KB ring 7.27 ms (one
// or two CTAs per SM); one row per tile 6.8-6.9 ms; no resident weights
// 7.61 ms.
#ifndef CTGB_DX_WMAX
#define CTGB_DX_WMAX 16384
#endif
#ifndef CTGB_DX_R32
#define CTGB_DX_R32 2
#endif
#ifndef CTGB_DX_R16
#define CTGB_DX_R16 2
#endif
constexpr int kDxWMax = CTGB_DX_WMAX;       // resident weights, at most
#ifndef CTGB_DX_BUDGET
#define CTGB_DX_BUDGET 49152
#endif
constexpr int kDxBudget = CTGB_DX_BUDGET;   // stage ring target
constexpr int kDxThreads = 192;             // producer warp, MMA warp, 4 epilogue warps
constexpr int kDxSmemLimit = 227 * 1024;

__host__ __device__ constexpr DxSizes dx_sizes(int cout, int cmax, bool res) {
    const int rows = cmax == 64 ? (cout <= 64 ? 2 : 1) : (cout <= 64 ? (cmax == 32 ? CTGB_DX_R32 : CTGB_DX_R16) : 2);
    const int abytes = (((rows + 2) * (kCvM + 2) * cmax * 2 + 1023) / 1024) * 1024;
    const int btap = cout * cmax * 2;
    const int stage = abytes + (res ? 0 : ((9 * btap + 1023) / 1024) * 1024);
    const int fit = kDxBudget / stage;
    const int stages = fit < 2 ? 2 : (fit > 6 ? 6 : fit);
    const int acc = cout <= 32 ? 32 : (cout <= 64 ? 64 : 128);
    return DxSizes{rows, abytes, btap, stage, stages, acc, 2 * rows * acc, stages * stage + 256 + 1024};
}

template <int COUT, int CMAX, bool RES>
struct ConvDxCfg {
    static constexpr DxSizes kS = dx_sizes(COUT, CMAX, RES);
    static constexpr int kR = kS.rows;
    static constexpr int kABytes = kS.abytes;
    static constexpr int kBTap = kS.btap;
    static constexpr int kStage = kS.stage;
    static constexpr int kStages = kS.stages;
    static constexpr int kAccCols = kS.acc_cols;
    static constexpr int kTmemCols = kS.tmem_cols;
    static constexpr int kWMax = kDxWMax;
    static constexpr int kSmemFixed = kS.fixed;
    static_assert(kTmemCols <= 512, "conv3d_tc_dx_kernel: accumulators above the TMEM of one SM");
};

// Host: whether the tap-reuse kernel fits for this shape (resident weights
// when they fit kDxWMax, as launch_conv_dx decides), and its rows per tile.
static bool dx_fits(int cout, int cmax, int nseg, int *rows) {
    const bool res = nseg * 27 * cout * cmax * 2 <= kDxWMax;
    const DxSizes z = dx_sizes(cout, cmax, res);
    *rows = z.rows;
    return (res ? kDxWMax : 0) + z.fixed <= kDxSmemLimit;
}

template <int COUT, int CMAX, int EPI, bool RES>
__global__ void __launch_bounds__(kDxThreads, 1)
conv3d_tc_dx_kernel(const __grid_constant__ CUtensorMap ta0, const __grid_constant__ CUtensorMap ta1,
                    const __grid_constant__ CUtensorMap tb0, const __grid_constant__ CUtensorMap tb1,
                    const ConvGeom g, int wres, const float *__restrict__ bias, void *__restrict__ out,
                    int *status) {
    using Cfg = ConvDxCfg<COUT, CMAX, RES>;
    extern __shared__ uint8_t smraw[];
    const uint32_t raw = smem_addr(smraw);
    uint8_t *wbase = smraw + (((raw + 1023u) & ~1023u) - raw);     // resident weights (wres bytes)
    uint8_t *base = wbase + wres;                                   // stage ring
    uint64_t *full = reinterpret_cast<uint64_t *>(base + Cfg::kStages * Cfg::kStage);
    uint64_t *empty = full + Cfg::kStages;
    uint64_t *acc_full = empty + Cfg::kStages;     // [2]: MMAs of a tile done
    uint64_t *acc_empty = acc_full + 2;            // [2]: epilogue has read the accumulator
    uint64_t *wbar = acc_empty + 2;                // resident weights landed
    uint32_t *tslot = reinterpret_cast<uint32_t *>(wbar + 1);
    volatile int *failed = reinterpret_cast<volatile int *>(tslot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int R = Cfg::kR;
    const int tiles_x = g.W / kCvM, tiles_y = (g.H + R - 1) / R;
    const int ntiles = g.N * g.D * tiles_y * tiles_x;

    if (threadIdx.x == 0) {
        for (int s = 0; s < Cfg::kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], 128);
        }
        mbar_init(wbar, 1);
        *failed = 0;
        fence_mbar_init();
    }
    if (warp == 0) tmem_alloc(tslot, Cfg::kTmemCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    const int steps_per_tile = 3 * g.nseg;

    if (warp == 0) {
        if (lane == 0) {
            if (RES) {
                uint32_t bytes = 0;
                for (int seg = 0; seg < g.nseg; ++seg) bytes += 27u * COUT * (uint32_t)(seg ? g.c1 : g.c0) * 2u;
                mbar_arrive_expect_tx(wbar, bytes);
                for (int seg = 0; seg < g.nseg; ++seg)
                    for (int tap = 0; tap < 27; ++tap)
                        tma_load_2d(wbase + (seg * 27 + tap) * Cfg::kBTap, seg ? &tb1 : &tb0, 0, tap * COUT, wbar);
            }
            // TMA producer: every tile's dz x segment steps, back to back.
            int i = 0;
            for (int tile = blockIdx.x; tile < ntiles && !*failed; tile += gridDim.x) {
                int t = tile;
                const int x0 = (t % tiles_x) * kCvM;
                t /= tiles_x;
                const int y0 = (t % tiles_y) * R;
                t /= tiles_y;
                const int d = t % g.D, n = t / g.D;
                for (int k = 0; k < steps_per_tile; ++k, ++i) {
                    const int s = i % Cfg::kStages;
                    if (i >= Cfg::kStages && !mbar_wait(&empty[s], ((i / Cfg::kStages) - 1) & 1, status)) {
                        *failed = 1;
                        break;
                    }
                    const int dzi = k / g.nseg, seg = k - dzi * g.nseg;
                    const int c = seg ? g.c1 : g.c0;
                    uint8_t *A = base + s * Cfg::kStage;
                    uint8_t *B = A + Cfg::kABytes;
                    mbar_arrive_expect_tx(&full[s], (uint32_t)((R + 2) * (kCvM + 2) * c * 2 +
                                                               (RES ? 0 : 9 * COUT * c * 2)));
                    tma_load_5d(A, seg ? &ta1 : &ta0, 0, x0 - 1, y0 - 1, d + dzi - 1, n, &full[s]);
                    if (!RES)
                        for (int q = 0; q < 9; ++q)
                            tma_load_2d(B + q * Cfg::kBTap, seg ? &tb1 : &tb0, 0, (dzi * 9 + q) * COUT, &full[s]);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer: accumulator j & 1 for the CTA's j-th tile.
            constexpr uint32_t idesc = umma_idesc_bf16_f32(kCvM, COUT);
            bool ok = !RES || mbar_wait(wbar, 0, status);
            const uint32_t w_addr = smem_addr(wbase);
            int i = 0, j = 0;
            for (int tile = blockIdx.x; ok && tile < ntiles && !*failed; tile += gridDim.x, ++j) {
                const int b = j & 1, u = j >> 1;
                if (u > 0 && !mbar_wait(&acc_empty[b], (u - 1) & 1, status)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t dacc = tmem + (uint32_t)(b * R * Cfg::kAccCols);
                for (int k = 0; k < steps_per_tile; ++k, ++i) {
                    const int s = i % Cfg::kStages;
                    if (!mbar_wait(&full[s], (i / Cfg::kStages) & 1, status)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const int dzi = k / g.nseg, seg = k - dzi * g.nseg;
                    const uint32_t c = (uint32_t)(seg ? g.c1 : g.c0), rowb = c * 2u, nk = c / 16u;
                    const uint32_t a_addr = smem_addr(base + s * Cfg::kStage), b_addr = a_addr + Cfg::kABytes;
                    // Base descriptors of the stage's input rows and of its (or
                    // the resident) weight blocks; every product's descriptor is
                    // one of these plus a start offset in 16-byte units.
                    const uint64_t a0 = umma_smem_desc(a_addr, rowb);
                    const uint64_t b0 =
                        umma_smem_desc(RES ? w_addr + (uint32_t)(seg * 27 + dzi * 9) * Cfg::kBTap : b_addr, rowb);
                    const uint32_t row16 = (uint32_t)(kCvM + 2) * (rowb >> 4), vox16 = rowb >> 4;
#pragma unroll
                    for (uint32_t q = 0; q < 9; ++q) {
                        const uint32_t dy = q / 3u, dx = q % 3u;
                        for (uint32_t kk = 0; kk < nk; ++kk) {
                            const uint64_t bd = desc_advance(b0, (q * (uint32_t)Cfg::kBTap >> 4) + 2u * kk);
                            const uint64_t ab = desc_advance(a0, dy * row16 + dx * vox16 + 2u * kk);
                            const uint32_t accum = (k > 0 || q > 0 || kk > 0) ? 1u : 0u;
#pragma unroll
                            for (uint32_t r = 0; r < (uint32_t)R; ++r)
                                umma_bf16(dacc + r * (uint32_t)Cfg::kAccCols, desc_advance(ab, r * row16), bd, idesc,
                                          accum);
                        }
                    }
                    umma_commit(&empty[s]);
                }
                if (!ok) break;
                umma_commit(&acc_full[b]);
            }
            if (!ok) *failed = 1;
        }
    } else {
        // Epilogue warps 2-5: warp w reads TMEM lanes 32 (w % 4) .. +31.
        const int quarter = warp & 3;
        const int row = quarter * 32 + lane;
        int j = 0;
        for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++j) {
            const int b = j & 1, u = j >> 1;
            const bool got = mbar_wait(&acc_full[b], u & 1, status);
            tc_fence_after();
            if (!__all_sync(0xffffffffu, got && !*failed)) break;
            int t = tile;
            const int x0 = (t % tiles_x) * kCvM;
            t /= tiles_x;
            const int y0 = (t % tiles_y) * R;
            t /= tiles_y;
            const int d = t % g.D, n = t / g.D;
            const int rows = g.H - y0 < R ? g.H - y0 : R;        // rows of this tile inside the volume
            for (int r = 0; r < rows; ++r) {
            const long long vox = (((long long)n * g.D + d) * g.H + y0 + r) * g.W + x0 + row;
            const uint32_t tbase = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)((b * R + r) * Cfg::kAccCols);
#pragma unroll
            for (int cb = 0; cb < COUT; cb += 16) {
                float v[16];
                tmem_ld16(tbase + (uint32_t)cb, v);
                if (EPI == 0) {
                    uint32_t p[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q)
                        p[q] = pack_bf16x2(fmaxf(v[2 * q] + bias[cb + 2 * q], 0.0f),
                                           fmaxf(v[2 * q + 1] + bias[cb + 2 * q + 1], 0.0f));
                    uint4 *o = reinterpret_cast<uint4 *>(static_cast<__nv_bfloat16 *>(out) + vox * COUT + cb);
                    o[0] = make_uint4(p[0], p[1], p[2], p[3]);
                    o[1] = make_uint4(p[4], p[5], p[6], p[7]);
                } else {
                    float4 *o = reinterpret_cast<float4 *>(static_cast<float *>(out) + vox * COUT + cb);
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                }
            }
            }
            tc_fence_before();
            mbar_arrive(&acc_empty[b]);
        }
    }
    __syncwarp();
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        if (RES && lane == 0 && *failed) mbar_wait(wbar, 0, status);   // resident weight copies have landed
        __syncwarp();
        tc_fence_after();
        tmem_dealloc(tmem, Cfg::kTmemCols);
    }
}

// ---- CUDA-core passes -------------------------------------------------------

// x fp32 [N][V] -> bf16 [N][V][16]: channel 0 = x / scale[n], the rest 0.
__global__ void unet_input_kernel(const float *__restrict__ x, const float *__restrict__ scale,
                                  __nv_bfloat16 *__restrict__ out, long long vps, long long total) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const float v = x[i] / scale[i / vps];
        uint4 *o = reinterpret_cast<uint4 *>(out + i * 16);
        o[0] = make_uint4(pack_bf16x2(v, 0.0f), 0u, 0u, 0u);
        o[1] = make_uint4(0u, 0u, 0u, 0u);
    }
}

// The first layer on CUDA cores: out = relu(conv(a) + bias) with
// a = bf16(x / scale[sample]) the network's single real input channel — the
// same values as ctgb_unet_input followed by the 16-channel tensor-core
// convolution, whose channels 1-15 are zeros.  A block owns 256 x 8 output
// voxels of one z plane: it first stages a for the 3 x 10 x 258 input
// neighbourhood in shared memory (each value divided and rounded once),
// then each thread computes two voxels of each of the 8 rows: per tap, the
// two neighbours and the tap's 16 weights (broadcast float4 reads) feed 32
// FMAs; bias, ReLU and one 32-byte store per voxel.
constexpr int kFirstThreads = 128, kFirstX = 256, kFirstRows = 8;

__device__ __forceinline__ void first_store(__nv_bfloat16 *dst, const float (&acc)[16], const float *bs) {
    uint32_t p[8];
#pragma unroll
    for (int q = 0; q < 8; ++q)
        p[q] = pack_bf16x2(fmaxf(acc[2 * q] + bs[2 * q], 0.0f), fmaxf(acc[2 * q + 1] + bs[2 * q + 1], 0.0f));
    uint4 *o = reinterpret_cast<uint4 *>(dst);
    o[0] = make_uint4(p[0], p[1], p[2], p[3]);
    o[1] = make_uint4(p[4], p[5], p[6], p[7]);
}

__global__ void __launch_bounds__(kFirstThreads)
unet_first_kernel(const float *__restrict__ x, const float *__restrict__ scale, const __nv_bfloat16 *__restrict__ w0,
                  int cin, const float *__restrict__ bias, __nv_bfloat16 *__restrict__ out, int D, int H, int W) {
    constexpr int SX = kFirstX + 2, SY = kFirstRows + 2;
    __shared__ float sa[3][SY][SX];
    __shared__ float4 ws[27][4];   // tap t, outputs 4q .. 4q + 3
    __shared__ float bs[16];
    const int x0 = blockIdx.x * kFirstX, y0 = blockIdx.y * kFirstRows;
    const int zz = blockIdx.z % D, nn = blockIdx.z / D;
    const float s = scale[nn];
    const float *__restrict__ xs = x + (size_t)nn * D * H * W;
    for (int i = threadIdx.x; i < 27 * 16; i += kFirstThreads)
        reinterpret_cast<float *>(&ws[0][0])[i] = __bfloat162float(w0[(size_t)i * cin]);
    if (threadIdx.x < 16) bs[threadIdx.x] = bias[threadIdx.x];
    for (int i = threadIdx.x; i < 3 * SY * SX; i += kFirstThreads) {
        const int rx = i % SX, ry = (i / SX) % SY, dz = i / (SX * SY);
        const int z = zz + dz - 1, y = y0 + ry - 1, xi = x0 + rx - 1;
        float v = 0.0f;
        if (z >= 0 && z < D && y >= 0 && y < H && xi >= 0 && xi < W)
            v = __bfloat162float(__float2bfloat16_rn(__ldg(xs + ((size_t)z * H + y) * W + xi) / s));
        sa[dz][ry][rx] = v;
    }
    __syncthreads();
    const int t0 = threadIdx.x, t1 = threadIdx.x + kFirstThreads;   // the thread's two voxels in the run
    const bool ok0 = x0 + t0 < W, ok1 = x0 + t1 < W;
    for (int r = 0; r < kFirstRows && y0 + r < H; ++r) {
        float acc0[16], acc1[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) acc0[c] = acc1[c] = 0.0f;
        // Taps rolled over (dz, dy): the weights are re-read from shared
        // memory per row instead of being hoisted into 432 registers.
#pragma unroll 1
        for (int tzy = 0; tzy < 9; ++tzy) {
#pragma unroll
        for (int dx = 0; dx < 3; ++dx) {
            const int t = tzy * 3 + dx, dz = tzy / 3, dy = tzy % 3;
            const float a0 = sa[dz][r + dy][t0 + dx], a1 = sa[dz][r + dy][t1 + dx];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float4 wq = ws[t][q];
                acc0[4 * q] = fmaf(wq.x, a0, acc0[4 * q]);
                acc0[4 * q + 1] = fmaf(wq.y, a0, acc0[4 * q + 1]);
                acc0[4 * q + 2] = fmaf(wq.z, a0, acc0[4 * q + 2]);
                acc0[4 * q + 3] = fmaf(wq.w, a0, acc0[4 * q + 3]);
                acc1[4 * q] = fmaf(wq.x, a1, acc1[4 * q]);
                acc1[4 * q + 1] = fmaf(wq.y, a1, acc1[4 * q + 1]);
                acc1[4 * q + 2] = fmaf(wq.z, a1, acc1[4 * q + 2]);
                acc1[4 * q + 3] = fmaf(wq.w, a1, acc1[4 * q + 3]);
            }
        }
        }
        __nv_bfloat16 *row = out + (((size_t)nn * D + zz) * H + y0 + r) * W * 16;
        if (ok0) first_store(row + (size_t)(x0 + t0) * 16, acc0, bs);
        if (ok1) first_store(row + (size_t)(x0 + t1) * 16, acc1, bs);
    }
}

__device__ __forceinline__ void unpack8(uint4 u, float *f) {
    const __nv_bfloat162 *h = reinterpret_cast<const __nv_bfloat162 *>(&u);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float2 t = __bfloat1622float2(h[i]);
        f[2 * i] = t.x;
        f[2 * i + 1] = t.y;
    }
}

__device__ __forceinline__ uint4 pack8(const float *f) {
    return make_uint4(pack_bf16x2(f[0], f[1]), pack_bf16x2(f[2], f[3]), pack_bf16x2(f[4], f[5]),
                      pack_bf16x2(f[6], f[7]));
}

// 2x2x2 average pooling, bf16 [N][D][H][W][C] -> [N][D/2][H/2][W/2][C]; one
// thread per (output voxel, 8-channel group).
__global__ void pool2_kernel(const __nv_bfloat16 *__restrict__ in, __nv_bfloat16 *__restrict__ out, int N, int D,
                             int H, int W, int C) {
    const int Do = D / 2, Ho = H / 2, Wo = W / 2, G = C / 8;
    const long long total = (long long)N * Do * Ho * Wo * G;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int gch = (int)(i % G);
        long long v = i / G;
        const int x = (int)(v % Wo);
        v /= Wo;
        const int y = (int)(v % Ho);
        v /= Ho;
        const int z = (int)(v % Do);
        const int n = (int)(v / Do);
        float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const long long src = ((((long long)n * D + 2 * z + (k >> 2)) * H + 2 * y + ((k >> 1) & 1)) * W + 2 * x +
                                   (k & 1)) * C + gch * 8;
            float f[8];
            unpack8(*reinterpret_cast<const uint4 *>(in + src), f);
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[j] += f[j];
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[j] *= 0.125f;
        *reinterpret_cast<uint4 *>(out + i * 8) = pack8(acc);
    }
}

// Nearest 2x upsampling, bf16 [N][D/2][H/2][W/2][C] -> [N][D][H][W][C].
__global__ void up2_kernel(const __nv_bfloat16 *__restrict__ in, __nv_bfloat16 *__restrict__ out, int N, int D,
                           int H, int W, int C) {
    const int G = C / 8;
    const long long total = (long long)N * D * H * W * G;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int gch = (int)(i % G);
        long long v = i / G;
        const int x = (int)(v % W);
        v /= W;
        const int y = (int)(v % H);
        v /= H;
        const int z = (int)(v % D);
        const int n = (int)(v / D);
        const long long src = ((((long long)n * (D / 2) + z / 2) * (H / 2) + y / 2) * (W / 2) + x / 2) * C + gch * 8;
        *reinterpret_cast<uint4 *>(out + i * 8) = *reinterpret_cast<const uint4 *>(in + src);
    }
}

// out[v][c] = act[v][c] > 0 ? g[v * gs + go + c] : 0, as bf16 (the gradient
// through a ReLU whose output is act).
__global__ void relu_grad_kernel(const float *__restrict__ g, int gs, int go, const __nv_bfloat16 *__restrict__ act,
                                 __nv_bfloat16 *__restrict__ out, long long nvox, int C) {
    const long long total = nvox * (C / 8);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const long long v = i / (C / 8);
        const int c0 = (int)(i % (C / 8)) * 8;
        float a[8], r[8];
        unpack8(*reinterpret_cast<const uint4 *>(act + v * C + c0), a);
#pragma unroll
        for (int j = 0; j < 8; ++j) r[j] = a[j] > 0.0f ? g[v * gs + go + c0 + j] : 0.0f;
        *reinterpret_cast<uint4 *>(out + v * C + c0) = pack8(r);
    }
}

// Gradient through pooling (and the skip branch) and the ReLU before it:
// out[v][c] = act[v][c] > 0 ? gp[parent(v)][c] / 8 + gskip[v * gs + go + c] : 0.
__global__ void pool2_grad_kernel(const float *__restrict__ gp, const float *__restrict__ gskip, int gs, int go,
                                  const __nv_bfloat16 *__restrict__ act, __nv_bfloat16 *__restrict__ out, int N,
                                  int D, int H, int W, int C) {
    const int G = C / 8;
    const long long total = (long long)N * D * H * W * G;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int c0 = (int)(i % G) * 8;
        long long v = i / G;
        const long long vox = v;
        const int x = (int)(v % W);
        v /= W;
        const int y = (int)(v % H);
        v /= H;
        const int z = (int)(v % D);
        const int n = (int)(v / D);
        const long long par = (((long long)n * (D / 2) + z / 2) * (H / 2) + y / 2) * (W / 2) + x / 2;
        float a[8], r[8];
        unpack8(*reinterpret_cast<const uint4 *>(act + vox * C + c0), a);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            float s = gp[par * C + c0 + j] * 0.125f;
            if (gskip) s += gskip[vox * gs + go + c0 + j];
            r[j] = a[j] > 0.0f ? s : 0.0f;
        }
        *reinterpret_cast<uint4 *>(out + vox * C + c0) = pack8(r);
    }
}

// Gradient through nearest upsampling and the ReLU before it (act at the
// coarse level): out[p][c] = act[p][c] > 0 ? sum of the 8 children's
// g[child * gs + go + c] : 0.  D, H, W are the coarse dims.
__global__ void up2_grad_kernel(const float *__restrict__ g, int gs, int go, const __nv_bfloat16 *__restrict__ act,
                                __nv_bfloat16 *__restrict__ out, int N, int D, int H, int W, int C) {
    const int G = C / 8;
    const long long total = (long long)N * D * H * W * G;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int c0 = (int)(i % G) * 8;
        long long v = i / G;
        const long long vox = v;
        const int x = (int)(v % W);
        v /= W;
        const int y = (int)(v % H);
        v /= H;
        const int z = (int)(v % D);
        const int n = (int)(v / D);
        float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const long long ch = ((((long long)n * 2 * D + 2 * z + (k >> 2)) * 2 * H + 2 * y + ((k >> 1) & 1)) * 2 * W +
                                  2 * x + (k & 1));
#pragma unroll
            for (int j = 0; j < 8; ++j) s[j] += g[ch * gs + go + c0 + j];
        }
        float a[8], r[8];
        unpack8(*reinterpret_cast<const uint4 *>(act + vox * C + c0), a);
#pragma unroll
        for (int j = 0; j < 8; ++j) r[j] = a[j] > 0.0f ? s[j] : 0.0f;
        *reinterpret_cast<uint4 *>(out + vox * C + c0) = pack8(r);
    }
}

// Head: y[v] = x[v] + scale[n] * (sum_c w[c] a[v][c] + b), a bf16 [V][16].
__global__ void head_kernel(const __nv_bfloat16 *__restrict__ a, const float *__restrict__ wb,
                            const float *__restrict__ x, const float *__restrict__ scale, float *__restrict__ y,
                            long long vps, long long total) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        float f[16];
        unpack8(*reinterpret_cast<const uint4 *>(a + i * 16), f);
        unpack8(*reinterpret_cast<const uint4 *>(a + i * 16 + 8), f + 8);
        float s = wb[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) s = fmaf(wb[c], f[c], s);
        y[i] = x[i] + scale[i / vps] * s;
    }
}

// Head gradient: gin = gy * scale (the gradient of the head's sum);
// ga[v][c] = a[v][c] > 0 ? gin w[c] : 0 (bf16); per-block partial sums of
// gin a[v][c] (16) and gin (1) -> partials[block][17].
__global__ void head_grad_kernel(const float *__restrict__ gy, const __nv_bfloat16 *__restrict__ a,
                                 const float *__restrict__ wb, const float *__restrict__ scale,
                                 __nv_bfloat16 *__restrict__ ga, float *__restrict__ partials, long long vps,
                                 long long total) {
    __shared__ float red[17][256];
    float acc[17];
#pragma unroll
    for (int c = 0; c < 17; ++c) acc[c] = 0.0f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const float gin = gy[i] * scale[i / vps];
        float f[16], r[16];
        unpack8(*reinterpret_cast<const uint4 *>(a + i * 16), f);
        unpack8(*reinterpret_cast<const uint4 *>(a + i * 16 + 8), f + 8);
#pragma unroll
        for (int c = 0; c < 16; ++c) {
            acc[c] = fmaf(gin, f[c], acc[c]);
            r[c] = f[c] > 0.0f ? gin * wb[c] : 0.0f;
        }
        acc[16] += gin;
        *reinterpret_cast<uint4 *>(ga + i * 16) = pack8(r);
        *reinterpret_cast<uint4 *>(ga + i * 16 + 8) = pack8(r + 8);
    }
#pragma unroll
    for (int c = 0; c < 17; ++c) red[c][threadIdx.x] = acc[c];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s)
            for (int c = 0; c < 17; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x < 17) partials[blockIdx.x * 17 + threadIdx.x] = red[threadIdx.x][0];
}

// Weight gradient of a 3x3x3 convolution (zero padding):
//   dW[tap][co][ci] = sum_v g[v][co] * x[v + offset(tap)][ci]
// The voxels are cut into x-row segments of at most kWgSeg voxels; a chunk
// is kWgSegs consecutive segments.  Block (chunk, dz, pair group): per
// segment, the output gradient g of the segment and the three input rows at
// (z + dz, y - 1 .. y + 1) over the segment plus one voxel each side are
// staged in shared memory as fp32; each thread owns at most kWgPairs
// (co, ci) pairs of the group and, for the 9 (dy, dx) taps of its dz,
// slides a three-voxel window along x, so each voxel costs it one g read and
// three x reads for nine FMAs per pair.  Per-block partials ->
// partials[chunk][tap][co][ci] (every block writes its 9 taps).
constexpr int kWgSeg = 64, kWgSegs = 64, kWgThreads = 256, kWgPairs = 2;

__device__ __forceinline__ void wgrad_segments(long long nseg, int segs_per_row, int W, int *sx0, int *slen,
                                               long long seg, long long *row) {
    *row = seg / segs_per_row;
    *sx0 = (int)(seg - *row * segs_per_row) * kWgSeg;
    *slen = min(kWgSeg, W - *sx0);
}

__global__ void __launch_bounds__(kWgThreads) wgrad_kernel(const __nv_bfloat16 *__restrict__ x, int cin,
                                                           const __nv_bfloat16 *__restrict__ g, int cout,
                                                           float *__restrict__ partials, int N, int D, int H,
                                                           int W) {
    extern __shared__ float wsm[];
    float *gs = wsm;                               // [kWgSeg][cout]
    float *xs = wsm + kWgSeg * cout;               // [3][kWgSeg + 2][cin]
    const int chunk = blockIdx.x, dzi = blockIdx.y, pgroup = blockIdx.z;
    const int dz = dzi - 1;
    const int segs_per_row = (W + kWgSeg - 1) / kWgSeg;
    const long long nseg = (long long)N * D * H * segs_per_row;
    const long long s0 = (long long)chunk * kWgSegs, s1 = min(nseg, s0 + kWgSegs);
    const int npairs = cout * cin;
    int co[kWgPairs], ci[kWgPairs];
    bool has[kWgPairs];
#pragma unroll
    for (int k = 0; k < kWgPairs; ++k) {
        const int p = (pgroup * kWgPairs + k) * kWgThreads + threadIdx.x;
        has[k] = p < npairs;
        co[k] = has[k] ? p / cin : 0;
        ci[k] = has[k] ? p % cin : 0;
    }
    float acc[kWgPairs][9];
#pragma unroll
    for (int k = 0; k < kWgPairs; ++k)
#pragma unroll
        for (int t = 0; t < 9; ++t) acc[k][t] = 0.0f;
    const int SX = kWgSeg + 2;
    for (long long sg = s0; sg < s1; ++sg) {
        long long row;
        int sx0, slen;
        wgrad_segments(nseg, segs_per_row, W, &sx0, &slen, sg, &row);
        const int yy = (int)(row % H), zz = (int)((row / H) % D), nn = (int)(row / ((long long)H * D));
        __syncthreads();                           // the previous segment's reads are done
        // 8 channels (16 bytes) per staged item; channel counts are multiples of 8
        const __nv_bfloat16 *grow = g + ((((long long)nn * D + zz) * H + yy) * W + sx0) * cout;
        const int gv8 = cout / 8;
        for (int e = threadIdx.x; e < kWgSeg * gv8; e += kWgThreads) {
            float f[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
            if (e < slen * gv8) unpack8(__ldg(reinterpret_cast<const uint4 *>(grow) + e), f);
            float4 *dstg = reinterpret_cast<float4 *>(gs + e * 8);
            dstg[0] = make_float4(f[0], f[1], f[2], f[3]);
            dstg[1] = make_float4(f[4], f[5], f[6], f[7]);
        }
        const int z2 = zz + dz, xv8 = cin / 8;
        for (int e = threadIdx.x; e < 3 * SX * xv8; e += kWgThreads) {
            const int c8 = e % xv8, r = e / xv8, xi = r % SX, dyi = r / SX;
            const int y2 = yy + dyi - 1, x2 = sx0 + xi - 1;
            float f[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
            if (z2 >= 0 && z2 < D && y2 >= 0 && y2 < H && x2 >= 0 && x2 < W && xi <= slen + 1)
                unpack8(__ldg(reinterpret_cast<const uint4 *>(x + ((((long long)nn * D + z2) * H + y2) * W + x2) * cin) +
                              c8),
                        f);
            float4 *dstx = reinterpret_cast<float4 *>(xs + (size_t)r * cin + c8 * 8);
            dstx[0] = make_float4(f[0], f[1], f[2], f[3]);
            dstx[1] = make_float4(f[4], f[5], f[6], f[7]);
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kWgPairs; ++k) {
            if (!has[k]) continue;
            float w0[3], w1[3];                    // x[v - 1], x[v] per dy row
#pragma unroll
            for (int dy = 0; dy < 3; ++dy) {
                w0[dy] = xs[(dy * SX + 0) * cin + ci[k]];
                w1[dy] = xs[(dy * SX + 1) * cin + ci[k]];
            }
#pragma unroll 4
            for (int v = 0; v < slen; ++v) {
                const float gv = gs[v * cout + co[k]];
#pragma unroll
                for (int dy = 0; dy < 3; ++dy) {
                    const float w2 = xs[(dy * SX + v + 2) * cin + ci[k]];
                    acc[k][dy * 3 + 0] = fmaf(gv, w0[dy], acc[k][dy * 3 + 0]);
                    acc[k][dy * 3 + 1] = fmaf(gv, w1[dy], acc[k][dy * 3 + 1]);
                    acc[k][dy * 3 + 2] = fmaf(gv, w2, acc[k][dy * 3 + 2]);
                    w0[dy] = w1[dy];
                    w1[dy] = w2;
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < kWgPairs; ++k) {
        if (!has[k]) continue;
        const int p = co[k] * cin + ci[k];
#pragma unroll
        for (int t = 0; t < 9; ++t)
            partials[((long long)chunk * 27 + dzi * 9 + t) * npairs + p] = acc[k][t];
    }
}

// Bias gradient partials: partials[block][c] = sum over the block's voxels of g[v][c].
__global__ void colsum_kernel(const __nv_bfloat16 *__restrict__ g, int C, long long nvox,
                              float *__restrict__ partials) {
    extern __shared__ float red[];   // [blockDim][C]
    for (int c = 0; c < C; ++c) red[threadIdx.x * C + c] = 0.0f;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvox;
         v += (long long)gridDim.x * blockDim.x)
        for (int c = 0; c < C; ++c) red[threadIdx.x * C + c] += __bfloat162float(g[v * C + c]);
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s)
            for (int c = 0; c < C; ++c) red[threadIdx.x * C + c] += red[(threadIdx.x + s) * C + c];
        __syncthreads();
    }
    if ((int)threadIdx.x < C) partials[blockIdx.x * C + threadIdx.x] = red[threadIdx.x];
}

static int grid_for(long long n, int threads = 256) {
    long long b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > 152 * 32) b = 152 * 32;
    return (int)b;
}

static bool good_c(int c) { return c == 16 || c == 32 || c == 64; }

template <int COUT, int CMAX, int EPI>
static int launch_conv(const CUtensorMap &a0, const CUtensorMap &a1, const CUtensorMap &b0, const CUtensorMap &b1,
                       const ConvGeom &g, const float *bias, void *out, cudaStream_t st) {
    using Cfg = ConvCfg<COUT, CMAX>;
    static std::atomic<unsigned long long> attr{0};
    cudaError_t ea = smem_limit_once((const void *)conv3d_tc_kernel<COUT, CMAX, EPI>, Cfg::kSmem, attr);
    if (ea != cudaSuccess) return set_error(CTGB_ERR_CUDA, "conv3d smem attribute: %s", cudaGetErrorString(ea));
    int *status = ctgb_status_ptr();
    if (!status) return set_error(CTGB_ERR_CUDA, "device status word unavailable");
    const long long tiles = (long long)g.N * g.D * (g.H / g.R) * (g.W / g.Wb);
    if (tiles > 0x7fffffffLL) return set_error(CTGB_ERR_SIZE, "conv3d: too many tiles");
    conv3d_tc_kernel<COUT, CMAX, EPI><<<(unsigned)tiles, kCvThreads, Cfg::kSmem, st>>>(a0, a1, b0, b1, g, bias,
                                                                                      out, status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "conv3d_tc_kernel: %s", cudaGetErrorString(e));
    return CTGB_OK;
}

template <int COUT, int CMAX, int EPI, bool RES>
static int launch_conv_dx_res(const CUtensorMap &a0, const CUtensorMap &a1, const CUtensorMap &b0,
                              const CUtensorMap &b1, const ConvGeom &g, const float *bias, void *out, cudaStream_t st) {
    using Cfg = ConvDxCfg<COUT, CMAX, RES>;
    // Resident weights, rounded up so that the stage ring starts 1024-byte
    // aligned (the 128-byte swizzle's repeat).
    const int wres = RES ? (g.nseg * 27 * Cfg::kBTap + 1023) / 1024 * 1024 : 0;
    const int smem = wres + Cfg::kSmemFixed;
    // Largest dynamic shared memory this instantiation can ask for; shapes
    // that would not fit never get here (ctgb_unet_conv3d routes them to
    // conv3d_tc_kernel).
    constexpr int kSmemMax = (RES ? Cfg::kWMax : 0) + Cfg::kSmemFixed;
    if constexpr (kSmemMax > kDxSmemLimit) {
        return set_error(CTGB_ERR_ARG, "conv3d: tap-reuse shape above the shared-memory limit");
    } else {
    static std::atomic<unsigned long long> attr{0};
    cudaError_t ea = smem_limit_once((const void *)conv3d_tc_dx_kernel<COUT, CMAX, EPI, RES>, kSmemMax, attr);
    if (ea != cudaSuccess) return set_error(CTGB_ERR_CUDA, "conv3d smem attribute: %s", cudaGetErrorString(ea));
    int *status = ctgb_status_ptr();
    if (!status) return set_error(CTGB_ERR_CUDA, "device status word unavailable");
    const long long tiles = (long long)g.N * g.D * ((g.H + Cfg::kR - 1) / Cfg::kR) * (g.W / kCvM);
    if (tiles > 0x7fffffffLL) return set_error(CTGB_ERR_SIZE, "conv3d: too many tiles");
    // Persistent grid: as many CTAs as fit on the GPU at once (shared memory,
    // TMEM and thread bound), never more than the tiles.
    int sms = 0, smem_sm = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    int per_sm = smem_sm / (smem + 1024);
    if (per_sm > 512 / Cfg::kTmemCols) per_sm = 512 / Cfg::kTmemCols;
    if (per_sm > 2048 / kDxThreads) per_sm = 2048 / kDxThreads;
    const long long resident = (long long)(per_sm < 1 ? 1 : per_sm) * (sms < 1 ? 1 : sms);
    const int grid = (int)(tiles < resident ? tiles : resident);
    conv3d_tc_dx_kernel<COUT, CMAX, EPI, RES><<<grid, kDxThreads, smem, st>>>(a0, a1, b0, b1, g, wres, bias, out,
                                                                             status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "conv3d_tc_dx_kernel: %s", cudaGetErrorString(e));
    return CTGB_OK;
    }
}

template <int COUT, int CMAX, int EPI>
static int launch_conv_dx(const CUtensorMap &a0, const CUtensorMap &a1, const CUtensorMap &b0,
                          const CUtensorMap &b1, const ConvGeom &g, const float *bias, void *out, cudaStream_t st) {
    // Weights resident when they fit kDxWMax.
    const long long wres = (long long)g.nseg * 27 * ConvDxCfg<COUT, CMAX, true>::kBTap;
    if (wres <= ConvDxCfg<COUT, CMAX, true>::kWMax)
        return launch_conv_dx_res<COUT, CMAX, EPI, true>(a0, a1, b0, b1, g, bias, out, st);
    return launch_conv_dx_res<COUT, CMAX, EPI, false>(a0, a1, b0, b1, g, bias, out, st);
}

}  // namespace ctgb

using namespace ctgb;

extern "C" int ctgb_unet_conv3d(const void *x0, int32_t c0, const void *x1, int32_t c1, const void *w0,
                                const void *w1, const float *bias, void *out, int32_t cout, int32_t n, int32_t d,
                                int32_t h, int32_t w, int32_t mode, void *stream) {
    clear_error();
    if (!x0 || !w0 || !out || (c1 && (!x1 || !w1)) || (mode == 0 && !bias))
        return set_error(CTGB_ERR_ARG, "ctgb_unet_conv3d: NULL argument");
    if (!good_c(c0) || !(c1 == 0 || good_c(c1)))
        return set_error(CTGB_ERR_ARG, "ctgb_unet_conv3d: input channels must be 16, 32 or 64");
    if (!(cout == 16 || cout == 32 || cout == 48 || cout == 64 || cout == 96))
        return set_error(CTGB_ERR_ARG, "ctgb_unet_conv3d: output channels must be 16, 32, 48, 64 or 96");
    if (mode != 0 && mode != 1) return set_error(CTGB_ERR_ARG, "ctgb_unet_conv3d: mode must be 0 or 1");
    if (n < 1 || d < 1 || h < 1 || w < 16) return set_error(CTGB_ERR_ARG, "ctgb_unet_conv3d: bad volume size");
    int wb;
    if (w % 128 == 0) wb = 128;
    else if (w == 16 || w == 32 || w == 64) wb = w;
    else return set_error(CTGB_ERR_ARG, "ctgb_unet_conv3d: W must be 16, 32, 64 or a multiple of 128");
    const int r = 128 / wb;
    if (h % r) return set_error(CTGB_ERR_ARG, "ctgb_unet_conv3d: H must be a multiple of %d for W = %d", r, w);
    ConvGeom g{n, d, h, w, wb, r, c0, c1, c1 ? 2 : 1};
    // Rows of 128 voxels take the tap reuse kernel: input boxes of C channels
    // x 130 voxels x (R + 2) rows, weight boxes as before.
    int dx_r = 1;
    const bool dxr = (w % kCvM) == 0 && dx_fits(cout, c0 > c1 ? c0 : c1, c1 ? 2 : 1, &dx_r);
    CUtensorMap ta0, ta1, tb0, tb1;
    {
        const uint64_t dims[5] = {(uint64_t)c0, (uint64_t)w, (uint64_t)h, (uint64_t)d, (uint64_t)n};
        const uint32_t box[5] = {(uint32_t)c0, dxr ? (uint32_t)(kCvM + 2) : (uint32_t)wb,
                                 dxr ? (uint32_t)(dx_r + 2) : (uint32_t)r, 1u, 1u};
        const uint64_t wd[2] = {(uint64_t)c0, (uint64_t)(27 * cout)};
        const uint32_t wbx[2] = {(uint32_t)c0, (uint32_t)cout};
        if (!ctgb_make_tmap_bf16(&ta0, x0, 5, dims, box) || !ctgb_make_tmap_bf16(&tb0, w0, 2, wd, wbx))
            return set_error(CTGB_ERR_ARG, "ctgb_unet_conv3d: tensor map rejected (alignment?)");
    }
    if (c1) {
        const uint64_t dims[5] = {(uint64_t)c1, (uint64_t)w, (uint64_t)h, (uint64_t)d, (uint64_t)n};
        const uint32_t box[5] = {(uint32_t)c1, dxr ? (uint32_t)(kCvM + 2) : (uint32_t)wb,
                                 dxr ? (uint32_t)(dx_r + 2) : (uint32_t)r, 1u, 1u};
        const uint64_t wd[2] = {(uint64_t)c1, (uint64_t)(27 * cout)};
        const uint32_t wbx[2] = {(uint32_t)c1, (uint32_t)cout};
        if (!ctgb_make_tmap_bf16(&ta1, x1, 5, dims, box) || !ctgb_make_tmap_bf16(&tb1, w1, 2, wd, wbx))
            return set_error(CTGB_ERR_ARG, "ctgb_unet_conv3d: tensor map rejected (alignment?)");
    } else {
        ta1 = ta0;
        tb1 = tb0;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int cmax = c0 > c1 ? c0 : c1;
#define CTGB_CONV_CM(CO, CM)                                                                      \
    if (cmax == CM && dxr)                                                                       \
        return mode == 0 ? launch_conv_dx<CO, CM, 0>(ta0, ta1, tb0, tb1, g, bias, out, st)       \
                         : launch_conv_dx<CO, CM, 1>(ta0, ta1, tb0, tb1, g, bias, out, st);     \
    if (cmax == CM)                                                                              \
        return mode == 0 ? launch_conv<CO, CM, 0>(ta0, ta1, tb0, tb1, g, bias, out, st)          \
                         : launch_conv<CO, CM, 1>(ta0, ta1, tb0, tb1, g, bias, out, st);
#define CTGB_CONV_CASE(CO)   \
    case CO:                 \
        CTGB_CONV_CM(CO, 16) \
        CTGB_CONV_CM(CO, 32) \
        CTGB_CONV_CM(CO, 64) \
        break;
    switch (cout) {
        CTGB_CONV_CASE(16)
        CTGB_CONV_CASE(32)
        CTGB_CONV_CASE(48)
        CTGB_CONV_CASE(64)
        CTGB_CONV_CASE(96)
    }
#undef CTGB_CONV_CASE
#undef CTGB_CONV_CM
    return set_error(CTGB_ERR_ARG, "ctgb_unet_conv3d: unsupported output channels");
}

static int ew_done(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(CTGB_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
    return CTGB_OK;
}

extern "C" int ctgb_unet_input(const float *x, const float *scale, void *out, int32_t n, int64_t vps, void *stream) {
    clear_error();
    if (!x || !scale || !out || n < 1 || vps < 1) return set_error(CTGB_ERR_ARG, "ctgb_unet_input: bad arguments");
    const long long total = (long long)n * vps;
    unet_input_kernel<<<grid_for(total), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        x, scale, static_cast<__nv_bfloat16 *>(out), vps, total);
    return ew_done("unet_input_kernel");
}

extern "C" int ctgb_unet_first(const float *x, const float *scale, const void *w0, int32_t cin, const float *bias,
                               void *out, int32_t n, int32_t d, int32_t h, int32_t w, void *stream) {
    clear_error();
    if (!x || !scale || !w0 || !bias || !out) return set_error(CTGB_ERR_ARG, "ctgb_unet_first: NULL argument");
    if (cin < 1 || n < 1 || d < 1 || h < 1 || w < 1)
        return set_error(CTGB_ERR_ARG, "ctgb_unet_first: bad sizes");
    if ((long long)n * d > 65535) return set_error(CTGB_ERR_SIZE, "ctgb_unet_first: N * D must be at most 65535");
    dim3 grid((unsigned)((w + kFirstX - 1) / kFirstX), (unsigned)((h + kFirstRows - 1) / kFirstRows),
              (unsigned)(n * d));
    unet_first_kernel<<<grid, kFirstThreads, 0, static_cast<cudaStream_t>(stream)>>>(
        x, scale, static_cast<const __nv_bfloat16 *>(w0), cin, bias, static_cast<__nv_bfloat16 *>(out), d, h, w);
    return ew_done("unet_first_kernel");
}

extern "C" int ctgb_unet_pool2(const void *in, void *out, int32_t n, int32_t d, int32_t h, int32_t w, int32_t c,
                               void *stream) {
    clear_error();
    if (!in || !out || c % 8 || c < 8 || d % 2 || h % 2 || w % 2 || n < 1 || d < 2)
        return set_error(CTGB_ERR_ARG, "ctgb_unet_pool2: bad arguments");
    const long long total = (long long)n * (d / 2) * (h / 2) * (w / 2) * (c / 8);
    pool2_kernel<<<grid_for(total), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const __nv_bfloat16 *>(in), static_cast<__nv_bfloat16 *>(out), n, d, h, w, c);
    return ew_done("pool2_kernel");
}

extern "C" int ctgb_unet_up2(const void *in, void *out, int32_t n, int32_t d, int32_t h, int32_t w, int32_t c,
                             void *stream) {
    clear_error();
    if (!in || !out || c % 8 || c < 8 || d % 2 || h % 2 || w % 2 || n < 1)
        return set_error(CTGB_ERR_ARG, "ctgb_unet_up2: bad arguments");
    const long long total = (long long)n * d * h * w * (c / 8);
    up2_kernel<<<grid_for(total), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const __nv_bfloat16 *>(in), static_cast<__nv_bfloat16 *>(out), n, d, h, w, c);
    return ew_done("up2_kernel");
}

extern "C" int ctgb_unet_relu_grad(const float *g, int32_t gs, int32_t go, const void *act, void *out, int64_t nvox,
                                   int32_t c, void *stream) {
    clear_error();
    if (!g || !act || !out || c % 8 || c < 8 || go < 0 || go + c > gs || nvox < 0)
        return set_error(CTGB_ERR_ARG, "ctgb_unet_relu_grad: bad arguments");
    relu_grad_kernel<<<grid_for(nvox * (c / 8)), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        g, gs, go, static_cast<const __nv_bfloat16 *>(act), static_cast<__nv_bfloat16 *>(out), nvox, c);
    return ew_done("relu_grad_kernel");
}

extern "C" int ctgb_unet_pool2_grad(const float *gp, const float *gskip, int32_t gs, int32_t go, const void *act,
                                    void *out, int32_t n, int32_t d, int32_t h, int32_t w, int32_t c, void *stream) {
    clear_error();
    if (!gp || !act || !out || c % 8 || c < 8 || d % 2 || h % 2 || w % 2 || (gskip && (go < 0 || go + c > gs)))
        return set_error(CTGB_ERR_ARG, "ctgb_unet_pool2_grad: bad arguments");
    const long long total = (long long)n * d * h * w * (c / 8);
    pool2_grad_kernel<<<grid_for(total), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        gp, gskip, gs, go, static_cast<const __nv_bfloat16 *>(act), static_cast<__nv_bfloat16 *>(out), n, d, h, w,
        c);
    return ew_done("pool2_grad_kernel");
}

extern "C" int ctgb_unet_up2_grad(const float *g, int32_t gs, int32_t go, const void *act, void *out, int32_t n,
                                  int32_t d, int32_t h, int32_t w, int32_t c, void *stream) {
    clear_error();
    if (!g || !act || !out || c % 8 || c < 8 || go < 0 || go + c > gs)
        return set_error(CTGB_ERR_ARG, "ctgb_unet_up2_grad: bad arguments");
    const long long total = (long long)n * d * h * w * (c / 8);
    up2_grad_kernel<<<grid_for(total), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        g, gs, go, static_cast<const __nv_bfloat16 *>(act), static_cast<__nv_bfloat16 *>(out), n, d, h, w, c);
    return ew_done("up2_grad_kernel");
}

extern "C" int ctgb_unet_head(const void *a, const float *wb, const float *x, const float *scale, float *y, int32_t n,
                              int64_t vps, void *stream) {
    clear_error();
    if (!a || !wb || !x || !scale || !y || n < 1 || vps < 1) return set_error(CTGB_ERR_ARG, "ctgb_unet_head: bad arguments");
    const long long total = (long long)n * vps;
    head_kernel<<<grid_for(total), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const __nv_bfloat16 *>(a), wb, x, scale, y, vps, total);
    return ew_done("head_kernel");
}

extern "C" int ctgb_unet_head_grad_blocks(int64_t total, int32_t *blocks) {
    clear_error();
    if (!blocks || total < 1) return set_error(CTGB_ERR_ARG, "ctgb_unet_head_grad_blocks: bad arguments");
    *blocks = grid_for(total);
    return CTGB_OK;
}

extern "C" int ctgb_unet_head_grad(const float *gy, const void *a, const float *wb, const float *scale, void *ga,
                                   float *partials, int32_t n, int64_t vps, void *stream) {
    clear_error();
    if (!gy || !a || !wb || !scale || !ga || !partials || n < 1 || vps < 1)
        return set_error(CTGB_ERR_ARG, "ctgb_unet_head_grad: bad arguments");
    const long long total = (long long)n * vps;
    head_grad_kernel<<<grid_for(total), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        gy, static_cast<const __nv_bfloat16 *>(a), wb, scale, static_cast<__nv_bfloat16 *>(ga), partials, vps,
        total);
    return ew_done("head_grad_kernel");
}

extern "C" int ctgb_unet_wgrad_chunks(int32_t n, int32_t d, int32_t h, int32_t w, int32_t *chunks) {
    clear_error();
    if (!chunks || n < 1 || d < 1 || h < 1 || w < 1) return set_error(CTGB_ERR_ARG, "ctgb_unet_wgrad_chunks: bad arguments");
    const long long nseg = (long long)n * d * h * ((w + kWgSeg - 1) / kWgSeg);
    const long long c = (nseg + kWgSegs - 1) / kWgSegs;
    if (c > 0x7fffffffLL) return set_error(CTGB_ERR_SIZE, "ctgb_unet_wgrad_chunks: volume too large");
    *chunks = (int)c;
    return CTGB_OK;
}

extern "C" int ctgb_unet_wgrad(const void *x, int32_t cin, const void *g, int32_t cout, float *partials, int32_t n,
                               int32_t d, int32_t h, int32_t w, void *stream) {
    clear_error();
    if (!x || !g || !partials || cin < 8 || cout < 8 || cin % 8 || cout % 8 || cin * cout > 6144 || n < 1 || d < 1 ||
        h < 1 || w < 1)
        return set_error(CTGB_ERR_ARG, "ctgb_unet_wgrad: bad arguments (channels: multiples of 8)");
    int chunks = 0;
    if (int st = ctgb_unet_wgrad_chunks(n, d, h, w, &chunks)) return st;
    const int pgroups = (cin * cout + kWgThreads * kWgPairs - 1) / (kWgThreads * kWgPairs);
    const size_t smem = sizeof(float) * ((size_t)kWgSeg * cout + 3 * (size_t)(kWgSeg + 2) * cin);
    if (cin > 96 || cout > 96) return set_error(CTGB_ERR_ARG, "ctgb_unet_wgrad: at most 96 channels");
    static std::atomic<unsigned long long> attr{0};
    cudaError_t ea = smem_limit_once((const void *)wgrad_kernel,
                                     (int)(sizeof(float) * (kWgSeg * 96 + 3 * (kWgSeg + 2) * 96)), attr);
    if (ea != cudaSuccess) return set_error(CTGB_ERR_CUDA, "wgrad smem attribute: %s", cudaGetErrorString(ea));
    dim3 grid(chunks, 3, pgroups);
    wgrad_kernel<<<grid, kWgThreads, smem, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const __nv_bfloat16 *>(x), cin, static_cast<const __nv_bfloat16 *>(g), cout, partials, n, d, h,
        w);
    return ew_done("wgrad_kernel");
}

extern "C" int ctgb_unet_colsum(const void *g, int32_t c, int64_t nvox, float *partials, int32_t blocks,
                                void *stream) {
    clear_error();
    if (!g || !partials || c < 1 || c > 64 || nvox < 1 || blocks < 1)
        return set_error(CTGB_ERR_ARG, "ctgb_unet_colsum: bad arguments");
    const int threads = 128;
    colsum_kernel<<<blocks, threads, sizeof(float) * threads * c, static_cast<cudaStream_t>(stream)>>>(
        static_cast<const __nv_bfloat16 *>(g), c, nvox, partials);
    return ew_done("colsum_kernel");
}
