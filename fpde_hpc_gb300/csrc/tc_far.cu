// Far-history contraction on the 5th-generation tensor cores (tcgen05), split precision.
//
// For a block of BN upcoming steps starting at n0, the history older than the block enters
// every step of the block through a dense product
//     C[i][j] = sum_{t < n0} A[i][t] * W[t][j],   A[i][t] = D_t[i] (node i, increment t),
//                                                  W[t][j] = w[n0 + j - t] (Toeplitz weights),
// M = nodes, N = BN = 64 steps, K = n0. This is the reference's mode-1 far-history tile
// product (fr_do.cpp:173-235, wmma 16x16x16 half/float), rebuilt for sm_103a:
//   * A and W are stored as 16-bit hi/lo pairs (fp16 with power-of-two scaling, or bf16);
//     three products A_hi W_hi + A_hi W_lo + A_lo W_hi run as kind::f16 MMAs
//     (M=128, N=64, K=16) accumulating in FP32 in TMEM;
//   * every 256 history columns the TMEM accumulator is folded into float-float (hi, lo)
//     registers by the epilogue warps while the MMA warp fills the other TMEM buffer; the
//     CTA's result is written as FP64 partial sums C[split][j][row];
//   * operands arrive by TMA (cp.async.bulk.tensor, 128-byte swizzle) into a 4-stage ring
//     guarded by mbarriers; no multicast.
// Warp roles (192 threads): warp 0 TMA producer, warp 1 TMEM allocator + MMA issuer,
// warps 2-5 epilogue (TMEM lane quadrant = warp % 4).
// Every wait is bounded (2 s of %globaltimer); on timeout the kernel raises
// DEVERR_MBAR_TIMEOUT, stops issuing, drains its own copies (bounded) and frees its TMEM.
#include <algorithm>
#include <cuda.h>
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.cuh"
#include "tc_far.cuh"

namespace fpde {
namespace tc {

constexpr int BM = 128, BN = 64, BK = 64;
constexpr int STAGES = 4;
constexpr int CHUNK_KT = 4;                          // k-tiles per TMEM accumulation chunk
constexpr int A_BYTES = BM * BK * 2;                 // 16 KB
constexpr int W_BYTES = BN * BK * 2;                 // 8 KB
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * W_BYTES;
constexpr int TMEM_COLS = 128;                       // two 64-column fp32 accumulators
constexpr int THREADS = 192;
constexpr int SMEM_BYTES = 1024 + STAGES * STAGE_BYTES + 256;
constexpr unsigned long long WAIT_NS = 2000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long gtimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait on the phase with the given parity.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, unsigned *flags, volatile int *abort_s)
{
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = gtimer();
    while (true) {
        if (mbar_try_wait(bar, parity)) return true;
        if (*abort_s) return false;
        if (gtimer() - t0 > WAIT_NS) {
            atomicOr(flags, DEVERR_MBAR_TIMEOUT);
            *abort_s = 1;
            return false;
        }
    }
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *tm, int x, int y, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst)), "l"((uint64_t)tm), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// K-major operand tile, 128-byte swizzle: rows of 128 B, 8-row atoms of 1024 B (SBO).
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);        // start address
    d |= (uint64_t)1 << 16;                          // leading byte offset (unused for SW128 K-major)
    d |= (uint64_t)(1024 >> 4) << 32;                // stride byte offset: 8 rows x 128 B
    d |= (uint64_t)1 << 46;                          // descriptor version (tcgen05)
    d |= (uint64_t)2 << 61;                          // SWIZZLE_128B
    return d;
}

// Instruction descriptor, kind::f16: D f32, A/B fp16 (0) or bf16 (1), both K-major.
__host__ __device__ constexpr uint32_t idesc_f16(int bf16, int M, int N)
{
    return (1u << 4) | ((uint32_t)bf16 << 7) | ((uint32_t)bf16 << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma(uint32_t dtm, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
        ::"r"(dtm), "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}
// Same MMA with both smem descriptors given as (low, high) 32-bit words: the high words are
// constant and the low words differ from a stage's base only by the operand offset >> 4 (the
// 14-bit start-address field cannot carry: shared memory ends below 256 KB), so the issuing
// thread forms each descriptor with one integer add.
__device__ __forceinline__ void umma_lo(uint32_t dtm, uint32_t alo, uint32_t blo, uint32_t dhi, uint32_t idesc,
                                        uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .b64 da, db;\n\t.reg .pred p;\n\t"
        "mov.b64 da, {%1, %3};\n\t"
        "mov.b64 db, {%2, %3};\n\t"
        "setp.ne.b32 p, %5, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], da, db, %4, p;\n\t}\n"
        ::"r"(dtm), "r"(alo), "r"(blo), "r"(dhi), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void umma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float *v)
{
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float *v)
{
    uint32_t r[4];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(taddr));
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = __uint_as_float(r[k]);
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

struct __align__(64) FarMaps {
    CUtensorMap a_hi, a_lo, w_hi, w_lo;
};

// grid = (row tiles, K splits); split y covers k-tiles [y*kt_per, min((y+1)*kt_per, kt_total)).
__global__ void __launch_bounds__(THREADS, 1)
    k_far_tc(const __grid_constant__ FarMaps maps, double *__restrict__ C, int64_t ldc_split, int64_t ldc_col,
             int64_t rows, int kt_total, int kt_per, uint32_t idesc, double out_scale,
             const double *__restrict__ out_scale_ptr, unsigned *flags)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *stage_base = smem;
    uint64_t *bars = (uint64_t *)(smem + STAGES * STAGE_BYTES);
    uint64_t *full = bars, *empty = bars + STAGES, *tfull = bars + 2 * STAGES, *tempty = bars + 2 * STAGES + 2;
    uint64_t *mma_done = bars + 2 * STAGES + 4;
    volatile uint32_t *tmem_slot = (volatile uint32_t *)(bars + 2 * STAGES + 5);
    volatile int *abort_s = (volatile int *)(bars + 2 * STAGES + 6);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int mt = blockIdx.x, split = blockIdx.y;
    const int kt0 = split * kt_per;
    const int kt1 = min(kt0 + kt_per, kt_total);
    const int nkt = max(0, kt1 - kt0);
    const int nchunks = (nkt + CHUNK_KT - 1) / CHUNK_KT;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
        for (int b = 0; b < 2; ++b) { mbar_init(&tfull[b], 1); mbar_init(&tempty[b], 128); }
        mbar_init(mma_done, 1);
        *abort_s = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32((const void *)tmem_slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        // ------------------------------------------------ TMA producer
        if (lane == 0) {
            int issued = 0;
            for (int it = 0; it < nkt; ++it) {
                const int s = it % STAGES;
                const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
                if (!mbar_wait(&empty[s], ph ^ 1u, flags, abort_s)) break;
                uint8_t *st = stage_base + s * STAGE_BYTES;
                mbar_expect_tx(&full[s], STAGE_BYTES);
                const int x = (kt0 + it) * BK, y = mt * BM;
                tma_load_2d(st, &maps.a_hi, x, y, &full[s]);
                tma_load_2d(st + A_BYTES, &maps.a_lo, x, y, &full[s]);
                tma_load_2d(st + 2 * A_BYTES, &maps.w_hi, x, 0, &full[s]);
                tma_load_2d(st + 2 * A_BYTES + W_BYTES, &maps.w_lo, x, 0, &full[s]);
                ++issued;
            }
            // Drain: every issued stage's copy must land before the CTA exits.
            for (int it = (issued > STAGES ? issued - STAGES : 0); it < issued; ++it) {
                const int s = it % STAGES;
                const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
                unsigned long long t0 = gtimer();
                while (!mbar_try_wait(&full[s], ph) && gtimer() - t0 < WAIT_NS) {}
            }
        }
    } else if (warp == 1) {
        // ------------------------------------------------ MMA issuer
        if (lane == 0) {
            int it = 0;
            for (int c = 0; c < nchunks && !*abort_s; ++c) {
                const int buf = c & 1;
                const uint32_t use = (uint32_t)(c >> 1);
                if (!mbar_wait(&tempty[buf], (use & 1u) ^ 1u, flags, abort_s)) break;
                tc_fence_after();
                const uint32_t dtm = tmem + (uint32_t)(buf * BN);
                const int kend = min(nkt, (c + 1) * CHUNK_KT);
                bool ok = true;
                for (int first = 1; it < kend; ++it, first = 0) {
                    const int s = it % STAGES;
                    const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
                    if (!mbar_wait(&full[s], ph, flags, abort_s)) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t st = smem_u32(stage_base + s * STAGE_BYTES);
                    const uint32_t a_hi = st, a_lo = st + A_BYTES, w_hi = st + 2 * A_BYTES,
                                   w_lo = st + 2 * A_BYTES + W_BYTES;
#pragma unroll
                    for (int k = 0; k < BK / 16; ++k) {
                        const uint32_t off = (uint32_t)(k * 32);     // 16 elements x 2 B along K
                        const uint32_t acc = (first && k == 0) ? 0u : 1u;
                        umma(dtm, sdesc_sw128(a_hi + off), sdesc_sw128(w_hi + off), idesc, acc);
                        umma(dtm, sdesc_sw128(a_hi + off), sdesc_sw128(w_lo + off), idesc, 1u);
                        umma(dtm, sdesc_sw128(a_lo + off), sdesc_sw128(w_hi + off), idesc, 1u);
                    }
                    umma_commit(&empty[s]);                 // frees the stage when these MMAs finish
                }
                if (!ok) break;
                umma_commit(&tfull[buf]);                   // chunk accumulator ready
            }
            // Every MMA of this CTA must have finished before its TMEM is released.
            umma_commit(mma_done);
            const unsigned long long t0 = gtimer();
            while (!mbar_try_wait(mma_done, 0) && gtimer() - t0 < WAIT_NS) {}
        }
    } else {
        // ------------------------------------------------ epilogue (warps 2..5)
        const int q = warp & 3;                            // TMEM lane quadrant of this warp
        const int64_t row = (int64_t)mt * BM + q * 32 + lane;
        float hi[BN], lo[BN];
#pragma unroll
        for (int j = 0; j < BN; ++j) { hi[j] = 0.f; lo[j] = 0.f; }
        bool ok = true;
        for (int c = 0; c < nchunks; ++c) {
            const int buf = c & 1;
            const uint32_t use = (uint32_t)(c >> 1);
            if (!mbar_wait(&tfull[buf], use & 1u, flags, abort_s)) { ok = false; break; }
            tc_fence_after();
            const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * BN);
            float v[BN];
            tmem_ld16(taddr + 0, v);
            tmem_ld16(taddr + 16, v + 16);
            tmem_ld16(taddr + 32, v + 32);
            tmem_ld16(taddr + 48, v + 48);
            tmem_ld_wait();
            tc_fence_before();
            mbar_arrive(&tempty[buf]);
#pragma unroll
            for (int j = 0; j < BN; ++j) {                 // float-float accumulation (TwoSum)
                const float s = hi[j] + v[j];
                const float bb = s - hi[j];
                const float e = (hi[j] - (s - bb)) + (v[j] - bb);
                hi[j] = s;
                lo[j] += e;
            }
        }
        if (ok && row < rows && nchunks > 0) {
            if (out_scale_ptr) out_scale *= *out_scale_ptr;
            double *out = C + (int64_t)split * ldc_split + row;
#pragma unroll
            for (int j = 0; j < BN; ++j) out[(int64_t)j * ldc_col] = ((double)hi[j] + (double)lo[j]) * out_scale;
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    }
}

// ------------------------------------------------------------------------------------
// Exact-slice variant (three bf16 slices per operand).
// A[i][t] = (a0 + a1' + a2') * 2^pA[i][kt], W[j][t] = (w0 + w1' + w2') * 2^pW[j][kt] with
// a0, w0 integers of at most 8 bits and a1' = a1 2^-8, a2' = a2 2^-16 (a1, a2 integers of
// at most 8 bits), per node (or step) and 64-column k-tile. Per k-tile the products
//   X0  = sum a0 w0                                  (integers < 2^16, 64 of them < 2^22:
//                                                    exact in the FP32 accumulator)
//   X12 = sum a0 w1' + a1' w0 + a0 w2' + a1' w1' + a2' w0     (2^-8 below X0)
// go to two TMEM accumulators; the epilogue scales both by 2^(pA+pW) every k-tile and folds them
// into a float-float pair (hi, lo): X0 by an error-free TwoSum into hi, X12 (2^-8 of X0) added
// into lo together with that sum's rounding error. The leading product is therefore free of
// accumulation error, whatever the rounding of the tensor core's FP32 adder, and the FP32
// rounding of lo stays near 2^-31 of the partial per k-tile.
constexpr int THREADS3 = 64 + 8 * 32;                         // TMA warp, MMA warp, 8 epilogue warps

// Shape of the three-slice kernel for NG weight groups (64 steps each) per item: one MMA of
// N = 64 NG columns reads the item's history tile once for all NG groups, so the shared-memory
// traffic per group (TMA writes + MMA operand reads) falls with NG.
template <int NG>
struct Far3Cfg {
    static constexpr int N = BN * NG;                         // MMA N: steps per item
    static constexpr int WB = N * BK * 2;                     // one weight slice of a stage
    static constexpr int STAGE = 3 * A_BYTES + 3 * WB;        // 72 KB (NG 1), 96 KB (NG 2)
    static constexpr int STAGES = NG == 1 ? 3 : 2;
    static constexpr int TMEM = 4 * N;                        // 2 buffers x (X0, X12)
    static constexpr int SMEM = 1024 + STAGES * STAGE + 256;
    static constexpr int COLS = N / 2;                        // columns per epilogue warp
    static constexpr int CH = NG == 1 ? 32 : 4;               // columns per TMEM read batch
};

struct __align__(64) FarMaps3 {
    CUtensorMap a[3], w[3], w2[3];                            // w: 64-row weight boxes, w2: 128-row
};

// 2^e as a float for e in [-127, 127], from the bits (exact; e = -127 is the subnormal 2^-127).
__device__ __forceinline__ float pow2f(int e)
{
    return e >= -126 ? __int_as_float((e + 127) << 23) : __int_as_float(0x00400000);
}

// Persistent: gridDim.x CTAs (at most one per SM) walk the items (128-row tile mt, k-split ks,
// weight-group set gi of NG groups) = blockIdx.x, blockIdx.x + gridDim.x, ...; the TMA producer,
// the MMA issuer and the epilogue follow the same static sequence of k-tiles, so the pipeline runs
// on across item boundaries and TMEM is allocated once. Every item writes its partial (zeros if
// its k range is empty).
template <int NG>
__global__ void __launch_bounds__(THREADS3, 1)
    k_far_tc3(const __grid_constant__ FarMaps3 maps, double *__restrict__ C, int64_t ldc_split, int64_t ldc_col,
              int64_t rows, int kt_begin, int kt_total, int kt_per, int n_split, uint32_t idesc,
              const int8_t *__restrict__ pA, const float *__restrict__ pW, int64_t ldp, const int *__restrict__ wcol,
              int n_sets, int grp0, int64_t ldc_grp, unsigned *flags)
{
    using Cfg = Far3Cfg<NG>;
    constexpr int STAGES = Cfg::STAGES, STAGE_BYTES3 = Cfg::STAGE, N = Cfg::N, COLS = Cfg::COLS, CH = Cfg::CH;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *stage_base = smem;
    uint64_t *bars = (uint64_t *)(smem + STAGES * STAGE_BYTES3);
    uint64_t *full = bars, *empty = bars + STAGES, *tfull = bars + 2 * STAGES, *tempty = bars + 2 * STAGES + 2;
    uint64_t *mma_done = bars + 2 * STAGES + 4;
    volatile uint32_t *tmem_slot = (volatile uint32_t *)(bars + 2 * STAGES + 5);
    volatile int *abort_s = (volatile int *)(bars + 2 * STAGES + 6);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n_mt = (int)(rows / BM);
    const int n_items = n_mt * n_split * n_sets;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
        for (int b = 0; b < 2; ++b) { mbar_init(&tfull[b], 1); mbar_init(&tempty[b], 256); }
        mbar_init(mma_done, 1);
        *abort_s = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32((const void *)tmem_slot)),
                     "r"(Cfg::TMEM));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {                                   // TMA producer
            const CUtensorMap *wm = NG == 1 ? maps.w : maps.w2;
            int g = 0;
            bool ok = true;
            for (int item = blockIdx.x; item < n_items && ok; item += gridDim.x) {
                const int gi = item % n_sets, mk = item / n_sets;
                const int mt = mk / n_split, ks = mk % n_split;
                const int kt0 = kt_begin + ks * kt_per, kt1 = min(kt0 + kt_per, kt_total);
                for (int kt = kt0; kt < kt1; ++kt, ++g) {
                    const int s = g % STAGES;
                    const uint32_t ph = (uint32_t)(g / STAGES) & 1u;
                    if (!mbar_wait(&empty[s], ph ^ 1u, flags, abort_s)) { ok = false; break; }
                    uint8_t *st = stage_base + s * STAGE_BYTES3;
                    mbar_expect_tx(&full[s], STAGE_BYTES3);
                    const int x = kt * BK, y = mt * BM, yw = ((wcol ? wcol[mt] : 0) + grp0 + NG * gi) * BN;
#pragma unroll
                    for (int q = 0; q < 3; ++q) tma_load_2d(st + q * A_BYTES, &maps.a[q], x, y, &full[s]);
#pragma unroll
                    for (int q = 0; q < 3; ++q) tma_load_2d(st + 3 * A_BYTES + q * Cfg::WB, &wm[q], x, yw, &full[s]);
                }
            }
            for (int it = (g > STAGES ? g - STAGES : 0); it < g; ++it) {   // own copies in flight
                const int s = it % STAGES;
                const uint32_t ph = (uint32_t)(it / STAGES) & 1u;
                unsigned long long t0 = gtimer();
                while (!mbar_try_wait(&full[s], ph) && gtimer() - t0 < WAIT_NS) {}
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {                                   // MMA issuer: one k-tile per chunk
            int g = 0;
            bool ok = true;
            for (int item = blockIdx.x; item < n_items && ok; item += gridDim.x) {
                const int ks = (item / n_sets) % n_split;
                const int kt0 = kt_begin + ks * kt_per, kt1 = min(kt0 + kt_per, kt_total);
                for (int kt = kt0; kt < kt1 && !*abort_s; ++kt, ++g) {
                    const int buf = g & 1;
                    const uint32_t use = (uint32_t)(g >> 1);
                    if (!mbar_wait(&tempty[buf], (use & 1u) ^ 1u, flags, abort_s)) { ok = false; break; }
                    tc_fence_after();
                    const int s = g % STAGES;
                    const uint32_t ph = (uint32_t)(g / STAGES) & 1u;
                    if (!mbar_wait(&full[s], ph, flags, abort_s)) { ok = false; break; }
                    tc_fence_after();
                    const uint32_t x0 = tmem + (uint32_t)(buf * 2 * N), x12 = x0 + N;
                    const uint64_t dst = sdesc_sw128(smem_u32(stage_base + s * STAGE_BYTES3));
                    const uint32_t dlo = (uint32_t)dst, dhi = (uint32_t)(dst >> 32);
                    constexpr uint32_t A1 = A_BYTES >> 4, A2 = 2 * A_BYTES >> 4;
                    constexpr uint32_t W0 = 3 * A_BYTES >> 4, W1 = W0 + (Cfg::WB >> 4), W2 = W0 + (2 * Cfg::WB >> 4);
#pragma unroll
                    for (int k = 0; k < BK / 16; ++k) {
                        const uint32_t o = dlo + (uint32_t)(k * 2);      // +32 bytes per K=16 step
                        const uint32_t acc = k ? 1u : 0u;
                        umma_lo(x0, o, o + W0, dhi, idesc, acc);
                        umma_lo(x12, o, o + W1, dhi, idesc, acc);
                        umma_lo(x12, o + A1, o + W0, dhi, idesc, 1u);
                        umma_lo(x12, o, o + W2, dhi, idesc, 1u);
                        umma_lo(x12, o + A1, o + W1, dhi, idesc, 1u);
                        umma_lo(x12, o + A2, o + W0, dhi, idesc, 1u);
                    }
                    umma_commit(&empty[s]);
                    umma_commit(&tfull[buf]);
                }
            }
            umma_commit(mma_done);
            const unsigned long long t0 = gtimer();
            while (!mbar_try_wait(mma_done, 0) && gtimer() - t0 < WAIT_NS) {}
        }
    } else {
        // 8 epilogue warps: warp w reads TMEM lane quadrant w % 4 (the hardware's rule) and
        // folds columns [c0, c0 + COLS) with c0 = COLS * ((w - 2) / 4)
        const int q = warp & 3;
        const int c0 = COLS * ((warp - 2) >> 2);
        int g = 0;
        bool ok = true;
        for (int item = blockIdx.x; item < n_items && ok; item += gridDim.x) {
            const int gi = item % n_sets, mk = item / n_sets;
            const int mt = mk / n_split, ks = mk % n_split;
            const int kt0 = kt_begin + ks * kt_per, kt1 = min(kt0 + kt_per, kt_total);
            const int64_t row = (int64_t)mt * BM + q * 32 + lane;
            const int64_t row_c = row < rows ? row : rows - 1;
            // this lane's row exponents and its columns' (c0 + 32u + lane) weight-tile scales; the
            // next k-tile's set is loaded while the current one is folded (both miss L1 often:
            // shared memory takes most of it), and each column's scale reaches the warp by a shuffle
            constexpr int NU = COLS / 32;
            const int8_t *pAr = pA + row_c * ldp;
            const float *pWl = pW + ((int64_t)((wcol ? wcol[mt] : 0) + grp0 + NG * gi) * BN + c0 + lane) * ldp;
            int e_nx = kt0 < kt1 ? (int)pAr[kt0] : 0;
            float w_nx[NU];
#pragma unroll
            for (int u = 0; u < NU; ++u) w_nx[u] = kt0 < kt1 ? __ldg(pWl + (int64_t)32 * u * ldp + kt0) : 0.f;
            float hi[COLS], lo[COLS];
#pragma unroll
            for (int j = 0; j < COLS; ++j) { hi[j] = 0.f; lo[j] = 0.f; }
            for (int kt = kt0; kt < kt1; ++kt, ++g) {
                const int buf = g & 1;
                const uint32_t use = (uint32_t)(g >> 1);
                const int e_cur = e_nx;
                float w_cur[NU];
#pragma unroll
                for (int u = 0; u < NU; ++u) w_cur[u] = w_nx[u];
                if (kt + 1 < kt1) {
                    e_nx = (int)pAr[kt + 1];
#pragma unroll
                    for (int u = 0; u < NU; ++u) w_nx[u] = __ldg(pWl + (int64_t)32 * u * ldp + kt + 1);
                }
                if (!mbar_wait(&tfull[buf], use & 1u, flags, abort_s)) { ok = false; break; }
                tc_fence_after();
                // 2^pA * 2^pW: a product of powers of two, exact while it stays normal
                const float sa = pow2f(e_cur);
                const uint32_t tb = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * 2 * N + c0);
#pragma unroll
                for (int h = 0; h < COLS / CH; ++h) {
                    // a batch of CH columns of both accumulators in flight before one wait
                    float v0[CH], v1[CH];
                    if constexpr (CH == 4) {
                        tmem_ld4(tb + CH * h, v0);
                        tmem_ld4(tb + N + CH * h, v1);
                    } else {
#pragma unroll
                        for (int b = 0; b < CH / 16; ++b) {
                            tmem_ld16(tb + CH * h + 16 * b, v0 + 16 * b);
                            tmem_ld16(tb + N + CH * h + 16 * b, v1 + 16 * b);
                        }
                    }
                    tmem_ld_wait();
#pragma unroll
                    for (int jj = 0; jj < CH; ++jj) {
                        const int j = CH * h + jj;
                        const float sc = sa * __shfl_sync(0xffffffffu, w_cur[j >> 5], j & 31);
                        // X0 (exact integer sum) enters hi by TwoSum; X12, 2^-8 of it, goes straight
                        // into lo with the rounding error (FP32 rounding of lo is ~2^-31 of hi per
                        // k-tile)
                        const float x = v0[jj] * sc;           // exact (power-of-two scaling)
                        const float s = hi[j] + x, bb = s - hi[j];
                        const float e = (hi[j] - (s - bb)) + (x - bb);
                        hi[j] = s;
                        lo[j] = fmaf(v1[jj], sc, lo[j] + e);
                    }
                }
                tc_fence_before();
                mbar_arrive(&tempty[buf]);
            }
            if (ok && row < rows) {                   // float pairs: no FP64 work here
                // column c of the item is step c % 64 of group NG gi + c / 64, i.e. at
                // C + (NG gi) ldc_grp + c ldc_col (ldc_grp = 64 ldc_col)
                float2 *out = reinterpret_cast<float2 *>(C + (int64_t)ks * ldc_split + (int64_t)NG * gi * ldc_grp + row) +
                              (int64_t)c0 * ldc_col;
#pragma unroll
                for (int j = 0; j < COLS; ++j) out[(int64_t)j * ldc_col] = make_float2(hi[j], lo[j]);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(Cfg::TMEM));
    }
}

// ---------------------------------------------------------------- host side

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn()
{
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    }
    return fn;
}

// 2D tensor map over a row-major [rows][cols] array of 16-bit values, box 64 cols x box_rows.
static int make_map(CUtensorMap *tm, const void *base, int64_t rows, int64_t cols, int box_rows)
{
    EncodeTiledFn enc = encode_fn();
    if (!enc) return set_error(FPDE_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available");
    if ((cols * 2) % 16 != 0 || ((uintptr_t)base % 16) != 0)
        return set_error(FPDE_ERR_ARG, "tensor map: row pitch and base must be 16-byte aligned");
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)(cols * 2)};
    cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = enc(tm, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, const_cast<void *>(base), dims, strides, box, es,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(FPDE_ERR_ARG, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return FPDE_OK;
}

}  // namespace tc

int far_plan_init(FarPlan *p, const void *a_hi, const void *a_lo, int64_t rows, int64_t lda, const void *w_hi,
                  const void *w_lo, int64_t ldw, int bf16)
{
    if (rows % tc::BM != 0 || lda % tc::BK != 0 || ldw % tc::BK != 0)
        return set_error(FPDE_ERR_ARG, "far contraction: rows must be a multiple of 128, pitches of 64");
    static_assert(sizeof(tc::FarMaps) <= sizeof(p->maps), "map storage");
    tc::FarMaps *m = (tc::FarMaps *)p->maps;
    int rc;
    if ((rc = tc::make_map(&m->a_hi, a_hi, rows, lda, tc::BM)) || (rc = tc::make_map(&m->a_lo, a_lo, rows, lda, tc::BM)) ||
        (rc = tc::make_map(&m->w_hi, w_hi, tc::BN, ldw, tc::BN)) || (rc = tc::make_map(&m->w_lo, w_lo, tc::BN, ldw, tc::BN)))
        return rc;
    p->rows = rows;
    p->idesc = tc::idesc_f16(bf16 ? 1 : 0, tc::BM, tc::BN);
    cudaError_t e = smem_opt_in((const void *)tc::k_far_tc, tc::SMEM_BYTES);
    if (e != cudaSuccess) return set_error(FPDE_ERR_CUDA, "far kernel smem attribute: %s", cudaGetErrorString(e));
    return FPDE_OK;
}

int far_plan3_init(FarPlan3 *p, const void *const a[3], int64_t rows, int64_t lda, const void *const w[3],
                   int64_t ldw, int w_tiles)
{
    if (rows % tc::BM != 0 || lda % tc::BK != 0 || ldw % tc::BK != 0)
        return set_error(FPDE_ERR_ARG, "far contraction: rows must be a multiple of 128, pitches of 64");
    static_assert(sizeof(tc::FarMaps3) <= sizeof(p->maps), "map storage");
    tc::FarMaps3 *m = (tc::FarMaps3 *)p->maps;
    int rc;
    const int64_t w_rows = (int64_t)tc::BN * (w_tiles > 0 ? w_tiles : 1);
    for (int q = 0; q < 3; ++q) {
        if ((rc = tc::make_map(&m->a[q], a[q], rows, lda, tc::BM))) return rc;
        if ((rc = tc::make_map(&m->w[q], w[q], w_rows, ldw, tc::BN))) return rc;
        // 128-row weight boxes (two groups per item) exist only when the slices hold two tiles
        if (w_rows >= 2 * tc::BN) {
            if ((rc = tc::make_map(&m->w2[q], w[q], w_rows, ldw, 2 * tc::BN))) return rc;
        } else {
            m->w2[q] = m->w[q];
        }
    }
    p->rows = rows;
    p->w_rows = w_rows;
    p->idesc = tc::idesc_f16(1, tc::BM, tc::BN);
    p->idesc2 = tc::idesc_f16(1, tc::BM, 2 * tc::BN);
    cudaError_t e = smem_opt_in((const void *)tc::k_far_tc3<1>, tc::Far3Cfg<1>::SMEM);
    if (e == cudaSuccess) e = smem_opt_in((const void *)tc::k_far_tc3<2>, tc::Far3Cfg<2>::SMEM);
    if (e != cudaSuccess) return set_error(FPDE_ERR_CUDA, "far kernel smem attribute: %s", cudaGetErrorString(e));
    return FPDE_OK;
}

int far3_launch(cudaStream_t st, const FarPlan3 *p, int k_cols, double *C, int64_t ldc_split, int64_t ldc_col,
                int splits, const int8_t *pA, const float *pW, int64_t ldp, unsigned *flags, const int *wcol,
                int k_begin, int n_grp, int grp0)
{
    if (n_grp < 1 || grp0 < 0 || (int64_t)(grp0 + n_grp) * tc::BN > p->w_rows)
        return set_error(FPDE_ERR_ARG, "far contraction: weight rows out of range");
    if (k_cols % tc::BK != 0 || k_begin % tc::BK != 0 || k_begin < 0 || k_begin > k_cols)
        return set_error(FPDE_ERR_ARG, "far contraction: K range must be in multiples of 64");
    if (k_cols == k_begin) return FPDE_OK;
    const int kt_total = k_cols / tc::BK, kt_begin = k_begin / tc::BK;
    if (splits < 1) splits = 1;
    if (splits > FAR_MAX_SPLITS) splits = FAR_MAX_SPLITS;
    const int kt_per = (kt_total - kt_begin + splits - 1) / splits;   // every split is written, possibly with zeros
    // Two weight groups per item (one N = 128 MMA reads the history tile once for both) when the
    // groups pair up; the item sets of one (row tile, split) are consecutive items, and a grid that
    // is a multiple of their count keeps them on neighbouring CTAs for the whole walk, so the
    // history tiles they share stream from HBM once and are re-read from L2.
    const int ng = (n_grp % 2 == 0) ? 2 : 1;
    const int n_sets = n_grp / ng;
    const int64_t items = (p->rows / tc::BM) * splits * n_sets;
    const int sms = device_sm_count();
    int64_t grid = std::min<int64_t>(items, sms);
    if (grid > n_sets) grid -= grid % n_sets;
    const tc::FarMaps3 *m = (const tc::FarMaps3 *)p->maps;
    const int64_t ldc_grp = (int64_t)tc::BN * ldc_col;
    if (ng == 2)
        tc::k_far_tc3<2><<<(unsigned)grid, tc::THREADS3, tc::Far3Cfg<2>::SMEM, st>>>(
            *m, C, ldc_split, ldc_col, p->rows, kt_begin, kt_total, kt_per, splits, p->idesc2, pA, pW, ldp, wcol,
            n_sets, grp0, ldc_grp, flags);
    else
        tc::k_far_tc3<1><<<(unsigned)grid, tc::THREADS3, tc::Far3Cfg<1>::SMEM, st>>>(
            *m, C, ldc_split, ldc_col, p->rows, kt_begin, kt_total, kt_per, splits, p->idesc, pA, pW, ldp, wcol,
            n_sets, grp0, ldc_grp, flags);
    FPDE_LAUNCHED(1);
    return FPDE_OK;
}

int far_splits(int kt_total, int64_t rows)
{
    // Splits of K only for balance of the persistent grid (one CTA per SM): the fewest splits
    // whose items fill the SMs within 5% (each split keeps at least 2 k-tiles).
    const int sms = device_sm_count();
    const int64_t tiles = rows / tc::BM;
    int best = 1;
    double best_waste = 1e30;
    for (int s = 1; s <= FAR_MAX_SPLITS && (s == 1 || kt_total / s >= 2); ++s) {
        const int64_t items = tiles * s;
        const double waves = (double)items / sms, full = (double)((items + sms - 1) / sms);
        const double waste = full / waves;
        if (waste < best_waste - 1e-9) { best_waste = waste; best = s; }
        if (waste <= 1.05) break;
    }
    return best;
}

int far_launch(cudaStream_t st, const FarPlan *p, int k_cols, double *C, int64_t ldc_split, int64_t ldc_col,
               int splits, double out_scale, const double *out_scale_ptr, unsigned *flags)
{
    if (k_cols % tc::BK != 0) return set_error(FPDE_ERR_ARG, "far contraction: K must be a multiple of 64");
    if (k_cols == 0) return FPDE_OK;
    const int kt_total = k_cols / tc::BK;
    if (splits < 1) splits = 1;
    if (splits > FAR_MAX_SPLITS) splits = FAR_MAX_SPLITS;
    const int kt_per = (kt_total + splits - 1) / splits;
    splits = (kt_total + kt_per - 1) / kt_per;
    dim3 grid((unsigned)(p->rows / tc::BM), (unsigned)splits);
    const tc::FarMaps *m = (const tc::FarMaps *)p->maps;
    tc::k_far_tc<<<grid, tc::THREADS, tc::SMEM_BYTES, st>>>(*m, C, ldc_split, ldc_col, p->rows, kt_total, kt_per,
                                                           p->idesc, out_scale, out_scale_ptr, flags);
    FPDE_LAUNCHED(1);
    return FPDE_OK;
}

}  // namespace fpde

using namespace fpde;

extern "C" int fpde_far_contract(fpde_ctx *ctx, const void *a_hi, const void *a_lo, int64_t rows, int64_t lda,
                                 const void *w_hi, const void *w_lo, int64_t ldw, int k_cols, int bf16,
                                 double out_scale, double *C, int splits)
{
    clear_error();
    int rc = ctx_enter(ctx);
    if (rc) return rc;
    FPDE_CHECK_ARG(a_hi && a_lo && w_hi && w_lo && C && rows > 0 && k_cols >= 0, "bad arguments");
    FPDE_CHECK_ARG(k_cols <= lda && k_cols <= ldw, "K beyond the operand pitch");
    FarPlan plan;
    if ((rc = far_plan_init(&plan, a_hi, a_lo, rows, lda, w_hi, w_lo, ldw, bf16))) return rc;
    const int kt_total = k_cols / 64;
    if (splits <= 0) splits = far_splits(kt_total, rows);
    if ((rc = far_launch(ctx->stream, &plan, k_cols, C, rows * 64, rows, splits, out_scale, nullptr, ctx->d_flags)))
        return rc;
    FPDE_CUDA(cudaStreamSynchronize(ctx->stream));
    return ctx_check_flags(ctx, "far contraction");
}

namespace fpde {
// Weight-tile exponents -> their scales 2^e (the far kernel takes the scales).
__global__ void k_exp_to_scale(const int8_t *e, float *s, int64_t n)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) s[i] = tc::pow2f((int)e[i]);
}
// In place: float-pair slots of a far contraction -> FP64 values.
__global__ void k_ff_to_double(double *C, int64_t n)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) C[i] = ff_to_double(C[i]);
}
}  // namespace fpde

extern "C" int fpde_far_contract3(fpde_ctx *ctx, const void *const a[3], int64_t rows, int64_t lda,
                                  const void *const w[3], int64_t ldw, int k_cols, const int8_t *pA,
                                  const int8_t *pW, int64_t ldp, double *C, int splits)
{
    clear_error();
    int rc = ctx_enter(ctx);
    if (rc) return rc;
    FPDE_CHECK_ARG(a && w && a[0] && a[1] && a[2] && w[0] && w[1] && w[2] && pA && pW && C, "null argument");
    FPDE_CHECK_ARG(rows > 0 && k_cols >= 0 && k_cols <= lda && k_cols <= ldw && ldp * 64 >= k_cols, "bad shape");
    FarPlan3 plan;
    if ((rc = far_plan3_init(&plan, a, rows, lda, w, ldw))) return rc;
    if (splits <= 0) splits = far_splits(k_cols / 64, rows);
    if (splits > FAR_MAX_SPLITS) splits = FAR_MAX_SPLITS;
    float *pWs = nullptr;
    const int64_t nw = 64 * ldp;
    if (dev_alloc((void **)&pWs, (size_t)nw * sizeof(float))) return FPDE_ERR_NOMEM;
    k_exp_to_scale<<<(unsigned)((nw + 255) / 256), 256, 0, ctx->stream>>>(pW, pWs, nw);
    FPDE_LAUNCHED(1);
    rc = far3_launch(ctx->stream, &plan, k_cols, C, rows * 64, rows, splits, pA, pWs, ldp, ctx->d_flags);
    if (rc) {
        cudaStreamSynchronize(ctx->stream);
        dev_free(pWs);
        return rc;
    }
    const int64_t n = (int64_t)splits * 64 * rows;
    if (k_cols > 0) {
        k_ff_to_double<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(C, n);
        FPDE_LAUNCHED(1);
    }
    FPDE_CUDA(cudaStreamSynchronize(ctx->stream));
    dev_free(pWs);
    return ctx_check_flags(ctx, "far contraction (three slices)");
}
