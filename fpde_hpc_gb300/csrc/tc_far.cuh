// Far-history tensor-core contraction (tc_far.cu): plan and launch helpers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fpde {

constexpr int FAR_MAX_SPLITS = 4;   // K splits (FP64 partial slices) per contraction
constexpr int FAR_MAX_SUPER = 4;    // 64-step weight groups per far super-block

struct FarPlan {
    alignas(64) unsigned char maps[4 * 128];   // four CUtensorMap (a_hi, a_lo, w_hi, w_lo)
    int64_t rows = 0;
    uint32_t idesc = 0;
};

// a_hi/a_lo: [rows][lda] 16-bit (rows % 128 == 0, lda % 64 == 0); w_hi/w_lo: [64][ldw].
int far_plan_init(FarPlan *p, const void *a_hi, const void *a_lo, int64_t rows, int64_t lda, const void *w_hi,
                  const void *w_lo, int64_t ldw, int bf16);
// C[split*ldc_split + j*ldc_col + row] = out_scale * sum over the split's K range.
// out_scale_ptr (device, may be null) multiplies out_scale at run time.
int far_launch(cudaStream_t st, const FarPlan *p, int k_cols, double *C, int64_t ldc_split, int64_t ldc_col,
               int splits, double out_scale, const double *out_scale_ptr, unsigned *flags);
int far_splits(int kt_total, int64_t rows);

// Exact-slice variant: three bf16 slices per operand, per-(row, k-tile) exponents pA
// ([rows][ldp] int8) and per-(j, k-tile) scales pW = 2^e ([64][ldp] float: the epilogue
// multiplies by them without rebuilding each power of two).
struct FarPlan3 {
    alignas(64) unsigned char maps[9 * 128];
    int64_t rows = 0;
    int64_t w_rows = 0;                        // rows of the W slices (64 per weight tile)
    uint32_t idesc = 0, idesc2 = 0;            // MMA instruction descriptors for N = 64 and 128
};
// w_tiles: number of 64-row weight tiles in the W slices (columns of an ensemble; 1 otherwise).
int far_plan3_init(FarPlan3 *p, const void *const a[3], int64_t rows, int64_t lda, const void *const w[3],
                   int64_t ldw, int w_tiles = 1);
// Writes each partial as a float pair (hi, lo) into the 8-byte slot of C (the fold's float-
// float value; hi + lo is exact in FP64): read it with ff_to_double.
// wcol (device, may be null): per 128-row tile the weight tile (column of an ensemble) it uses,
// whose 64 rows start at row wcol[tile] * 64 of the W slices and of pW.
// k_begin (a multiple of 64): the contraction covers history columns [k_begin, k_cols) only
// (a restricted history window); the splits divide that range.
// n_grp, grp0: every row tile is contracted against the n_grp weight tiles grp0 .. grp0+n_grp-1
// (64 steps each, W rows (grp0+g)*64 ..; plus wcol's tile) and writes group g's 64 steps at
// C + g*64*ldc_col: one launch covers n_grp*64 upcoming steps (a super-block).
int far3_launch(cudaStream_t st, const FarPlan3 *p, int k_cols, double *C, int64_t ldc_split, int64_t ldc_col,
                int splits, const int8_t *pA, const float *pW, int64_t ldp, unsigned *flags,
                const int *wcol = nullptr, int k_begin = 0, int n_grp = 1, int grp0 = 0);

// float -> double from the bits (integer instructions only; exact for every float).
__device__ __forceinline__ double f2d_bits(float x)
{
    const uint32_t b = (uint32_t)__float_as_int(x);
    const uint64_t sign = (uint64_t)(b >> 31) << 63;
    const uint32_t e = (b >> 23) & 0xFFu, m = b & 0x7FFFFFu;
    uint64_t r;
    if (e == 0) {
        if (m == 0) {
            r = sign;
        } else {                                        // subnormal: m * 2^-149
            const int k = 31 - __clz((int)m);           // highest set bit, 0..22
            r = sign | ((uint64_t)(k - 149 + 1023) << 52) | (((uint64_t)m << (52 - k)) & 0xFFFFFFFFFFFFFull);
        }
    } else if (e == 0xFFu) {
        r = sign | (0x7FFull << 52) | ((uint64_t)m << 29);
    } else {
        r = sign | ((uint64_t)(e - 127 + 1023) << 52) | ((uint64_t)m << 29);
    }
    return __longlong_as_double((long long)r);
}
// A far-contraction slot (float pair) as one double: hi + lo, exact.
__device__ __forceinline__ double ff_to_double(double slot)
{
    const float2 v = *reinterpret_cast<const float2 *>(&slot);
    return f2d_bits(v.x) + f2d_bits(v.y);
}

}  // namespace fpde
