// Far-history tensor-core contraction (tc_far.cu): plan and launch helpers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fpde {

constexpr int FAR_MAX_SPLITS = 4;   // K splits (FP64 partial slices) per contraction

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
// ([rows][ldp] int8) and per-(j, k-tile) exponents pW ([64][ldp] int8).
struct FarPlan3 {
    alignas(64) unsigned char maps[6 * 128];
    int64_t rows = 0;
    uint32_t idesc = 0;
};
int far_plan3_init(FarPlan3 *p, const void *const a[3], int64_t rows, int64_t lda, const void *const w[3],
                   int64_t ldw);
int far3_launch(cudaStream_t st, const FarPlan3 *p, int k_cols, double *C, int64_t ldc_split, int64_t ldc_col,
                int splits, const int8_t *pA, const int8_t *pW, int64_t ldp, unsigned *flags);

}  // namespace fpde
