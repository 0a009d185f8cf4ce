// Declarations shared between the translation units of libfpde_gb300.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace fpde {

constexpr int KS_MAX = 64;   // maximum number of row splits of the FP64 history sum

double l1_interval_weight(double alpha, double a, double d);
double l1_lag(double alpha, int64_t j);

// part[ks][i] = sum over the rows of split ks of wt[t] * D[t][i] (P doubles per row, P even).
int launch_l1_partial(cudaStream_t st, const double *D, int64_t P, int n, const double *wt,
                      double *part, int KS);
int choose_splits(int n, int64_t P);

}  // namespace fpde
