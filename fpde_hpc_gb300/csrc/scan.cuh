// Warp-level scans of first-order affine recurrences x_i = P_i x_{i-1} + X_i, kept as
// (product, value) pairs: composing segment (P1, X1) then (P2, X2) gives (P2 P1, P2 X1 + X2).
#pragma once
#include <cuda_runtime.h>

namespace fpde {

constexpr unsigned FULL = 0xffffffffu;

// Inclusive scan towards higher lanes: lane l ends with the composition of lanes 0..l.
__device__ __forceinline__ void warp_scan_up(double &P, double &X, int lane)
{
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        double Pp = __shfl_up_sync(FULL, P, off), Xp = __shfl_up_sync(FULL, X, off);
        if (lane >= off) { X = fma(P, Xp, X); P = P * Pp; }
    }
}
// Inclusive scan towards lower lanes: lane l ends with the composition of lanes 31..l.
__device__ __forceinline__ void warp_scan_down(double &P, double &X, int lane)
{
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        double Pn = __shfl_down_sync(FULL, P, off), Xn = __shfl_down_sync(FULL, X, off);
        if (lane + off < 32) { X = fma(P, Xn, X); P = P * Pn; }
    }
}

__device__ __forceinline__ unsigned long long gtimer_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

}  // namespace fpde
