// Closures of the reference's Richards problem (fpde_hpc_1d.cpp, analytic_test 0 with the van
// Genuchten-Mualem water content of cv_form 4): water content wetness :2493-2522, the inverse
// of its derivative inv_dw_dh :2523-2566 and the relative conductivity of KK :2625-2655
// (k_form 1 van Genuchten-Mualem, 2 Averianov), as functions of the suction P in metres. The
// soil constants are the reference's. The expressions keep its operation order; they are
// evaluated with CUDA's pow, so values agree with the host's to a few ulps.
#pragma once

namespace fpde {

constexpr double RICH_N = 1.25, RICH_S0 = 0.0736, RICH_S1 = 0.55, RICH_A = 0.066;
constexpr double RICH_SATURATED = 1e20;          // inv_dw_dh where the soil is saturated

__device__ __forceinline__ double rich_wetness(double P)
{
    const double n = RICH_N, s0 = RICH_S0, s1 = RICH_S1, a = RICH_A;
    P *= 100.0;                                   // centimetres
    if (P <= 0.0) return s1;
    return s0 + ((s1 - s0) / pow(1 + pow(a * P, n), (1 - 1 / n)));
}

__device__ __forceinline__ double rich_inv_dw_dh(double P)
{
    const double n = RICH_N, s0 = RICH_S0, s1 = RICH_S1, a = RICH_A;
    if (P <= 0.0) return RICH_SATURATED;
    const double hn = pow(100.0, n), h2n = pow(100.0, 2.0 * n);
    const double apn = pow(a * P, n);
    const double Ch = ((((1 - n) * hn * s0 + (n - 1) * hn * s1) * apn * pow(1 + hn * apn, (1 / n))) /
                       (h2n * P * pow(a * P, 2 * n) + 2 * hn * P * apn + P));
    return Ch != 0.0 ? 1.0 / Ch : RICH_SATURATED;
}

// KK = Kr(wetness) * k_sat
__device__ __forceinline__ double rich_KK(double P, int kform, double ksat)
{
    const double n = RICH_N, s0 = RICH_S0, s1 = RICH_S1;
    const double x = (rich_wetness(P) - s0) / (s1 - s0);
    double Kr = 1.0;
    if (kform == 1) Kr = pow(x, 0.5) * pow(1.0 - pow(1.0 - pow(x, (1.0 / (1.0 - 1.0 / n))), (1.0 - 1.0 / n)), 2.0);
    if (kform == 2) Kr = pow(x, 3.5);
    return Kr * ksat;
}

}  // namespace fpde
