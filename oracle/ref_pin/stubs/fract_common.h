/* Stand-in for fract_common.h, which fr_do.cpp includes but which the reference does
 * not ship. fr_do.cpp needs two host functions from it:
 *   Gamma(x)      -- the Gamma function; here the C library's tgamma. The oracle and the
 *                    GPU path receive the same Gamma values as inputs, so the pin does
 *                    not depend on which Gamma implementation the original header had.
 *   bk(d1,d2,b)   -- d1^(1-b) - d2^(1-b) with the zero-argument cases, the host twin of
 *                    the device function in fr_do.cpp:129-134.
 * Test infrastructure only. */
#ifndef FPDE_PIN_FRACT_COMMON_H
#define FPDE_PIN_FRACT_COMMON_H
#include <math.h>
static inline double Gamma(double x) { return tgamma(x); }
static inline double bk(double d1, double d2, double beta)
{
    if (d1 == 0.0) return pow(d2, 1.0 - beta);
    if (d2 == 0.0) return pow(d1, 1.0 - beta);
    return pow(d1, 1.0 - beta) - pow(d2, 1.0 - beta);
}
#endif
