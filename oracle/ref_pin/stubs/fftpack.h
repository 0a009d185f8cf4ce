/* Stand-in for libfftpack's fftpack.h, which the reference includes but which is not
 * present in this image. The reference reaches these only through its FFT Toeplitz
 * product (space-fractional path, TMA 1), which no pinned scenario uses: every entry
 * aborts so an accidental call cannot go unnoticed. Test infrastructure only. */
#ifndef FPDE_PIN_FFTPACK_STUB_H
#define FPDE_PIN_FFTPACK_STUB_H
#include <stdio.h>
#include <stdlib.h>
typedef void *real_plan;
static inline real_plan make_real_plan(size_t n) { (void)n; fprintf(stderr, "fftpack stub called\n"); abort(); return 0; }
static inline void kill_real_plan(real_plan p) { (void)p; abort(); }
static inline void real_plan_forward_c(real_plan p, double *v) { (void)p; (void)v; abort(); }
static inline void real_plan_backward_c(real_plan p, double *v) { (void)p; (void)v; abort(); }
#endif
