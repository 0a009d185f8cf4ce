/* Empty stand-in for libfftpack ls_fft.h (see fftpack.h). */
