/* Empty stand-in for libfftpack bluestein.h (see fftpack.h). */
