/* Stand-in for <fftw3.h> used when compiling the reference's host setup files
 * (they include the header but call no FFTW routine). */
#ifndef TCSEM_FFTW3_SHIM_H
#define TCSEM_FFTW3_SHIM_H
#include <stdlib.h>
typedef double fftw_complex[2];
typedef void *fftw_plan;
static inline void *fftw_malloc(size_t n) { return malloc(n); }
static inline void fftw_free(void *p) { free(p); }
#endif
