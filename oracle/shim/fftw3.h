/*
 * fftw3.h (shim) -- lets the reference's filter sources compile without FFTW.
 *
 * Oracle build only: declares the handful of FFTW3 entry points that
 * filter/main.c:58-59, filter/filter.c:22-23 and filter/hamiltonian.c:33-41
 * use, with FFTW's conventions (interleaved complex128, dims slowest-first,
 * FFTW_FORWARD = -1, unnormalised).  fftw_shim.c implements them on the
 * oracle's own Stockham FFT (fft_cpu.c).
 */
#ifndef SEP_SHIM_FFTW3_H
#define SEP_SHIM_FFTW3_H
#include <stddef.h>

typedef double fftw_complex[2];
typedef struct sep_shim_fftw_plan_s *fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in, fftw_complex *out,
                           int sign, unsigned flags);
void fftw_execute(const fftw_plan plan);
void fftw_destroy_plan(fftw_plan plan);
void *fftw_malloc(size_t n);
void fftw_free(void *p);

#endif
