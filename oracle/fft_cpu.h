/*
 * fft_cpu.h -- CPU 3-D complex FFT used by the oracle (test infrastructure only).
 *
 * The reference links FFTW3 (filter/Makefile:4-5) and plans its transforms with
 * fftw_plan_dft_3d(nz, ny, nx, ...) on interleaved complex128, x fastest
 * (filter/main.c:58-59, filter/init.c:139-141).  FFTW is not installed here, so
 * the oracle carries its own transform with the same conventions:
 *   forward  (sign = -1): X[k] = sum_j x[j] exp(-2 pi i j k / n), per axis
 *   backward (sign = +1): X[k] = sum_j x[j] exp(+2 pi i j k / n), unnormalised
 * Algorithm: mixed-radix Stockham autosort (radix 4, 2 and odd primes), applied
 * to panels of W adjacent lines so that the inner loops run over contiguous
 * memory.  Supported lengths: any n >= 1 (prime factors > 7 use an O(r^2)
 * butterfly).
 */
#ifndef ORC_FFT_CPU_H
#define ORC_FFT_CPU_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_fft3 orc_fft3;

/* dims in FFTW order: slowest (z) first, fastest (x) last. */
orc_fft3 *orc_fft3_create(long nz, long ny, long nx);
/* In-place transform of nz*ny*nx interleaved complex doubles. sign = -1 or +1.
 * Thread-safe: a plan may be executed concurrently on different buffers. */
void orc_fft3_exec(const orc_fft3 *plan, double *data, int sign);
void orc_fft3_destroy(orc_fft3 *plan);

#ifdef __cplusplus
}
#endif

#endif
