/*
 * fftw_shim.c -- oracle build only: the FFTW3 subset declared in shim/fftw3.h,
 * implemented on the oracle's Stockham FFT.  Plans remember their buffer as
 * FFTW's do; execution is in place (the reference only plans in-place
 * transforms: filter/main.c:58-59, filter/filter.c:22-23).
 */
#include <stdlib.h>
#include <string.h>

#include "../fft_cpu.h"
#include "fftw3.h"

struct sep_shim_fftw_plan_s {
  orc_fft3 *fft;
  fftw_complex *in, *out;
  size_t n;
  int sign;
};

fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in, fftw_complex *out,
                           int sign, unsigned flags) {
  (void)flags;
  fftw_plan p = (fftw_plan)calloc(1, sizeof(*p));
  if (!p) return NULL;
  p->fft = orc_fft3_create(n0, n1, n2);
  p->in = in;
  p->out = out;
  p->n = (size_t)n0 * (size_t)n1 * (size_t)n2;
  p->sign = sign;
  return p;
}

void fftw_execute(const fftw_plan p) {
  if (p->in != p->out) memcpy(p->out, p->in, p->n * sizeof(fftw_complex));
  orc_fft3_exec(p->fft, &p->out[0][0], p->sign);
}

void fftw_destroy_plan(fftw_plan p) {
  if (!p) return;
  orc_fft3_destroy(p->fft);
  free(p);
}

void *fftw_malloc(size_t n) {
  void *q = NULL;
  if (posix_memalign(&q, 64, n ? n : 64) != 0) return NULL;
  return q;
}

void fftw_free(void *q) { free(q); }
