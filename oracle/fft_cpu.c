/*
 * fft_cpu.c -- mixed-radix Stockham autosort FFT for the oracle (CPU only).
 *
 * Test infrastructure: only the oracle, the tests and the CPU baseline use it.
 *
 * One axis of length n is factored into radices r_0 r_1 ... (4 first, then 2,
 * then odd primes).  Stage s with radix r and span Ns (product of the radices
 * already applied) maps, for every j in [0, n/r):
 *     v_q = x[j + q n/r] * w^(q k),  k = j mod Ns,  w = exp(sign 2 pi i/(Ns r))
 *     y[(j/Ns) Ns r + k + p Ns] = sum_q v_q exp(sign 2 pi i p q / r)
 * which leaves the result in natural order after the last stage (Stockham
 * autosort; see e.g. Govindaraju et al., "High Performance Discrete Fourier
 * Transforms on Graphics Processors", SC'08, section 3).
 *
 * Each butterfly acts on a "panel": W adjacent lines held as split real/imag
 * arrays [n][W], so every inner loop is a contiguous length-W loop that the
 * compiler vectorises.
 */
#include "fft_cpu.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define PANEL_W 16
#define MAX_FACTORS 40

typedef struct {
  long n;
  int nstage;
  int radix[MAX_FACTORS];
  long span[MAX_FACTORS];   /* Ns before the stage */
  double *tw_re[MAX_FACTORS]; /* [Ns][r-1], forward sign */
  double *tw_im[MAX_FACTORS];
  /* cos/sin(2 pi p q / r) for the odd-radix butterflies: [r][r] */
  double *rc[MAX_FACTORS];
  double *rs[MAX_FACTORS];
} axis_plan;

struct orc_fft3 {
  long n[3]; /* z, y, x */
  axis_plan ax[3];
};

/* cos and sin of 2 pi t / m, evaluated in long double and rounded once. */
static void unit_root(long t, long m, double *c, double *s) {
  t %= m;
  if (t < 0) t += m;
  /* exact values at the quarter points keep the butterflies symmetric */
  if (t == 0) { *c = 1.0; *s = 0.0; return; }
  if (2 * t == m) { *c = -1.0; *s = 0.0; return; }
  if (4 * t == m) { *c = 0.0; *s = 1.0; return; }
  if (4 * t == 3 * m) { *c = 0.0; *s = -1.0; return; }
  const long double two_pi = 6.283185307179586476925286766559005768L;
  long double a = two_pi * (long double)t / (long double)m;
  *c = (double)cosl(a);
  *s = (double)sinl(a);
}

static int factorize(long n, int *radix) {
  int nf = 0;
  while (n % 4 == 0 && n > 1) { radix[nf++] = 4; n /= 4; }
  while (n % 2 == 0) { radix[nf++] = 2; n /= 2; }
  for (long p = 3; n > 1; p += 2) {
    while (n % p == 0) { radix[nf++] = (int)p; n /= p; }
  }
  return nf;
}

static void axis_init(axis_plan *a, long n) {
  memset(a, 0, sizeof(*a));
  a->n = n;
  a->nstage = (n > 1) ? factorize(n, a->radix) : 0;
  long Ns = 1;
  for (int s = 0; s < a->nstage; s++) {
    int r = a->radix[s];
    a->span[s] = Ns;
    a->tw_re[s] = (double *)malloc(sizeof(double) * (size_t)Ns * (size_t)(r - 1) + 8);
    a->tw_im[s] = (double *)malloc(sizeof(double) * (size_t)Ns * (size_t)(r - 1) + 8);
    for (long k = 0; k < Ns; k++) {
      for (int q = 1; q < r; q++) {
        double c, si;
        unit_root((long)q * k, Ns * r, &c, &si);
        a->tw_re[s][k * (r - 1) + (q - 1)] = c;
        a->tw_im[s][k * (r - 1) + (q - 1)] = -si; /* forward: exp(-i...) */
      }
    }
    if (r != 2 && r != 4) {
      a->rc[s] = (double *)malloc(sizeof(double) * (size_t)r * (size_t)r);
      a->rs[s] = (double *)malloc(sizeof(double) * (size_t)r * (size_t)r);
      for (int p = 0; p < r; p++)
        for (int q = 0; q < r; q++) {
          double c, si;
          unit_root((long)p * q, r, &c, &si);
          a->rc[s][p * r + q] = c;
          a->rs[s][p * r + q] = si;
        }
    }
    Ns *= r;
  }
}

static void axis_free(axis_plan *a) {
  for (int s = 0; s < a->nstage; s++) {
    free(a->tw_re[s]);
    free(a->tw_im[s]);
    free(a->rc[s]);
    free(a->rs[s]);
  }
}

orc_fft3 *orc_fft3_create(long nz, long ny, long nx) {
  if (nz < 1 || ny < 1 || nx < 1) return NULL;
  orc_fft3 *p = (orc_fft3 *)calloc(1, sizeof(orc_fft3));
  if (!p) return NULL;
  p->n[0] = nz;
  p->n[1] = ny;
  p->n[2] = nx;
  for (int d = 0; d < 3; d++) axis_init(&p->ax[d], p->n[d]);
  return p;
}

void orc_fft3_destroy(orc_fft3 *p) {
  if (!p) return;
  for (int d = 0; d < 3; d++) axis_free(&p->ax[d]);
  free(p);
}

/* ------------------------------------------------------------------------- */
/* One Stockham stage on a panel: x -> y, arrays [n][W] split re/im.         */

typedef struct {
  double *re, *im;
} panel;

static void stage(const axis_plan *a, int s, int sign, const panel x, panel y, int W) {
  const long n = a->n;
  const int r = a->radix[s];
  const long Ns = a->span[s];
  const long nr = n / r;
  const double *twr = a->tw_re[s];
  const double *twi = a->tw_im[s];
  const double sg = (double)sign; /* imag parts of roots carry the sign */
  /* radices above 64 are not produced for the grids this oracle serves */
  double vr[64][PANEL_W], vi[64][PANEL_W];
  for (long j = 0; j < nr; j++) {
    const long k = j % Ns;
    const long out0 = (j / Ns) * Ns * r + k;
    /* gather and twiddle */
    for (int q = 0; q < r; q++) {
      const double *xr = x.re + (size_t)(j + q * nr) * W;
      const double *xi = x.im + (size_t)(j + q * nr) * W;
      if (q == 0 || k == 0) {
        for (int w = 0; w < W; w++) { vr[q][w] = xr[w]; vi[q][w] = xi[w]; }
      } else {
        /* the table holds exp(-i theta); multiply by exp(sign i theta) */
        const double c = twr[k * (r - 1) + (q - 1)];
        const double sn = (sign < 0) ? twi[k * (r - 1) + (q - 1)] : -twi[k * (r - 1) + (q - 1)];
        for (int w = 0; w < W; w++) {
          const double ar = xr[w], ai = xi[w];
          vr[q][w] = ar * c - ai * sn;
          vi[q][w] = ar * sn + ai * c;
        }
      }
    }
    /* butterfly */
    double *yr[64], *yi[64];
    for (int p = 0; p < r; p++) {
      yr[p] = y.re + (size_t)(out0 + p * Ns) * W;
      yi[p] = y.im + (size_t)(out0 + p * Ns) * W;
    }
    if (r == 2) {
      for (int w = 0; w < W; w++) {
        const double ar = vr[0][w], ai = vi[0][w], br = vr[1][w], bi = vi[1][w];
        yr[0][w] = ar + br; yi[0][w] = ai + bi;
        yr[1][w] = ar - br; yi[1][w] = ai - bi;
      }
    } else if (r == 4) {
      for (int w = 0; w < W; w++) {
        const double t0r = vr[0][w] + vr[2][w], t0i = vi[0][w] + vi[2][w];
        const double t1r = vr[0][w] - vr[2][w], t1i = vi[0][w] - vi[2][w];
        const double t2r = vr[1][w] + vr[3][w], t2i = vi[1][w] + vi[3][w];
        const double t3r = vr[1][w] - vr[3][w], t3i = vi[1][w] - vi[3][w];
        /* sign * i * t3 */
        const double ur = -sg * t3i, ui = sg * t3r;
        yr[0][w] = t0r + t2r; yi[0][w] = t0i + t2i;
        yr[2][w] = t0r - t2r; yi[2][w] = t0i - t2i;
        yr[1][w] = t1r + ur;  yi[1][w] = t1i + ui;
        yr[3][w] = t1r - ur;  yi[3][w] = t1i - ui;
      }
    } else {
      /* odd radix: pair q with r-q */
      const int h = (r - 1) / 2;
      const double *rc = a->rc[s], *rs = a->rs[s];
      double sr[32][PANEL_W], si[32][PANEL_W], dr[32][PANEL_W], di[32][PANEL_W];
      for (int q = 1; q <= h; q++)
        for (int w = 0; w < W; w++) {
          sr[q][w] = vr[q][w] + vr[r - q][w];
          si[q][w] = vi[q][w] + vi[r - q][w];
          dr[q][w] = vr[q][w] - vr[r - q][w];
          di[q][w] = vi[q][w] - vi[r - q][w];
        }
      for (int w = 0; w < W; w++) {
        double accr = vr[0][w], acci = vi[0][w];
        for (int q = 1; q <= h; q++) { accr += sr[q][w]; acci += si[q][w]; }
        yr[0][w] = accr; yi[0][w] = acci;
      }
      for (int p = 1; p <= h; p++) {
        for (int w = 0; w < W; w++) {
          double cr = vr[0][w], ci = vi[0][w], er = 0.0, ei = 0.0;
          for (int q = 1; q <= h; q++) {
            const double c = rc[p * r + q], sn = sg * rs[p * r + q];
            cr += c * sr[q][w];
            ci += c * si[q][w];
            /* i * sn * d */
            er += -sn * di[q][w];
            ei += sn * dr[q][w];
          }
          yr[p][w] = cr + er;     yi[p][w] = ci + ei;
          yr[r - p][w] = cr - er; yi[r - p][w] = ci - ei;
        }
      }
    }
  }
}

/* Run all stages of axis a on panel A (scratch B); returns the panel holding
 * the result. */
static panel run_axis(const axis_plan *a, int sign, panel A, panel B, int W) {
  for (int s = 0; s < a->nstage; s++) {
    stage(a, s, sign, A, B, W);
    panel t = A; A = B; B = t;
  }
  return A;
}

void orc_fft3_exec(const orc_fft3 *p, double *data, int sign) {
  const long nz = p->n[0], ny = p->n[1], nx = p->n[2];
  long nmax = nz > ny ? nz : ny;
  if (nx > nmax) nmax = nx;
  const size_t psz = (size_t)nmax * PANEL_W;
  double *buf = (double *)malloc(sizeof(double) * psz * 4);
  panel A = {buf, buf + psz}, B = {buf + 2 * psz, buf + 3 * psz};

  /* x axis: lines contiguous; a panel is W consecutive lines */
  {
    const axis_plan *a = &p->ax[2];
    const long nlines = ny * nz;
    for (long l0 = 0; l0 < nlines; l0 += PANEL_W) {
      const int W = (int)((nlines - l0) < PANEL_W ? (nlines - l0) : PANEL_W);
      for (int w = 0; w < W; w++) {
        const double *src = data + 2 * (size_t)(l0 + w) * nx;
        for (long i = 0; i < nx; i++) {
          A.re[i * W + w] = src[2 * i];
          A.im[i * W + w] = src[2 * i + 1];
        }
      }
      panel R = run_axis(a, sign, A, B, W);
      for (int w = 0; w < W; w++) {
        double *dst = data + 2 * (size_t)(l0 + w) * nx;
        for (long i = 0; i < nx; i++) {
          dst[2 * i] = R.re[i * W + w];
          dst[2 * i + 1] = R.im[i * W + w];
        }
      }
    }
  }
  /* y and z axes: a panel is W consecutive x at each position of the axis */
  for (int d = 1; d >= 0; d--) {
    const axis_plan *a = &p->ax[d];
    const long n = a->n;
    const long stride = (d == 1) ? nx : nx * ny;     /* between axis points */
    const long nouter = (d == 1) ? nz : ny;          /* other slow index */
    const long ostride = (d == 1) ? nx * ny : nx;
    if (n == 1) continue;
    for (long o = 0; o < nouter; o++) {
      for (long x0 = 0; x0 < nx; x0 += PANEL_W) {
        const int W = (int)((nx - x0) < PANEL_W ? (nx - x0) : PANEL_W);
        for (long i = 0; i < n; i++) {
          const double *src = data + 2 * (size_t)(o * ostride + i * stride + x0);
          for (int w = 0; w < W; w++) {
            A.re[i * W + w] = src[2 * w];
            A.im[i * W + w] = src[2 * w + 1];
          }
        }
        panel R = run_axis(a, sign, A, B, W);
        for (long i = 0; i < n; i++) {
          double *dst = data + 2 * (size_t)(o * ostride + i * stride + x0);
          for (int w = 0; w < W; w++) {
            dst[2 * w] = R.re[i * W + w];
            dst[2 * w + 1] = R.im[i * W + w];
          }
        }
      }
    }
  }
  free(buf);
}
