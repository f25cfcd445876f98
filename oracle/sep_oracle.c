/*
 * sep_oracle.c -- CPU restatement of the reference's filter path.
 *
 * TEST INFRASTRUCTURE ONLY (parity checker, golden-vector source, timed CPU
 * baseline).  Nothing in the product links or loads this file.  Each function
 * restates the reference lines cited beside it; operation order is kept where
 * the result must match bit for bit (random numbers, k^2 table, Newton
 * coefficients, grid coordinates).  Compile with -ffp-contract=off.
 *
 * Parity is pinned against the reference's own sources (Makefile.ref build)
 * and the In13_P16 fixture; see the oracle tests.
 */
#define _GNU_SOURCE
#include "sep_oracle.h"

#include <dlfcn.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "fft_cpu.h"

#define ORC_PI 3.14159265358979323846
#define ORC_TWO_PI 6.28318530717958647692

static double now_s(void) {
  struct timeval tv;
  gettimeofday(&tv, NULL);
  return (double)tv.tv_sec + 1e-6 * (double)tv.tv_usec;
}

/* ========================================================================= */
/* Random numbers -- filter/rand.c:28-66.  L'Ecuyer's combined generator     */
/* (moduli 2147483563 and 2147483399) with a 32-entry Bays-Durham shuffle, as  */
/* published in Numerical Recipes (ran2).  The reference keeps the second     */
/* stream and the shuffle table in statics; here they live in orc_rng.        */

enum { L1_M = 2147483563, L2_M = 2147483399, L1_A = 40014, L2_A = 40692, L1_Q = 53668,
       L2_Q = 52774, L1_R = 12211, L2_R = 3791, SHUF = 32 };

void orc_rng_seed(orc_rng *r, long idum) {
  memset(r, 0, sizeof(*r));
  r->idum = idum;
  r->idum2 = 123456789; /* rand.c:32 initial value of the static */
  r->iy = 0;
}

static long schrage(long v, long a, long q, long rr, long m) {
  long k = v / q;
  v = a * (v - k * q) - k * rr;
  if (v < 0) v += m;
  return v;
}

double orc_rng_next(orc_rng *r) {
  if (r->idum <= 0) { /* rand.c:36-48: (re)initialise */
    r->idum = (-(r->idum) < 1) ? 1 : -(r->idum);
    r->idum2 = r->idum;
    for (int j = SHUF + 7; j >= 0; j--) {
      r->idum = schrage(r->idum, L1_A, L1_Q, L1_R, L1_M);
      if (j < SHUF) r->iv[j] = r->idum;
    }
    r->iy = r->iv[0];
  }
  r->idum = schrage(r->idum, L1_A, L1_Q, L1_R, L1_M);
  r->idum2 = schrage(r->idum2, L2_A, L2_Q, L2_R, L2_M);
  const long ndiv = 1 + (L1_M - 1) / SHUF;
  long j = r->iy / ndiv;
  r->iy = r->iv[j] - r->idum2;
  r->iv[j] = r->idum;
  if (r->iy < 1) r->iy += L1_M - 1;
  const double am = 1.0 / (double)L1_M;
  const double rnmx = 1.0 - 1.2e-7;
  double t = am * (double)r->iy;
  return (t > rnmx) ? rnmx : t;
}

/* filter/init.c:236-251 and filter/norm.c:9-36 (normalize divides by the norm) */
void orc_init_psi(orc_rng *r, long ngrid, double dv, double *psi_re) {
  double s = 0.0;
  for (long g = 0; g < ngrid; g++) psi_re[g] = -1.0 + 2.0 * orc_rng_next(r);
  for (long g = 0; g < ngrid; g++) s += psi_re[g] * psi_re[g];
  const double nrm = sqrt(s * dv);
  for (long g = 0; g < ngrid; g++) psi_re[g] /= nrm;
}

/* ========================================================================= */
/* Set-up.                                                                   */

/* filter/read.c:16-30: subtract the mean position */
void orc_center_atoms(long natom, double *rx, double *ry, double *rz) {
  double mx = 0.0, my = 0.0, mz = 0.0;
  for (long i = 0; i < natom; i++) { mx += rx[i]; my += ry[i]; mz += rz[i]; }
  mx /= (double)natom;
  my /= (double)natom;
  mz /= (double)natom;
  for (long i = 0; i < natom; i++) { rx[i] -= mx; ry[i] -= my; rz[i] -= mz; }
}

/* filter/init.c:90-92 with filter/size.c:30-44 (largest pairwise extent) */
double orc_box_half(const double *r, long natom) {
  double lo = r[0], hi = r[0];
  for (long i = 1; i < natom; i++) {
    if (r[i] < lo) lo = r[i];
    if (r[i] > hi) hi = r[i];
  }
  return rint(0.5 * (hi - lo) + 5.0);
}

/* filter/init.c:124-144 -- k^2/2 pre-scaled by 1/N and capped at Ekinmax/N.
 * The three axis tables multiply their 1/n factors in the reference's order. */
void orc_ksqr(long nx, long ny, long nz, double dx, double dy, double dz, double ekinmax,
              double *ksqr) {
  const double nx1 = 1.0 / (double)nx, ny1 = 1.0 / (double)ny, nz1 = 1.0 / (double)nz;
  const double dkx = ORC_TWO_PI / ((double)nx * dx);
  const double dky = ORC_TWO_PI / ((double)ny * dy);
  const double dkz = ORC_TWO_PI / ((double)nz * dz);
  double *kx = calloc(nx, sizeof(double)), *ky = calloc(ny, sizeof(double)),
         *kz = calloc(nz, sizeof(double));
  for (long j = 1; j <= nx / 2; j++) {
    double k = (double)j * dkx;
    kx[j] = kx[nx - j] = 0.5 * (k * k) * nx1 * ny1 * nz1 / 1.0;
  }
  for (long j = 1; j <= ny / 2; j++) {
    double k = (double)j * dky;
    ky[j] = ky[ny - j] = 0.5 * (k * k) * ny1 * nx1 * nz1 / 1.0;
  }
  for (long j = 1; j <= nz / 2; j++) {
    double k = (double)j * dkz;
    kz[j] = kz[nz - j] = 0.5 * (k * k) * nz1 * nx1 * ny1 / 1.0;
  }
  const double cap = ekinmax * (ny1 * nx1 * nz1);
  for (long jz = 0; jz < nz; jz++)
    for (long jy = 0; jy < ny; jy++)
      for (long jx = 0; jx < nx; jx++) {
        double v = kx[jx] + ky[jy] + kz[jz];
        ksqr[nx * (ny * jz + jy) + jx] = (v > cap) ? cap : v;
      }
  free(kx);
  free(ky);
  free(kz);
}

/* filter/read.c:105-108: every value minus the original last one */
void orc_shift_table(double *v, long n) {
  const double last = v[n - 1];
  for (long i = 0; i < n; i++) v[i] -= last;
}

/* filter/interpolate.c:11-23 (scale = 1) and
 * filterStrainCube/interpolate.c:11-25 (per-atom strain scale) */
static double table_value(double r, double dr, const double *tr, const double *tv, long n,
                          double scale, int scaled) {
  long i = (long)(r / dr);
  if (i > n - 2) return 0.0;
  double a, b;
  if (scaled) {
    a = scale * (tv[i + 1] - tv[i]) / (tr[i + 1] - tr[i]);
    b = scale * tv[i] - tr[i] * a;
  } else {
    a = (tv[i + 1] - tv[i]) / (tr[i + 1] - tr[i]);
    b = tv[i] - tr[i] * a;
  }
  return a * r + b;
}

/* filter/init.c:157-182: grid coordinates by running sums from xmin, then
 * V(r_g) = sum over atoms of the type's table at |r_g - R_a| (no cutoff). */
void orc_vbuild(long natom, const double *rx, const double *ry, const double *rz,
                const long *type, const double *scale, const double *tab_r,
                const double *tab_v, const long *tab_n, long tab_stride, long nx, long ny,
                long nz, double xmin, double ymin, double zmin, double dx, double dy,
                double dz, double *potl) {
  double *vx = malloc(sizeof(double) * nx), *vy = malloc(sizeof(double) * ny),
         *vz = malloc(sizeof(double) * nz);
  double c = xmin;
  for (long j = 0; j < nx; j++, c += dx) vx[j] = c;
  c = ymin;
  for (long j = 0; j < ny; j++, c += dy) vy[j] = c;
  c = zmin;
  for (long j = 0; j < nz; j++, c += dz) vz[j] = c;
#pragma omp parallel for schedule(static)
  for (long jz = 0; jz < nz; jz++)
    for (long jy = 0; jy < ny; jy++)
      for (long jx = 0; jx < nx; jx++) {
        double sum = 0.0;
        for (long a = 0; a < natom; a++) {
          const double ddx = vx[jx] - rx[a], ddy = vy[jy] - ry[a], ddz = vz[jz] - rz[a];
          const double d = sqrt(ddx * ddx + ddy * ddy + ddz * ddz);
          const long t = type[a];
          const double *tr = tab_r + t * tab_stride, *tv = tab_v + t * tab_stride;
          sum += table_value(d, tr[1] - tr[0], tr, tv, tab_n[t], scale ? scale[a] : 1.0,
                             scale != NULL);
        }
        potl[nx * (ny * jz + jy) + jx] = sum;
      }
  free(vx);
  free(vy);
  free(vz);
}

/* pseudopotFitting/hamiltonian.c:91-94 */
double orc_form_factor(double q, const double a[4]) {
  return a[0] * (q * q - a[1]) / (a[2] * exp(a[3] * q * q) + 1.0);
}

/* pseudopotFitting/pot.c:35-63: l = 0 sine transform of v(q) on 1024 points,
 * q in [0, 5), r step 0.02*2pi/(1024 dq); r = 0 uses sin(qr)/(qr) -> 1. */
void orc_form_factor_table(const double a[4], double vol_per_atom, double *r, double *v) {
  enum { NG = 1024 };
  const double dq = (5.0 - 0.0) / (double)NG;
  const double dr = 0.02 * ORC_TWO_PI / ((double)NG * dq);
  double q[NG], vq[NG];
  double s = 0.0;
  for (int i = 0; i < NG; i++, s += dq) q[i] = s;
  s = 0.0;
  for (int i = 0; i < NG; i++, s += dr) r[i] = s;
  for (int i = 0; i < NG; i++) vq[i] = orc_form_factor(q[i], a) * vol_per_atom;
  const double pref = pow(ORC_TWO_PI, 3.0);
  for (int ir = 1; ir < NG; ir++) {
    double acc = 0.0;
    for (int i = 0; i < NG; i++) acc += q[i] * sin(q[i] * r[ir]) * vq[i];
    v[ir] = acc * (dq * 4.0 * ORC_PI / (pref * r[ir]));
  }
  double acc = 0.0;
  for (int i = 0; i < NG; i++) acc += q[i] * q[i] * vq[i];
  v[0] = acc * (dq * 4.0 * ORC_PI / pref);
}

/* ========================================================================= */
/* Newton interpolation -- filter/coeff.c                                    */

/* coeff.c:82-134 (samp_points_ashkenazy with range = 0): 32*nc candidates,
 * 7/8 of them evenly on [-2, 2] and 1/8 at the origin; each new point
 * maximises the sum of log squared distances to the points already taken
 * (first index wins ties); candidates closer than 1e-5 to a taken point are
 * retired. */
void orc_leja_points(long nc, double *zre, double *zim) {
  const long ncand = 32 * nc, nimag = ncand / 8;
  const double lo = -2.0, hi = 2.0, span_im = 0.0 * lo, span_im_hi = 0.0 * hi;
  const double step_re = (hi - lo) / (double)(ncand - 1 - nimag);
  const double step_im = (span_im_hi - span_im) / (double)(nimag - 1);
  double *cre = calloc(ncand, sizeof(double)), *cim = calloc(ncand, sizeof(double));
  double *score = calloc(ncand, sizeof(double));
  for (long k = 0; k < ncand - nimag; k++) cre[k] = lo + (double)k * step_re;
  for (long k = ncand - nimag; k < ncand; k++)
    cim[k] = span_im + (double)(k - ncand + nimag) * step_im;
  zre[0] = cre[0];
  zim[0] = cim[0];
  for (long k = 0; k < ncand; k++) {
    const double a = cre[k] - zre[0], b = cim[k] - zim[0];
    const double d2 = a * a + b * b;
    score[k] = (d2 < 1.0e-10) ? -1.0e30 : log(d2);
  }
  for (long j = 1; j < nc; j++) {
    long best = 0;
    double top = -2.0e30;
    for (long k = 0; k < ncand; k++)
      if (score[k] > top) { top = score[k]; best = k; }
    zre[j] = cre[best];
    zim[j] = cim[best];
    for (long k = 0; k < ncand; k++) {
      const double a = cre[k] - zre[j], b = cim[k] - zim[j];
      const double d2 = a * a + b * b;
      if (d2 < 1.0e-10) score[k] = -1.0e30;
      else score[k] += log(d2);
    }
  }
  free(cre);
  free(cim);
  free(score);
}

/* Gaussian filter value, coeff.c:11 */
static double gauss_filter(double x, double dt) {
  return sqrt(dt / ORC_PI) * exp(-(x * x) * dt);
}

/* coeff.c:16-63: Newton divided differences of the Gaussian filter centred
 * at el[e], sampled at x_j = (z_j + 2)/(4/dE) + vmin. */
void orc_coefficients(long ms, long nc, double dE, double vmin, double dt, const double *el,
                      double *an_re, double *an_im, double *zn) {
  double *zre = malloc(sizeof(double) * nc), *zim = malloc(sizeof(double) * nc);
  orc_leja_points(nc, zre, zim);
  for (long j = 0; j < nc; j++) zn[j] = zre[j];
  const double scale = (2.0 - (-2.0)) / dE;
  for (long e = 0; e < ms; e++) {
    double *ar = an_re + e * nc, *ai = an_im + e * nc;
    double x = (zn[0] + 2.0) / scale + vmin;
    ar[0] = gauss_filter(x - el[e], dt);
    ai[0] = 0.0;
    if (nc < 2) continue;
    x = (zn[1] + 2.0) / scale + vmin;
    ar[1] = (gauss_filter(x - el[e], dt) - ar[0]) / (zn[1] - zn[0]);
    ai[1] = (-ai[0]) / (zn[1] - zn[0]);
    for (long j = 2; j < nc; j++) {
      double prod = 1.0, sr = 0.0, si = 0.0;
      for (long i = 1; i < j; i++) {
        prod *= (zn[j] - zn[i - 1]);
        sr += ar[i] * prod;
        si += ai[i] * prod;
      }
      prod *= (zn[j] - zn[j - 1]);
      x = (zn[j] + 2.0) / scale + vmin;
      ar[j] = (gauss_filter(x - el[e], dt) - ar[0] - sr) / prod;
      ai[j] = (-ai[0] - si) / prod;
    }
  }
  free(zre);
  free(zim);
}

/* ========================================================================= */
/* Hamiltonian -- filter/hamiltonian.c:11-44, filter/hnorm.c:11-39           */

struct orc_ctx {
  long nx, ny, nz, ngrid;
  const double *potl, *ksqr;
  double dv;
  orc_fft3 *fft;
};

orc_ctx *orc_ctx_create(long nx, long ny, long nz, const double *potl, const double *ksqr,
                        double dv) {
  orc_ctx *c = calloc(1, sizeof(orc_ctx));
  c->nx = nx;
  c->ny = ny;
  c->nz = nz;
  c->ngrid = nx * ny * nz;
  c->potl = potl;
  c->ksqr = ksqr;
  c->dv = dv;
  c->fft = orc_fft3_create(nz, ny, nx);
  return c;
}

void orc_ctx_destroy(orc_ctx *c) {
  if (!c) return;
  orc_fft3_destroy(c->fft);
  free(c);
}

/* T psi: forward FFT, times k^2/2N, backward FFT (hamiltonian.c:27-44),
 * then + V psi (hamiltonian.c:15-20). */
void orc_hamiltonian(const orc_ctx *c, const double *psi, double *hpsi) {
  const long n = c->ngrid;
  double *w = malloc(sizeof(double) * 2 * n);
  memcpy(w, psi, sizeof(double) * 2 * n);
  orc_fft3_exec(c->fft, w, -1);
  for (long g = 0; g < n; g++) {
    w[2 * g] *= c->ksqr[g];
    w[2 * g + 1] *= c->ksqr[g];
  }
  orc_fft3_exec(c->fft, w, +1);
  for (long g = 0; g < n; g++) {
    const double v = c->potl[g];
    const double pr = psi[2 * g], pi = psi[2 * g + 1];
    hpsi[2 * g] = w[2 * g] + v * pr;
    hpsi[2 * g + 1] = w[2 * g + 1] + v * pi;
  }
  free(w);
}

void orc_hnorm(const orc_ctx *c, const double *psim1, double *psin, double dE_1, double vmin,
               double zm1) {
  const long n = c->ngrid;
  orc_hamiltonian(c, psim1, psin);
  const double shift = 2.0 + zm1 + vmin * dE_1;
  for (long g = 0; g < 2 * n; g++) psin[g] = dE_1 * psin[g] - shift * psim1[g];
}

/* filter/filter.c:59-83 */
void orc_filter_cycle(const orc_ctx *c, const double *start, const double *an_re,
                      const double *zn, long ms, long nc, double dE_1, double vmin,
                      double *psi0) {
  const long n = c->ngrid;
  double *cur = calloc(2 * n, sizeof(double)), *prev = calloc(2 * n, sizeof(double));
  for (long g = 0; g < n; g++) cur[2 * g] = start[g];
  for (long e = 0; e < ms; e++)
    for (long g = 0; g < n; g++) psi0[e * n + g] = an_re[e * nc] * cur[2 * g];
  for (long j = 1; j < nc; j++) {
    double *t = prev; prev = cur; cur = t;
    orc_hnorm(c, prev, cur, dE_1, vmin, zn[j - 1]);
    for (long e = 0; e < ms; e++) {
      const double a = an_re[e * nc + j];
      double *p = psi0 + e * n;
      for (long g = 0; g < n; g++) p[g] += a * cur[2 * g];
    }
  }
  free(cur);
  free(prev);
}

/* filter/norm.c:40-54 */
void orc_normalize_all(double *psi, double dv, long m, long ngrid) {
  for (long e = 0; e < m; e++) {
    double *p = psi + e * ngrid, s = 0.0;
    for (long g = 0; g < ngrid; g++) s += p[g] * p[g];
    if (s != 0.0) s = 1.0 / sqrt(s * dv);
    for (long g = 0; g < ngrid; g++) p[g] *= s;
  }
}

/* filter/energy.c:28-49: <psi|H|psi> dv for real states */
void orc_energy_all(const orc_ctx *c, const double *psi0, long m, double *ene) {
  const long n = c->ngrid;
  double *z = calloc(2 * n, sizeof(double)), *hz = malloc(sizeof(double) * 2 * n);
  for (long e = 0; e < m; e++) {
    for (long g = 0; g < n; g++) { z[2 * g] = psi0[e * n + g]; z[2 * g + 1] = 0.0; }
    orc_hamiltonian(c, z, hz);
    double s = 0.0;
    for (long g = 0; g < n; g++) s += z[2 * g] * hz[2 * g] + z[2 * g + 1] * hz[2 * g + 1];
    ene[e] = s * c->dv;
  }
  free(z);
  free(hz);
}

/* filter/energy.c:53-83: power iteration from the fixed seed -874917403,
 * psi <- H psi / |H psi|, E = <psi|H|psi>, until |dE/E| <= 1e-4 or 500
 * iterations; then dE = 1.1 (E - vmin). */
long orc_energy_range(const orc_ctx *c, double vmin, double *emax, double *dE) {
  const long n = c->ngrid;
  double *psi = calloc(2 * n, sizeof(double)), *hp = malloc(sizeof(double) * 2 * n);
  double *re = malloc(sizeof(double) * n);
  orc_rng r;
  orc_rng_seed(&r, -874917403);
  orc_init_psi(&r, n, c->dv, re);
  for (long g = 0; g < n; g++) psi[2 * g] = re[g];
  double ene = 0.0 + 0.1, old = 0.0;
  long it;
  for (it = 0; fabs((ene - old) / ene) > 1.0e-4 && it < 500; it++) {
    orc_hamiltonian(c, psi, hp);
    double s = 0.0;
    for (long g = 0; g < 2 * n; g++) s += hp[g] * hp[g];
    const double nrm = sqrt(s * c->dv);
    for (long g = 0; g < 2 * n; g++) psi[g] = hp[g] / nrm;
    old = ene;
    orc_hamiltonian(c, psi, hp);
    s = 0.0;
    for (long g = 0; g < n; g++) s += psi[2 * g] * hp[2 * g] + psi[2 * g + 1] * hp[2 * g + 1];
    ene = s * c->dv;
  }
  *emax = ene;
  *dE = 1.1 * (ene - vmin);
  free(psi);
  free(hp);
  free(re);
  return it;
}

/* ========================================================================= */
/* Subspace -- filter/ortho.c, filter/Hmat.c, filter/energy.c:88-119         */

typedef void (*dgesvd_fn)(const char *, const char *, const long long *, const long long *,
                          double *, const long long *, double *, double *, const long long *,
                          double *, const long long *, double *, const long long *,
                          long long *, size_t, size_t);
typedef void (*dsyev_fn)(const char *, const char *, const long long *, double *,
                         const long long *, double *, double *, const long long *,
                         long long *, size_t, size_t);
static dgesvd_fn p_dgesvd;
static dsyev_fn p_dsyev;

int orc_lapack_load(const char *path) {
  void *h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h) return -1;
  p_dgesvd = (dgesvd_fn)dlsym(h, "scipy_dgesvd_64_");
  p_dsyev = (dsyev_fn)dlsym(h, "scipy_dsyev_64_");
  return (p_dgesvd && p_dsyev) ? 0 : -2;
}

/* ortho.c:11-52: in-place thin SVD (U overwrites psi, column-major ngrid x m),
 * keep the leading columns with S_i/S_0 >= 1e-10.  Returns the kept count,
 * or -1 when LAPACK is missing or fails. */
long orc_portho(double *psi, long ngrid, long m, double *sv_out) {
  if (!p_dgesvd) return -1;
  long long M = ngrid, N = m, one = 1, info = 0;
  long long lwork = 5 * ((long long)m * m + ngrid);
  double *s = malloc(sizeof(double) * m), *work = malloc(sizeof(double) * lwork);
  p_dgesvd("O", "N", &M, &N, psi, &M, s, NULL, &one, NULL, &one, work, &lwork, &info, 1, 1);
  long kept = m;
  if (info != 0) kept = -1;
  else
    for (long i = 0; i < m; i++)
      if (s[i] / s[0] < 1.0e-10) { kept = i; break; }
  if (sv_out) memcpy(sv_out, s, sizeof(double) * m);
  free(s);
  free(work);
  return kept;
}

/* Hmat.c:11-86: H_ij = <H psi_i | psi_j> dv, dsyev("V","U"), psi <- psi V */
int orc_hmat(const orc_ctx *c, double *psi, long m, double *eval) {
  if (!p_dsyev) return -1;
  const long n = c->ngrid;
  double *h = calloc((size_t)m * m, sizeof(double));
  double *z = calloc(2 * n, sizeof(double)), *hz = malloc(sizeof(double) * 2 * n);
  for (long i = 0; i < m; i++) {
    for (long g = 0; g < n; g++) { z[2 * g] = psi[i * n + g]; z[2 * g + 1] = 0.0; }
    orc_hamiltonian(c, z, hz);
    for (long j = 0; j < m; j++) {
      double s = 0.0;
      const double *pj = psi + j * n;
      for (long g = 0; g < n; g++) s += hz[2 * g] * pj[g];
      h[i * m + j] = s * c->dv;
    }
  }
  long long M = m, lwk = 3 * m, info = 0;
  double *work = malloc(sizeof(double) * lwk);
  p_dsyev("V", "U", &M, h, &M, eval, work, &lwk, &info, 1, 1);
  if (info != 0) { free(h); free(z); free(hz); free(work); return -2; }
  double *row = malloc(sizeof(double) * m);
  for (long g = 0; g < n; g++) {
    for (long i = 0; i < m; i++) row[i] = psi[i * n + g];
    for (long k = 0; k < m; k++) {
      double s = 0.0;
      for (long i = 0; i < m; i++) s += h[k * m + i] * row[i];
      psi[k * n + g] = s;
    }
  }
  free(row);
  free(h);
  free(z);
  free(hz);
  free(work);
  return 0;
}

/* energy.c:88-119: sigma = sqrt(|<psi|H H psi> - <psi|H psi>^2|) */
void orc_sigma(const orc_ctx *c, const double *psi, long m, double *sige) {
  const long n = c->ngrid;
  double *z = calloc(2 * n, sizeof(double)), *hz = malloc(sizeof(double) * 2 * n);
  double *hhz = malloc(sizeof(double) * 2 * n);
  for (long k = 0; k < m; k++) {
    const double *p = psi + k * n;
    for (long g = 0; g < n; g++) { z[2 * g] = p[g]; z[2 * g + 1] = 0.0; }
    orc_hamiltonian(c, z, hz);
    double e = 0.0;
    for (long g = 0; g < n; g++) e += p[g] * hz[2 * g];
    e *= c->dv;
    orc_hamiltonian(c, hz, hhz);
    double e2 = 0.0;
    for (long g = 0; g < n; g++) e2 += p[g] * hhz[2 * g];
    e2 *= c->dv;
    sige[k] = sqrt(fabs(e2 - e * e));
  }
  free(z);
  free(hz);
  free(hhz);
}

static int omp_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* filter/main.c:92-98: the filter cycles of ns start states, one per OpenMP
 * thread as the reference runs them; returns the wall time in seconds. */
double orc_filter_batch(const orc_ctx *c, long ns, const double *start, const double *an_re,
                        const double *zn, long ms, long nc, double dE_1, double vmin,
                        double *out, int nthreads) {
  const long n = c->ngrid;
  /* the thread count applies to this region only (no process-wide setting) */
  const int nt = nthreads > 0 ? nthreads : omp_max_threads();
  double t0 = now_s();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
  for (long s = 0; s < ns; s++)
    orc_filter_cycle(c, start + (size_t)s * n, an_re, zn, ms, nc, dE_1, vmin,
                     out + (size_t)s * ms * n);
  return now_s() - t0;
}

/* ========================================================================= */
/* Whole pipeline, filter/main.c:64-142, OpenMP over start states as          */
/* main.c:92-98.                                                              */
long orc_pipeline(const orc_ctx *c, long ns, long ms, long nc, const double *el, double vmin,
                  double dE_in, const double *start, double *psitot, double *eval,
                  double *sige, int nthreads, int do_subspace, orc_timing *t) {
  const long n = c->ngrid;
  orc_timing tt;
  memset(&tt, 0, sizeof(tt));
  double t0 = now_s();
  double dE = dE_in;
  if (dE <= 0.0) tt.iters = orc_energy_range(c, vmin, &tt.emax, &dE);
  tt.energy_range_s = now_s() - t0;
  tt.dE = dE;
  const double dt = ((double)nc / (2.5 * dE)) * ((double)nc / (2.5 * dE));
  tt.dt = dt;
  double *an_re = malloc(sizeof(double) * ms * nc), *an_im = malloc(sizeof(double) * ms * nc);
  double *zn = malloc(sizeof(double) * nc);
  orc_coefficients(ms, nc, dE, vmin, dt, el, an_re, an_im, zn);
  const double dE_1 = 4.0 / dE;
  t0 = now_s();
  const int nt = nthreads > 0 ? nthreads : omp_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
  for (long s = 0; s < ns; s++) {
    /* filtering, filter.c:11-55: filter, normalise, energies of the block */
    double *blk = psitot + (size_t)s * ms * n;
    double *ene = malloc(sizeof(double) * ms);
    orc_filter_cycle(c, start + (size_t)s * n, an_re, zn, ms, nc, dE_1, vmin, blk);
    orc_normalize_all(blk, c->dv, ms, n);
    orc_energy_all(c, blk, ms, ene);
    free(ene);
  }
  tt.filter_s = now_s() - t0;
  long mk = ns * ms;
  if (do_subspace) {
    t0 = now_s();
    mk = orc_portho(psitot, n, ns * ms, NULL);
    if (mk > 0) orc_normalize_all(psitot, c->dv, mk, n);
    tt.ortho_s = now_s() - t0;
    t0 = now_s();
    if (mk > 0 && orc_hmat(c, psitot, mk, eval) == 0) orc_normalize_all(psitot, c->dv, mk, n);
    tt.hmat_s = now_s() - t0;
    t0 = now_s();
    if (mk > 0) orc_sigma(c, psitot, mk, sige);
    tt.sigma_s = now_s() - t0;
  }
  tt.mkept = mk;
  if (t) *t = tt;
  free(an_re);
  free(an_im);
  free(zn);
  return mk;
}
