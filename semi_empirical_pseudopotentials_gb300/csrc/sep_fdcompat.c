/*
 * sep_fdcompat.c -- the reference's filter entry points (include/sep_fd_compat.h)
 * on top of the GPU C ABI (include/sep_gb300.h).
 *
 * Each thread keeps one device context for the grid / potential it last
 * used; the reference calls filtering() concurrently from its OpenMP threads
 * (filter/main.c:92-98), and every thread then drives its own stream.  A
 * context is rebuilt when the grid, the spacing, the cap or the potential
 * pointer changes; the caller's k^2 array is checked once against the
 * context's own (filter/init.c:124-144) and a mismatch is an error.
 * Failures end the program the way the reference's nerror does
 * (filter/nerror.c:9-16).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "sep_fd_compat.h"
#include "sep_gb300.h"

typedef struct {
  sep_ctx *ctx;
  long nx, ny, nz;
  double dx, dy, dz, kcap;
  const double *potl;
} compat_slot;

static __thread compat_slot slot;

static void compat_fail(const char *where, int status) {
  char msg[512];
  snprintf(msg, sizeof msg, "%s: sep status %d: %s", where, status, sep_last_error());
  FILE *pf = fopen("error", "w");
  if (pf) {
    fprintf(pf, "%s\n", msg);
    fclose(pf);
  }
  fprintf(stderr, "%s\n", msg);
  exit(1);
}

#define OK(where, call)                  \
  do {                                   \
    int _s = (call);                     \
    if (_s != SEP_OK) compat_fail(where, _s); \
  } while (0)

/* the thread's context for this grid; potl / ksqr may be NULL (no physics) */
static sep_ctx *ctx_for(const long_st *ist, const par_st *par, const double *potl,
                        const double *ksqr) {
  const double dx = par ? par->dx : 1.0, dy = par ? par->dy : 1.0, dz = par ? par->dz : 1.0;
  const double kcap = par ? par->Ekinmax : 0.0;
  int same = slot.ctx && slot.nx == ist->nx && slot.ny == ist->ny && slot.nz == ist->nz;
  if (same && par) same = slot.dx == dx && slot.dy == dy && slot.dz == dz && slot.kcap == kcap;
  if (same && potl && slot.potl != potl) {
    OK("set potential", sep_ctx_set_potential(slot.ctx, potl));
    slot.potl = potl;
  }
  if (same) return slot.ctx;
  if (slot.ctx) sep_ctx_destroy(slot.ctx);
  memset(&slot, 0, sizeof slot);
  const long dims[3] = {ist->nx, ist->ny, ist->nz};
  const double steps[3] = {dx, dy, dz};
  OK("create context", sep_ctx_create(dims, steps, 10.0, potl, SEP_PREC_F64, &slot.ctx));
  if (par && kcap > 0.0) OK("kinetic cap", sep_ctx_set_kcap(slot.ctx, kcap));
  if (ksqr) {
    double *mine = (double *)malloc(sizeof(double) * (size_t)ist->ngrid);
    if (!mine) compat_fail("ksqr check", SEP_ERR_NOMEM);
    OK("ksqr", sep_ctx_ksqr(slot.ctx, mine));
    for (long g = 0; g < ist->ngrid; g++)
      if (mine[g] != ksqr[g]) {
        free(mine);
        compat_fail("ksqr differs from the grid's capped k^2 (filter/init.c:124-144)",
                    SEP_ERR_ARG);
      }
    free(mine);
  }
  slot.nx = ist->nx;
  slot.ny = ist->ny;
  slot.nz = ist->nz;
  slot.dx = dx;
  slot.dy = dy;
  slot.dz = dz;
  slot.kcap = kcap;
  slot.potl = potl;
  return slot.ctx;
}

/* ---- filter/hamiltonian.c ------------------------------------------------ */
void kinetic(zomplex *psi, double *ksqr, fftw_plan_loc planfw, fftw_plan_loc planbw,
             fftw_complex *fftwpsi, long_st ist) {
  (void)planfw; (void)planbw; (void)fftwpsi;
  /* T alone needs only the grid; the spacing lives in ksqr, so recover the
   * cap from the thread's context when it matches, else use the array max */
  sep_ctx *c = slot.ctx;
  if (!c || slot.nx != ist.nx || slot.ny != ist.ny || slot.nz != ist.nz)
    compat_fail("kinetic: call hamiltonian/hnorm on this grid first", SEP_ERR_ARG);
  (void)ksqr;
  OK("kinetic", sep_apply(c, (const double *)psi, NULL, (double *)psi, 1, 1.0, 0.0));
}

void hamiltonian(zomplex *phi, zomplex *psi, double *potl, double *ksqr, long_st ist,
                 par_st par, fftw_plan_loc planfw, fftw_plan_loc planbw, fftw_complex *fftwpsi) {
  (void)planfw; (void)planbw; (void)fftwpsi;
  sep_ctx *c = ctx_for(&ist, &par, potl, ksqr);
  memcpy(psi, phi, sizeof(zomplex) * (size_t)ist.ngrid);
  OK("hamiltonian", sep_hamiltonian(c, (const double *)psi, (double *)phi, 1));
}

/* ---- filter/hnorm.c ------------------------------------------------------ */
void hamiltonian_norm(zomplex *psi, zomplex *phi, double *potl, double *ksqr, long_st ist,
                      par_st par, fftw_plan_loc planfw, fftw_plan_loc planbw,
                      fftw_complex *fftwpsi) {
  (void)planfw; (void)planbw; (void)fftwpsi;
  sep_ctx *c = ctx_for(&ist, &par, potl, ksqr);
  OK("hamiltonian_norm", sep_apply(c, (const double *)phi, (const double *)psi, (double *)phi,
                                   1, 1.0, 0.0));
}

void hnorm(zomplex *psim1, zomplex *psin, double *potl, double *ksqr, par_st par, double zm1,
           long_st ist, fftw_plan_loc planfw, fftw_plan_loc planbw, fftw_complex *fftwpsi) {
  (void)planfw; (void)planbw; (void)fftwpsi;
  sep_ctx *c = ctx_for(&ist, &par, potl, ksqr);
  /* the reference applies H to psin, which filter() has just set to psim1 */
  const double shift = 2.0 + zm1 + par.Vmin * par.dE_1;
  OK("hnorm", sep_apply(c, (const double *)psin, (const double *)psim1, (double *)psin, 1,
                        par.dE_1, -shift));
}

/* ---- filter/filter.c ----------------------------------------------------- */
static void filter_core(zomplex *psin, double *psi0, double *potl, double *ksqr, par_st par,
                        zomplex *an, double *zn, long_st ist, long tid, long jns) {
  sep_ctx *c = ctx_for(&ist, &par, potl, ksqr);
  const long n = ist.ngrid, ms = ist.ms, nc = ist.nc;
  double *start = (double *)malloc(sizeof(double) * (size_t)n);
  double *an_re = (double *)malloc(sizeof(double) * (size_t)ms * nc);
  if (!start || !an_re) compat_fail("filter", SEP_ERR_NOMEM);
  for (long g = 0; g < n; g++) start[g] = psin[g].re;
  for (long i = 0; i < ms * nc; i++) an_re[i] = an[i].re;
  OK("filter", sep_filter(c, start, 1, an_re, zn, ms, nc, par.dE_1, par.Vmin, psi0));
  free(start);
  free(an_re);
  /* progress file of filter.c:66-80: one line per 100 Newton steps */
  char str[100];
  snprintf(str, sizeof str, "prop%ld.dat", tid);
  FILE *pf = fopen(str, "w");
  if (pf) {
    for (long j = 100; j < nc; j += 100) fprintf(pf, "%ld %ld\n", j, jns);
    fclose(pf);
  }
}

void filter(zomplex *psin, zomplex *psim1, double *psi0, double *potl, double *ksqr, par_st par,
            zomplex *an, double *zn, long_st ist, fftw_plan_loc planfw, fftw_plan_loc planbw,
            fftw_complex *fftwpsi, long tid, long jns) {
  (void)psim1; (void)planfw; (void)planbw; (void)fftwpsi;
  filter_core(psin, psi0, potl, ksqr, par, an, zn, ist, tid, jns);
}

void filtering(double *psitot, double *potl, double *ksqr, zomplex *an, double *zn, double *el,
               long_st ist, par_st par, long tid, long jns, long *idum) {
  (void)idum;
  const long n = ist.ngrid, ms = ist.ms;
  zomplex *psi = (zomplex *)calloc((size_t)n, sizeof(zomplex));
  double *eval = (double *)calloc((size_t)ms, sizeof(double));
  if (!psi || !eval) compat_fail("filtering", SEP_ERR_NOMEM);
  for (long g = 0; g < n; g++) psi[g].re = psitot[g];
  filter_core(psi, psitot, potl, ksqr, par, an, zn, ist, tid, jns);
  sep_ctx *c = ctx_for(&ist, &par, potl, ksqr);
  OK("normalize_all", sep_normalize_all(c, psitot, ms));
  OK("energy_all", sep_energy_all(c, psitot, ms, eval));
  char str[100];
  snprintf(str, sizeof str, "eval-filt-%ld-%ld.dat", tid, jns);
  OK("filtering", sep_write_filter_eval(str, eval, el, ms));
  snprintf(str, sizeof str, "psi-filt-%ld-%ld.dat", tid, jns);
  OK("filtering", sep_write_states(str, psitot, ms, n));
  free(psi);
  free(eval);
}

/* ---- filter/norm.c ------------------------------------------------------- */
double norm(zomplex *psi, double dr, long ngrid, long nthreads) {
  (void)nthreads;
  double s = 0.0;
  OK("norm", sep_row_sumsq((const double *)psi, 1, 2 * ngrid, &s));
  return sqrt(s * dr);
}

double normalize(zomplex *psi, double dr, long ngrid, long nthreads) {
  const double N = norm(psi, dr, ngrid, nthreads);
  OK("normalize", sep_normalize_states((double *)psi, 1, 2 * ngrid, dr));
  return N;
}

void normalize_all(double *psi, double dr, long ms, long ngrid, long nthreads) {
  (void)nthreads;
  OK("normalize_all", sep_normalize_states(psi, ms, ngrid, dr));
}

/* ---- filter/energy.c ----------------------------------------------------- */
double energy(zomplex *psi, zomplex *phi, double *potl, double *ksqr, long_st ist, par_st par,
              fftw_plan_loc planfw, fftw_plan_loc planbw, fftw_complex *fftwpsi) {
  (void)planfw; (void)planbw; (void)fftwpsi;
  sep_ctx *c = ctx_for(&ist, &par, potl, ksqr);
  OK("energy", sep_hamiltonian(c, (const double *)psi, (double *)phi, 1));
  double e = 0.0;
  for (long g = 0; g < ist.ngrid; g++) e += psi[g].re * phi[g].re + psi[g].im * phi[g].im;
  return e * par.dv;
}

void energy_all(zomplex *psi, zomplex *phi, double *psi0, double *potl, double *ksqr,
                double *ene, long_st ist, par_st par, fftw_plan_loc planfw,
                fftw_plan_loc planbw, fftw_complex *fftwpsi) {
  (void)psi; (void)phi; (void)planfw; (void)planbw; (void)fftwpsi;
  sep_ctx *c = ctx_for(&ist, &par, potl, ksqr);
  OK("energy_all", sep_energy_all(c, psi0, ist.ms, ene));
}

void get_energy_range(zomplex *psi, zomplex *phi, double *potl, double *vx, double *vy,
                      double *vz, double *ksqr, par_st *par, long_st ist, fftw_plan_loc planfw,
                      fftw_plan_loc planbw, fftw_complex *fftwpsi) {
  (void)psi; (void)phi; (void)vx; (void)vy; (void)vz; (void)planfw; (void)planbw; (void)fftwpsi;
  sep_ctx *c = ctx_for(&ist, par, potl, ksqr);
  double emax = 0.0, dE = 0.0;
  long it = 0;
  OK("get_energy_range", sep_energy_range(c, par->Vmin, &emax, &dE, &it));
  par->dE = dE;
  par->dE_1 = 4.0 / par->dE;
  printf("dE = %g\n", par->dE);
  fflush(stdout);
}

void calc_sigma_E(zomplex *psi, zomplex *phi, double *psitot, double *potl, double *ksqr,
                  double *eval, long_st ist, par_st par, fftw_plan_loc planfw,
                  fftw_plan_loc planbw, fftw_complex *fftwpsi) {
  (void)psi; (void)phi; (void)planfw; (void)planbw; (void)fftwpsi;
  sep_ctx *c = ctx_for(&ist, &par, potl, ksqr);
  OK("calc_sigma_E", sep_sigma(c, psitot, ist.mstot, eval));
}

/* ---- filter/ortho.c ------------------------------------------------------ */
long portho(double *psi, double dv, long_st ist) {
  (void)dv; /* main.c normalises with dv right after (filter/main.c:112) */
  sep_ctx *c = ctx_for(&ist, NULL, NULL, NULL);
  long kept = 0;
  OK("portho", sep_ortho(c, psi, ist.mstot, &kept));
  printf("cutoff is %ld\n", kept);
  return kept;
}

/* ---- filter/Hmat.c ------------------------------------------------------- */
void Hmatreal(zomplex *psi, zomplex *phi, double *psi0, double *potl, double *ksqr,
              double *eval, long_st ist, par_st par, fftw_plan_loc planfw, fftw_plan_loc planbw,
              fftw_complex *fftwpsi) {
  (void)psi; (void)phi; (void)planfw; (void)planbw; (void)fftwpsi;
  sep_ctx *c = ctx_for(&ist, &par, potl, ksqr);
  OK("Hmatreal", sep_rayleigh_ritz(c, psi0, ist.mstot, eval));
}

/* ---- filter/coeff.c ------------------------------------------------------ */
void coefficient(zomplex *an, double *samp, double *El, par_st par, long_st ist) {
  const long ms = ist.ms, nc = ist.nc;
  double *re = (double *)malloc(sizeof(double) * (size_t)ms * nc);
  double *im = (double *)malloc(sizeof(double) * (size_t)ms * nc);
  if (!re || !im) compat_fail("coefficient", SEP_ERR_NOMEM);
  OK("coefficient", sep_coefficients(ms, nc, par.dE, par.Vmin, par.dt, El, re, im, samp));
  for (long i = 0; i < ms * nc; i++) {
    an[i].re = re[i];
    an[i].im = im[i];
  }
  free(re);
  free(im);
}
