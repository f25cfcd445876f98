/*
 * sep_oracle.h -- CPU restatement of the reference's filter-diagonalisation
 * path (the filter/ sources), used ONLY as test infrastructure: the parity checker for
 * the CUDA path, the generator of golden vectors, and the timed CPU baseline.
 * The product (libsep_gb300.so) never links, loads or calls anything here.
 *
 * Every function cites the reference lines it restates.  Conventions follow
 * the reference: grids are x-fastest (jxyz = nx*(ny*jz + jy) + jx,
 * filter/init.c:139-141); complex arrays are interleaved {re, im} doubles;
 * real state blocks are state-major (psitot[state*ngrid + g], filter/main.c:86).
 *
 * Parity is pinned: the reference's own sources, compiled by Makefile.ref,
 * reproduce the In13_P16 fixture's eval.dat, and the tests check this
 * restatement against that build and against the fixture.
 */
#ifndef SEP_ORACLE_H
#define SEP_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- random numbers: filter/rand.c:28-66 (ran_nrc) ---------------------- */
typedef struct {
  long idum;   /* the caller's seed / running state, as *idum in ran_nrc */
  long idum2;
  long iy;
  long iv[32];
} orc_rng;

void orc_rng_seed(orc_rng *r, long idum); /* idum <= 0 re-initialises on first draw */
double orc_rng_next(orc_rng *r);
/* filter/init.c:236-251: uniform(-1,1) per point, x fastest, then normalised */
void orc_init_psi(orc_rng *r, long ngrid, double dv, double *psi_re);

/* ---- system set-up: filter/init.c:90-144, filter/read.c:16-30,105-108 ---- */
void orc_center_atoms(long natom, double *rx, double *ry, double *rz);
double orc_box_half(const double *r, long natom); /* rint(0.5*extent + 5) */
void orc_ksqr(long nx, long ny, long nz, double dx, double dy, double dz, double ekinmax,
              double *ksqr);
void orc_shift_table(double *v, long n);
/* filter/init.c:157-182 + filter/interpolate.c:11-23 (+ filterStrainCube
 * per-atom scale, filterStrainCube/interpolate.c:11-25, when scale != NULL) */
void orc_vbuild(long natom, const double *rx, const double *ry, const double *rz,
                const long *type, const double *scale, const double *tab_r,
                const double *tab_v, const long *tab_n, long tab_stride, long nx, long ny,
                long nz, double xmin, double ymin, double zmin, double dx, double dy,
                double dz, double *potl);
/* pseudopotFitting/hamiltonian.c:91-94 and pseudopotFitting/pot.c:35-63 */
double orc_form_factor(double q, const double a[4]);
void orc_form_factor_table(const double a[4], double vol_per_atom, double *r, double *v);

/* ---- Newton interpolation coefficients: filter/coeff.c:16-134 ----------- */
void orc_leja_points(long nc, double *zre, double *zim);
void orc_coefficients(long ms, long nc, double dE, double vmin, double dt, const double *el,
                      double *an_re, double *an_im, double *zn);

/* ---- Hamiltonian and filter: filter/hamiltonian.c, hnorm.c, filter.c ---- */
typedef struct orc_ctx orc_ctx;
orc_ctx *orc_ctx_create(long nx, long ny, long nz, const double *potl, const double *ksqr,
                        double dv);
void orc_ctx_destroy(orc_ctx *c);
/* hpsi = H psi for complex psi (may alias). filter/hamiltonian.c:11-44 */
void orc_hamiltonian(const orc_ctx *c, const double *psi, double *hpsi);
/* psin = dE_1 * H psim1 - (2 + zm1 + vmin dE_1) psim1. filter/hnorm.c:11-39 */
void orc_hnorm(const orc_ctx *c, const double *psim1, double *psin, double dE_1, double vmin,
               double zm1);
/* filter/filter.c:59-83 for one start state (real), psi0: ms x ngrid */
void orc_filter_cycle(const orc_ctx *c, const double *start, const double *an_re,
                      const double *zn, long ms, long nc, double dE_1, double vmin,
                      double *psi0);
/* filter/norm.c:40-54 */
void orc_normalize_all(double *psi, double dv, long m, long ngrid);
/* filter/energy.c:28-49 */
void orc_energy_all(const orc_ctx *c, const double *psi0, long m, double *ene);
/* filter/energy.c:53-83; returns the number of power iterations */
long orc_energy_range(const orc_ctx *c, double vmin, double *emax, double *dE);

/* ---- subspace: filter/ortho.c, Hmat.c, energy.c:88-119 ------------------ */
/* LAPACK comes from an ILP64 OpenBLAS (scipy_ prefix); returns 0 on success */
int orc_lapack_load(const char *path);
long orc_portho(double *psi, long ngrid, long m, double *sv_out);
int orc_hmat(const orc_ctx *c, double *psi, long m, double *eval);
void orc_sigma(const orc_ctx *c, const double *psi, long m, double *sige);

/* filter/main.c:92-98: ns filter cycles over OpenMP threads; returns seconds */
double orc_filter_batch(const orc_ctx *c, long ns, const double *start, const double *an_re,
                        const double *zn, long ms, long nc, double dE_1, double vmin,
                        double *out, int nthreads);

/* ---- whole pipeline (CPU baseline): filter/main.c:64-142 ----------------- */
typedef struct {
  double energy_range_s, filter_s, ortho_s, hmat_s, sigma_s;
  long iters, mkept;
  double emax, dE, dt;
} orc_timing;
/* start: ns x ngrid real start states; psitot out: ns*ms x ngrid.
 * dE <= 0 means: compute it with orc_energy_range.  Returns kept count. */
long orc_pipeline(const orc_ctx *c, long ns, long ms, long nc, const double *el, double vmin,
                  double dE_in, const double *start, double *psitot, double *eval,
                  double *sige, int nthreads, int do_subspace, orc_timing *t);

#ifdef __cplusplus
}
#endif
#endif
