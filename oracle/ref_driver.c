/*
 * ref_driver.c -- oracle build only: a fixed-seed driver for the reference's
 * own filter sources, compiled unmodified from filter/ (or filterStrainCube/,
 * whose stage functions have the same prototypes).
 *
 * It runs the reference's stages in the order of filter/main.c:19-142:
 *   init_size -> init -> get_energy_range -> dt -> coefficient -> start
 *   states (init_psi) -> filtering (OpenMP over cycles) -> portho ->
 *   normalize_all -> Hmatreal -> normalize_all -> psi.dat -> calc_sigma_E ->
 *   eval.dat
 * and differs from main.c in three ways: the start-state seed comes from the
 * command line instead of the clock (main.c:79 seeds from time()), FFT plans
 * come from the shim, and stage wall times are printed as one JSON line so a
 * caller can time the stages.
 *
 * usage: filter_ref <idum> [nthreads]      (idum < 0, as main.c:79 produces)
 * Reads input.par, conf.par, pot*.par from the working directory and writes
 * the reference's output files there.
 */
#include "fd.h"

#include <stdlib.h>
#include <sys/time.h>

static double wall(void) {
  struct timeval tv;
  gettimeofday(&tv, NULL);
  return (double)tv.tv_sec + 1e-6 * (double)tv.tv_usec;
}

int main(int argc, char *argv[]) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s <idum> [nthreads]\n", argv[0]);
    return 2;
  }
  long seed = strtol(argv[1], NULL, 10);
  par_st par;
  long_st ist;
  init_size(argc, argv, &par, &ist);
  if (argc > 2) ist.nthreads = strtol(argv[2], NULL, 10);

  const long N = ist.ngrid;
  fftw_complex *scratch = fftw_malloc(sizeof(fftw_complex) * N);
  zomplex *psi = calloc(N, sizeof(zomplex));
  zomplex *phi = calloc(N, sizeof(zomplex));
  double *potl = calloc(N, sizeof(double));
  double *ksqr = calloc(N, sizeof(double));
  double *vx = calloc(ist.nx, sizeof(double));
  double *vy = calloc(ist.ny, sizeof(double));
  double *vz = calloc(ist.nz, sizeof(double));
  double *rx = calloc(ist.natom, sizeof(double));
  double *ry = calloc(ist.natom, sizeof(double));
  double *rz = calloc(ist.natom, sizeof(double));
  atm_st *atm = calloc(ist.natom, sizeof(atm_st));
  double *psitot = calloc((size_t)ist.mstot * N, sizeof(double));
  double *eval = calloc(ist.mstot, sizeof(double));
  double *sige = calloc(ist.mstot, sizeof(double));
  double *el = calloc(ist.ms, sizeof(double));
  if (!scratch || !psi || !phi || !potl || !ksqr || !psitot) {
    fprintf(stderr, "allocation failed\n");
    return 1;
  }
  fftw_plan_loc pf, pb;
  double t0 = wall();
  init(potl, vx, vy, vz, ksqr, rx, ry, rz, atm, &par, el, &ist, &pf, &pb, scratch);
  pf = fftw_plan_dft_3d(ist.nz, ist.ny, ist.nx, scratch, scratch, FFTW_FORWARD, 0);
  pb = fftw_plan_dft_3d(ist.nz, ist.ny, ist.nx, scratch, scratch, FFTW_BACKWARD, 0);
  double t1 = wall();
  get_energy_range(psi, phi, potl, vx, vy, vz, ksqr, &par, ist, pf, pb, scratch);
  double t2 = wall();
  par.dt = sqr((double)ist.nc / (2.5 * par.dE));
  zomplex *an = calloc((size_t)ist.nc * ist.ms, sizeof(zomplex));
  double *zn = calloc(ist.nc, sizeof(double));
  coefficient(an, zn, el, par, ist);
  printf("nc = %ld dt = %.17g dE = %.17g Vmin = %.17g seed = %ld\n", ist.nc, par.dt, par.dE,
         par.Vmin, seed);
  fflush(stdout);

  long idum = seed;
  for (long s = 0; s < ist.ns; s++) {
    init_psi(psi, ist, par, &idum);
    for (long e = 0; e < ist.ms; e++)
      for (long g = 0; g < N; g++) psitot[((size_t)s * ist.ms + e) * N + g] = psi[g].re;
  }
  double t3 = wall();
  omp_set_dynamic(0);
  omp_set_num_threads((int)ist.nthreads);
  long s;
#pragma omp parallel for private(s) schedule(dynamic, 1)
  for (s = 0; s < ist.ns; s++) {
    filtering(&psitot[(size_t)s * ist.ms * N], potl, ksqr, an, zn, el, ist, par,
              (long)omp_get_thread_num(), s, &idum);
  }
  double t4 = wall();
  ist.mstot = portho(psitot, par.dv, ist);
  normalize_all(psitot, par.dv, ist.mstot, N, ist.nthreads);
  double t5 = wall();
  Hmatreal(psi, phi, psitot, potl, ksqr, eval, ist, par, pf, pb, scratch);
  normalize_all(psitot, par.dv, ist.mstot, N, ist.nthreads);
  double t6 = wall();
  FILE *fp = fopen("psi.dat", "w");
  fwrite(psitot, sizeof(double), (size_t)ist.mstot * N, fp);
  fclose(fp);
  calc_sigma_E(psi, phi, psitot, potl, ksqr, sige, ist, par, pf, pb, scratch);
  double t7 = wall();
  fp = fopen("eval.dat", "w");
  for (long k = 0; k < ist.mstot; k++) fprintf(fp, "%ld %.16g %g\n", k, eval[k], sige[k]);
  fclose(fp);
  printf("{\"init_s\": %.4f, \"energy_range_s\": %.4f, \"filter_s\": %.4f, \"ortho_s\": %.4f, "
         "\"hmat_s\": %.4f, \"sigma_s\": %.4f, \"mstot\": %ld, \"nthreads\": %ld}\n",
         t1 - t0, t2 - t1, t4 - t3, t5 - t4, t6 - t5, t7 - t6, ist.mstot, ist.nthreads);
  fftw_destroy_plan(pf);
  fftw_destroy_plan(pb);
  return 0;
}
