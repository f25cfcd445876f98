/*
 * sep_fd_compat.h -- the reference's own filter entry points, backed by the
 * GPU (libsep_fdcompat.so over libsep_gb300.so).
 *
 * Same symbol names, argument lists and struct layouts as the reference's
 * filter/fd.h:17-36 and fd.h:97-140, so the reference's filter/main.c (and
 * its init.c, read.c, interpolate.c, rand.c, size.c, write.c, nerror.c)
 * links against this library in place of hamiltonian.c, hnorm.c, filter.c,
 * energy.c, norm.c, ortho.c, Hmat.c and coeff.c.  The FFT plan and scratch
 * arguments are accepted and ignored.  Errors end the program like the
 * reference's nerror (filter/nerror.c:9-16): the message goes to ./error and
 * the exit status is 1.
 *
 * Do not include this header together with the reference's fd.h: both
 * declare the same types.  It documents the ABI for callers written anew.
 */
#ifndef SEP_FD_COMPAT_H
#define SEP_FD_COMPAT_H

#ifdef __cplusplus
extern "C" {
#endif

/* filter/fd.h:17-19 */
typedef struct st0 {
  double re, im;
} zomplex;

/* filter/fd.h:23-27 */
typedef struct st1 {
  double dx, dy, dz, dr, dkx, dky, dkz, dv, dt;
  double xmin, xmax, ymin, ymax, zmin, zmax;
  double Vmin, Vmax, dE, dE_1, Elmin, Elmax, Ekinmax;
} par_st;

/* filter/fd.h:29-36 */
typedef struct st4 {
  long natom, lumo, homo;
  long ms, ns, nc, npot, mstot;
  long nx, ny, nz, ngrid;
  long natomtype;
  long nthreads;
  double nx_1, ny_1, nz_1;
} long_st;

/* FFTW's plan and complex types, pointer- and layout-compatible */
typedef void *fftw_plan_loc;
typedef double fftw_complex[2];

/* filter/hamiltonian.c:27-44: psi <- T psi */
void kinetic(zomplex *psi, double *ksqr, fftw_plan_loc planfw, fftw_plan_loc planbw,
             fftw_complex *fftwpsi, long_st ist);
/* filter/hamiltonian.c:11-23: phi <- H phi, psi <- the old phi */
void hamiltonian(zomplex *phi, zomplex *psi, double *potl, double *ksqr, long_st ist,
                 par_st par, fftw_plan_loc planfw, fftw_plan_loc planbw, fftw_complex *fftwpsi);
/* filter/hnorm.c:29-39: phi <- T phi + V psi */
void hamiltonian_norm(zomplex *psi, zomplex *phi, double *potl, double *ksqr, long_st ist,
                      par_st par, fftw_plan_loc planfw, fftw_plan_loc planbw,
                      fftw_complex *fftwpsi);
/* filter/hnorm.c:11-25: psin <- dE_1 H psim1 - (2 + zm1 + Vmin dE_1) psim1 */
void hnorm(zomplex *psim1, zomplex *psin, double *potl, double *ksqr, par_st par, double zm1,
           long_st ist, fftw_plan_loc planfw, fftw_plan_loc planbw, fftw_complex *fftwpsi);
/* filter/filter.c:59-83: psi0[e] = sum_j Re(an[nc e + j]) Re psi_j */
void filter(zomplex *psin, zomplex *psim1, double *psi0, double *potl, double *ksqr, par_st par,
            zomplex *an, double *zn, long_st ist, fftw_plan_loc planfw, fftw_plan_loc planbw,
            fftw_complex *fftwpsi, long tid, long jns);
/* filter/filter.c:11-55: one cycle, writes eval-filt-<tid>-<jns>.dat and
 * psi-filt-<tid>-<jns>.dat as the reference does */
void filtering(double *psitot, double *potl, double *ksqr, zomplex *an, double *zn, double *el,
               long_st ist, par_st par, long tid, long jns, long *idum);
/* filter/norm.c:9-54 */
double norm(zomplex *psi, double dr, long ngrid, long nthreads);
double normalize(zomplex *psi, double dr, long ngrid, long nthreads);
void normalize_all(double *psi, double dr, long ms, long ngrid, long nthreads);
/* filter/energy.c:11-119 */
double energy(zomplex *psi, zomplex *phi, double *potl, double *ksqr, long_st ist, par_st par,
              fftw_plan_loc planfw, fftw_plan_loc planbw, fftw_complex *fftwpsi);
void energy_all(zomplex *psi, zomplex *phi, double *psi0, double *potl, double *ksqr,
                double *ene, long_st ist, par_st par, fftw_plan_loc planfw,
                fftw_plan_loc planbw, fftw_complex *fftwpsi);
void get_energy_range(zomplex *psi, zomplex *phi, double *potl, double *vx, double *vy,
                      double *vz, double *ksqr, par_st *par, long_st ist, fftw_plan_loc planfw,
                      fftw_plan_loc planbw, fftw_complex *fftwpsi);
void calc_sigma_E(zomplex *psi, zomplex *phi, double *psitot, double *potl, double *ksqr,
                  double *eval, long_st ist, par_st par, fftw_plan_loc planfw,
                  fftw_plan_loc planbw, fftw_complex *fftwpsi);
/* filter/ortho.c:11-52 */
long portho(double *psi, double dv, long_st ist);
/* filter/Hmat.c:11-86 */
void Hmatreal(zomplex *psi, zomplex *phi, double *psi0, double *potl, double *ksqr,
              double *eval, long_st ist, par_st par, fftw_plan_loc planfw, fftw_plan_loc planbw,
              fftw_complex *fftwpsi);
/* filter/coeff.c:16-63 */
void coefficient(zomplex *an, double *samp, double *El, par_st par, long_st ist);

#ifdef __cplusplus
}
#endif
#endif
