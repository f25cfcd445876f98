/*
 * mkl.h (shim) -- oracle build only.
 *
 * The reference calls MKL's ILP64 LAPACK (filter/Makefile:5, -DMKL_ILP64):
 * dgesvd_ in filter/ortho.c:32 and dsyev_ in filter/Hmat.c:55, with every
 * integer argument a 64-bit long long.  MKL is not installed here; the same
 * routines come from the ILP64 OpenBLAS that numpy bundles, whose symbols
 * carry a scipy_ prefix and a _64_ suffix and take the Fortran hidden
 * string-length arguments explicitly.  Thread-control calls become no-ops
 * (OpenBLAS threads are set through OPENBLAS_NUM_THREADS).
 */
#ifndef SEP_SHIM_MKL_H
#define SEP_SHIM_MKL_H
#include <stddef.h>
#include <stdlib.h> /* the real mkl.h pulls this in; the reference relies on it */

void scipy_dgesvd_64_(const char *jobu, const char *jobvt, const long long *m,
                      const long long *n, double *a, const long long *lda, double *s,
                      double *u, const long long *ldu, double *vt, const long long *ldvt,
                      double *work, const long long *lwork, long long *info, size_t l1,
                      size_t l2);
void scipy_dsyev_64_(const char *jobz, const char *uplo, const long long *n, double *a,
                     const long long *lda, double *w, double *work, const long long *lwork,
                     long long *info, size_t l1, size_t l2);

static inline void sep_shim_dgesvd(const char *jobu, const char *jobvt, long long *m,
                                   long long *n, double *a, long long *lda, double *s,
                                   double *u, long long *ldu, double *vt, long long *ldvt,
                                   double *work, long long *lwork, long long *info) {
  scipy_dgesvd_64_(jobu, jobvt, m, n, a, lda, s, u, ldu, vt, ldvt, work, lwork, info, 1, 1);
}

static inline void sep_shim_dsyev(const char *jobz, const char *uplo, long long *n, double *a,
                                  long long *lda, double *w, double *work, long long *lwork,
                                  long long *info) {
  scipy_dsyev_64_(jobz, uplo, n, a, lda, w, work, lwork, info, 1, 1);
}

/* complex routines of spinors/filterSpinors (zgesvd_ in ortho.c:27, zheev_
 * in Hmat.c:43); pointer arguments pass through untyped, as MKL's C
 * prototypes accept the reference's own complex type */
typedef struct {
  double real, imag;
} MKL_Complex16;
void scipy_zgesvd_64_(const char *jobu, const char *jobvt, const long long *m,
                      const long long *n, void *a, const long long *lda, double *s, void *u,
                      const long long *ldu, void *vt, const long long *ldvt, void *work,
                      const long long *lwork, double *rwork, long long *info, size_t l1,
                      size_t l2);
void scipy_zheev_64_(const char *jobz, const char *uplo, const long long *n, void *a,
                     const long long *lda, double *w, void *work, const long long *lwork,
                     double *rwork, long long *info, size_t l1, size_t l2);

static inline void sep_shim_zgesvd(const char *jobu, const char *jobvt, const void *m,
                                   const void *n, void *a, const void *lda, double *s, void *u,
                                   const void *ldu, void *vt, const void *ldvt, void *work,
                                   const void *lwork, double *rwork, void *info) {
  scipy_zgesvd_64_(jobu, jobvt, (const long long *)m, (const long long *)n, a,
                   (const long long *)lda, s, u, (const long long *)ldu, vt,
                   (const long long *)ldvt, work, (const long long *)lwork, rwork,
                   (long long *)info, 1, 1);
}

static inline void sep_shim_zheev(const char *jobz, const char *uplo, const void *n, void *a,
                                  const void *lda, double *w, void *work, const void *lwork,
                                  double *rwork, void *info) {
  scipy_zheev_64_(jobz, uplo, (const long long *)n, a, (const long long *)lda, w, work,
                  (const long long *)lwork, rwork, (long long *)info, 1, 1);
}

#define zgesvd_ sep_shim_zgesvd
#define zheev_ sep_shim_zheev
#define dgesvd_ sep_shim_dgesvd
#define dsyev_ sep_shim_dsyev
#define mkl_set_dynamic(x) ((void)(x))
#define mkl_set_num_threads(x) ((void)(x))

#endif
