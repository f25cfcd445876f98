/* mkl_lapacke.h (shim) -- oracle build only; filterStrainCube/fd.h:15
 * includes it but only uses the Fortran-style dgesvd_/dsyev_ of mkl.h. */
#ifndef SEP_SHIM_MKL_LAPACKE_H
#define SEP_SHIM_MKL_LAPACKE_H
#include "mkl.h"
#endif
