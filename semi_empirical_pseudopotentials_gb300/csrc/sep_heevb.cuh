// sep_heevb.cuh -- the lowest eigenpairs of many small Hermitian matrices
// (one CTA per matrix): Householder tridiagonalisation, bisection, inverse
// iteration and back-transformation (see sep_heevb.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace sep {
namespace hb {

constexpr int kMaxWanted = 64;  // eigenpairs per matrix

struct Work {
  double* d = nullptr;       // tridiagonal diagonal (nmat x n)
  double* e = nullptr;       // off-diagonal
  double2* tau = nullptr;    // reflector scalars
  double* tnorm = nullptr;   // |T|_1 per matrix
  int* info = nullptr;       // eigenvectors whose inverse iteration did not grow
  double* z = nullptr;       // eigenvectors of T (nmat x nw x n)
  double2* x = nullptr;      // eigenvectors of A (nmat x nw x n)
  double* scratch = nullptr; // inverse-iteration rows and vectors
};

bool supported(int n, int nw);
size_t work_bytes(int n, int nmat, int nw);
// A: nmat Hermitian matrices of order n, column-major, both triangles, one
// after another; destroyed.  w (nmat x n): the lowest nw eigenvalues of each
// ascending, NaN after them.  With vectors, the matching unit eigenvectors in
// the first nw columns of each matrix.
cudaError_t lowest(double2* A, int n, int nmat, int nw, bool vectors, double* w, void* work,
                   cudaStream_t s);
// eigenvectors (all matrices) whose inverse iteration never reached the growth test
cudaError_t failed_vectors(const void* work, int n, int nmat, int nw, int* host_count,
                           cudaStream_t s);

}  // namespace hb
}  // namespace sep
