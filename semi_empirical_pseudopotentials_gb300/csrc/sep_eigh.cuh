// sep_eigh.cuh -- the library's FP64 symmetric eigensolver (sep_eigh.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace sep {
namespace eigh {
// device workspace (doubles) of solve() for an n x n matrix
size_t work_doubles(long long n);
// A (n x n symmetric, device) <- eigenvectors as columns (column-major),
// w (device, n) <- eigenvalues ascending; work: work_doubles(n) doubles.
// Synchronises the stream (the divide-and-conquer merges sort on the host).
// *bad != 0 when a leaf's QL iteration did not converge.  stage_ms (3, may
// be null): device times of the tridiagonalisation, the divide and conquer
// and the back-transformation.
cudaError_t solve(double* A, int n, double* w, double* work, cudaStream_t s, int* bad,
                  double* stage_ms = nullptr);
}  // namespace eigh
}  // namespace sep
