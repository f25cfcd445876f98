// sep_kernels.cuh -- the non-FFT device work of the filter path: Newton
// accumulation, pair packing, batched reductions and the FP64 contractions of
// the subspace stages.
#pragma once

#include <cuda_runtime.h>

#include "sep_dd.cuh"

namespace sep {

// ---- state packing: real [2B][N] <-> complex [B][N] (odd count: zero imag)
template <typename T, typename TR>
cudaError_t pack_pairs(const TR* real, long long nstates, long long n, cx<T>* out,
                       cudaStream_t s);
template <typename T, typename TR>
cudaError_t unpack_pairs(const cx<T>* in, long long nstates, long long n, TR* real,
                         cudaStream_t s);

// ---- Newton accumulation (filter/filter.c:60-78), blocked over K steps:
//   acc[b][g][c ms + e] (+)= sum_{s<count} an[e nc + j0 + s] * comp_c(hist[slot(j0+s)][b][g])
// hist is a ring of `slots` grids [slots][B][n]; slot(j) = j % slots.  The 2 ms
// accumulators of a point are adjacent; unpack_accumulators writes them out
// state-major, out[(2b + c) ms + e][g] as double (the reference's psitot).
template <typename T, typename TA>
cudaError_t newton_accumulate(const cx<T>* hist, int slots, int B, long long n, long long j0,
                              int count, const TA* an, long long nc, int ms, TA* acc,
                              long long nstates, bool init, cudaStream_t s);

template <typename TA>
cudaError_t unpack_accumulators(const TA* acc, long long B, long long n, int ms,
                                long long nstates, double* out, cudaStream_t s);

// ---- reductions (FP64 sums, deterministic two-level)
// complex pairs: out[b] = (sum x.re y.re, sum x.im y.im) * w
template <typename T>
cudaError_t pair_dots(const cx<T>* x, const cx<T>* y, int B, long long n, double w,
                      double2* out_dev, double* partial, cudaStream_t s);
// real rows: out[m] = sum_g x[m][g] y[m][g] * w
template <typename T>
cudaError_t row_dots(const T* x, const T* y, long long M, long long n, double w,
                     double* out_dev, double* partial, cudaStream_t s);
// rows scaled by 1/sqrt(norm * dv) where norm = sum x^2 (filter/norm.c:40-54)
template <typename T>
cudaError_t normalize_rows(T* x, long long M, long long n, double dv, double* partial,
                           double* norms_dev, cudaStream_t s);
size_t reduce_partial_doubles(long long rows);
// x rows scaled by 1/sqrt(norms[m] * dv): the scaling of normalize_rows with
// norms already computed (applied to a second array that must follow the first)
template <typename T>
cudaError_t scale_rows(T* x, long long M, long long n, const double* norms_dev, double dv,
                       cudaStream_t s);

// ---- FP64 contractions
// C[m][n] = alpha * sum_k A[m][k] B[n][k]   (K contiguous in both; split over K,
// partial tiles summed in a fixed order).  sym: only tiles n0 >= m0, mirrored.
cudaError_t gemm_nt_f64(const double* A, const double* B, long long M, long long Nn,
                        long long K, double alpha, double* C, bool sym, double* work,
                        size_t work_doubles, cudaStream_t s);
size_t gemm_nt_work_doubles(long long M, long long Nn, long long K);
// C[m][n] = sum_k A[m][k] B[k][n] (row-major), C does not alias A or B
cudaError_t gemm_nn_f64(const double* A, const double* B, long long M, long long Nn,
                        long long K, double* C, cudaStream_t s);
// the same with B's rows ldb apart (a column slice of a wider matrix); C is M x Nn dense
cudaError_t gemm_nn_f64_ld(const double* A, const double* B, long long M, long long Nn,
                           long long K, long long ldb, double* C, cudaStream_t s);
// dst[r][c] -= src[r][c] for r < rows, c < w (dst rows ld apart, src dense)
cudaError_t sub_2d_f64(double* dst, long long ld, const double* src, long long rows,
                       long long w, cudaStream_t s);
// rho[g] = dv * sum_k w[k] psi[k][g]^2 (Hellmann-Feynman weights)
cudaError_t weighted_density(const double* psi, const double* w, long long m, long long n,
                             double dv, double* rho, cudaStream_t s);
// A <- (A + A^T) / 2, m x m
cudaError_t symmetrize_f64(double* A, long long m, cudaStream_t s);
// S[l][i] = R[l][i] / sqrt(lam[l]), k x k
cudaError_t scale_rows_isqrt(const double* R, const double* lam, long long k, double* S,
                             cudaStream_t s);
// out = in * f (complex)
template <typename T>
cudaError_t scale_copy(const cx<T>* in, cx<T>* out, long long count, double f, cudaStream_t s);
// out[j][i] = in[i][j]
cudaError_t transpose_f64(const double* in, long long rows, long long cols, double* out,
                          cudaStream_t s);
// W[i][k] = V[i][k] / sqrt(lam[k]) for the kept columns k in [k0, M) (ascending
// eigenvalues), written as rows r = M-1-k (largest first): out[r][i]
cudaError_t scale_eigvecs(const double* V, const double* lam, long long M, long long k0,
                          double* out, cudaStream_t s);
// residual norms: out[m] = sqrt(sum_g (hx[m][g] - e[m] x[m][g])^2 * dv)
cudaError_t residual_norms(const double* x, const double* hx, const double* e, long long M,
                           long long n, double dv, double* out_dev, double* partial,
                           cudaStream_t s);
// residual rows: out[m][g] = hx[m][g] - e[m] x[m][g] (out may alias hx)
cudaError_t residual_rows(const double* x, const double* hx, const double* e, long long M,
                          long long n, double* out, cudaStream_t s);
// precision conversion
cudaError_t convert_f32_to_f64(const float* in, double* out, long long count, cudaStream_t s);
cudaError_t convert_f64_to_f32(const double* in, float* out, long long count, cudaStream_t s);
cudaError_t convert_f64_to_dd(const double* in, ddf* out, long long count, cudaStream_t s);

}  // namespace sep
