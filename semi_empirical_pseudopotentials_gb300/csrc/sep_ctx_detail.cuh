// sep_ctx_detail.cuh -- context helpers of sep_ctx.cu used by other
// translation units of the library (the spinor path): workspace growth, the
// FP64 Hamiltonian on complex grids, the Hermitian/symmetric eigensolvers and
// the subspace contractions.  Status codes and error strings as sep_ctx.cu.
#pragma once

#include <cuda_runtime.h>

#include "sep_ctx.cuh"

namespace sep {

int cuda_fail(cudaError_t e, const char* what, int line);
int arg_fail(const char* msg);

namespace detail {
void drop_graphs(sep_ctx* c);
// grow a workspace buffer (a reallocation invalidates the context's graphs)
int grow(sep_ctx* c, DevBuf& b, size_t bytes);
size_t free_device_bytes();
// (T + V) applied to nst complex grids in FP64, in chunks through w_fft
int apply_h_chunked(sep_ctx* c, const cx<double>* in, cx<double>* out, long long nst);
// real symmetric eigen-decomposition in place (column-major), w ascending
int syevd(sep_ctx* c, double* d_a, long long m, double* d_w);
int oz_check(sep_ctx* c);
// C (M x Nn) = alpha A B^T, rows K apart; sym: A == B
int sub_gemm_nt(sep_ctx* c, const double* A, const double* B, long long M, long long Nn,
                long long K, double alpha, double* C, bool sym);
// C (M x w) = W (M x K) X[0:K, 0:w] (rows of X ldx apart)
int sub_gemm_nn_ld(sep_ctx* c, const double* W, const double* X, long long M, long long w,
                   long long K, long long ldx, double* C);
}  // namespace detail

}  // namespace sep

#ifndef SEP_DETAIL_MACROS
#define SEP_DETAIL_MACROS
#define SEP_CK(...)                                                                  \
  do {                                                                               \
    cudaError_t _e = (__VA_ARGS__);                                                  \
    if (_e != cudaSuccess) return ::sep::cuda_fail(_e, #__VA_ARGS__, __LINE__);      \
  } while (0)
#define SEP_RET(...)                  \
  do {                                \
    int _r = (__VA_ARGS__);           \
    if (_r != ::sep::kOk) return _r;  \
  } while (0)
#endif
