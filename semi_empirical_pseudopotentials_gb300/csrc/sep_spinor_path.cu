// sep_spinor_path.cu -- the spinor filter program (the reference's
// spinors/filterSpinors/) on the GPU, in FP64.
//
// A spinor is 2 ngrid complex values: the spin-up grid, then the spin-down
// grid (filterSpinors/hamiltonian.c:38-44).  H = T + V on each component
// grid plus the non-local spin-orbit operator Vso, which couples them
// (sep_spinor.cu).  Stages, in the order of filterSpinors/main.c:84-175:
//   energy range   damped iteration for Emin, power iteration for Emax
//                  (energy.c:49-109), one H apply per iteration;
//   Newton filter  psims[e] = sum_j an[e][j] psi_j, psi_j = (H^ - z_{j-1})
//                  psi_{j-1} (filter.c:48-80).  Each spinor component is one
//                  complex grid of the line-FFT Newton step; Vso psi_{j-1}
//                  enters the x pass's epilogue.  The complex coefficients
//                  accumulate as two real target sets (Re a, Im a) through
//                  the filter's accumulation kernel and are combined once;
//   ortho          filter/ortho.c's two-level Gram scheme on the Hermitian
//                  Gram matrix (in place of zgesvd, ortho.c:5-40);
//   Rayleigh-Ritz  projected H, Hermitian eigensolve, rotation (Hmat.c:5-75);
//                  the Hermitian eigensolves run on the library's symmetric
//                  solver (sep_eigh.cu) through the real embedding
//                  [[Re H, -Im H], [Im H, Re H]] (cuSOLVER's Zheevd with
//                  sep_ctx_set_eigensolver(ctx, 0));
//   sigma          |H psi - E psi| (energy.c:114-145 forms the same
//                  quantity as sqrt(<H^2> - <H>^2)).
// Complex products run on the real subspace contractions: for rows x = a+ib
// stored as interleaved doubles, Re <x|y> = x . y and Im <x|y> = -x . (i y),
// and W X = Re W . X + Im W . (i X), with (i y) the rows (-Im y, Re y).
#include <cuComplex.h>
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/sep_gb300.h"
#include "sep_ctx.cuh"
#include "sep_ctx_detail.cuh"
#include "sep_eigh.cuh"

namespace sep {

cudaError_t spinor_vso_launch(const double* psi, long ngrid, long nsp, long natom, long nnlc,
                              const sep_nlc* nlc, const long* nl, double sigma, double dv,
                              int flagkb, const double* elkb, double* psinl, cudaStream_t st);

namespace {

using detail::apply_h_chunked;
using detail::free_device_bytes;
using detail::grow;
using detail::sub_gemm_nn_ld;
using detail::sub_gemm_nt;

#define CK SEP_CK
#define RET SEP_RET

constexpr int kT = 256;
constexpr double kLevel1 = 2.0e-7;  // singular-value ratio one Gram pass resolves
constexpr double kRatio = 1.0e-10;  // filter/ortho.c:41-46 (filterSpinors/ortho.c)

unsigned blocks(long long n) {
  long long b = (n + kT - 1) / kT;
  return (unsigned)std::max<long long>(1, std::min<long long>(b, 152LL * 32));
}

// y += a x over count doubles
__global__ void k_axpy(double* __restrict__ y, const double* __restrict__ x, double a,
                       long long count) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x)
    y[i] += a * x[i];
}

// out = i x on interleaved complex values: (re, im) -> (-im, re)
__global__ void k_times_i(const double* __restrict__ x, double* __restrict__ out,
                          long long pairs) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < pairs;
       i += (long long)gridDim.x * blockDim.x) {
    const double re = x[2 * i], im = x[2 * i + 1];
    out[2 * i] = -im;
    out[2 * i + 1] = re;
  }
}

// out[i + j m] = re[i n + j] + i im[i n + j] (column-major complex m x n)
__global__ void k_pack_colmajor(const double* __restrict__ re, const double* __restrict__ im,
                                long long m, long long n, cuDoubleComplex* __restrict__ out) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < m * n;
       t += (long long)gridDim.x * blockDim.x) {
    const long long i = t / n, j = t - i * n;
    out[i + j * m] = make_cuDoubleComplex(re[t], im[t]);
  }
}

// A <- (A + A^H) / 2, column-major m x m
__global__ void k_hermitize(cuDoubleComplex* __restrict__ A, long long m) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < m * m;
       t += (long long)gridDim.x * blockDim.x) {
    const long long i = t % m, j = t / m;
    if (i > j) continue;
    const cuDoubleComplex a = A[i + j * m], b = A[j + i * m];
    const double re = 0.5 * (a.x + b.x), im = 0.5 * (a.y - b.y);
    A[i + j * m] = make_cuDoubleComplex(re, im);
    A[j + i * m] = make_cuDoubleComplex(re, -im);
  }
}

// Rotation weights from eigenvectors (column-major V, component i of vector
// j at V[i + j m]): row r of W (k x 2m, real) holds [Re w, Im w] of
// w_i = V_i,j(r) / s_j, for the kept vectors j(r) = m-1-r (largest first,
// count k, mode 1: s = sqrt(lam)) or j(r) = r (mode 0: s = 1, all).
__global__ void k_weights(const cuDoubleComplex* __restrict__ V, const double* __restrict__ lam,
                          long long m, long long k, int mode, double* __restrict__ W) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < k * m;
       t += (long long)gridDim.x * blockDim.x) {
    const long long r = t / m, i = t - r * m;
    const long long j = mode ? m - 1 - r : r;
    const double s = mode ? 1.0 / sqrt(lam[j]) : 1.0;
    const cuDoubleComplex v = V[i + j * m];
    W[r * 2 * m + i] = v.x * s;
    W[r * 2 * m + m + i] = v.y * s;
  }
}

// W (m x 2k) of the projection Y = X - P^T Q: row i holds [Re, Im] of P_li
// (P = <Q_l|X_i>, column-major k x m complex from k_pack_colmajor of Q.X)
__global__ void k_proj_weights(const cuDoubleComplex* __restrict__ P, long long k, long long m,
                               double* __restrict__ W) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < m * k;
       t += (long long)gridDim.x * blockDim.x) {
    const long long i = t / k, l = t - i * k;
    const cuDoubleComplex p = P[l + i * k];
    W[i * 2 * k + l] = p.x;
    W[i * 2 * k + k + l] = p.y;
  }
}

// spinors from the accumulators: acc[(b n + g) 4 ms + q] with the filter
// accumulation's layout for 2 ms real target sets (Re a, then Im a) on slot
// b: q < 2 ms sums over Re psi, q >= 2 ms over Im psi.  Slot b = 2 s + c is
// component c of spinor s; out[((s ms + e) 2 + c) n + g] (complex)
__global__ void k_unpack_spinor(const double* __restrict__ acc, long long slots, long long n,
                                int ms, double* __restrict__ out) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < slots * n;
       t += (long long)gridDim.x * blockDim.x) {
    const long long b = t / n, g = t - b * n;
    const long long s = b / 2, c = b - 2 * s;
    const double* pa = acc + t * (4 * ms);
    for (int e = 0; e < ms; ++e) {
      const double rr = pa[e], ir = pa[ms + e], ri = pa[2 * ms + e], ii = pa[3 * ms + e];
      double* o = out + 2 * (((s * ms + e) * 2 + c) * n + g);
      o[0] = rr - ii;  // Re(a psi) = Re a Re psi - Im a Im psi
      o[1] = ri + ir;  // Im(a psi) = Re a Im psi + Im a Re psi
    }
  }
}

// Vso applied to nsp spinors into out
int vso(sep_ctx* c, const double* psi, long long nsp, double* out) {
  if (nsp > 65535) return arg_fail("spinor path: more than 65535 spinors in one call");
  CK(spinor_vso_launch(psi, (long)c->n, (long)nsp, c->so_natom, c->so_nnlc,
                       c->w_nlc.as<sep_nlc>(), c->w_nl.as<long>(), c->so_sigma, c->dv,
                       c->so_flagkb, c->w_elkb.as<double>(), out, c->stream));
  return kOk;
}

// H psi for nsp spinors: (T + V) on each component grid, plus Vso
int spinor_h(sep_ctx* c, const double* psi, double* out, long long nsp) {
  RET(apply_h_chunked(c, reinterpret_cast<const cx<double>*>(psi),
                      reinterpret_cast<cx<double>*>(out), 2 * nsp));
  const long long L = 4 * c->n;
  for (long long s0 = 0; s0 < nsp; s0 += 4096) {
    const long long k = std::min<long long>(4096, nsp - s0);
    RET(grow(c, c->w_so, sizeof(double) * (size_t)(L * k)));
    RET(vso(c, psi + s0 * L, k, c->w_so.as<double>()));
    k_axpy<<<blocks(L * k), kT, 0, c->stream>>>(out + s0 * L, c->w_so.as<double>(), 1.0, L * k);
    CK(cudaGetLastError());
  }
  return kOk;
}

// M (2m x 2m, symmetric) = [[Re H, -Im H], [Im H, Re H]] for the Hermitian H
// whose upper triangle A holds (column-major): H_ij = A[i + j m] for i <= j,
// conj(A[j + i m]) otherwise
__global__ void k_embed(const cuDoubleComplex* __restrict__ A, long long m,
                        double* __restrict__ M) {
  const long long n2 = 2 * m;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n2 * n2;
       t += (long long)gridDim.x * blockDim.x) {
    const long long r = t / n2, q = t - r * n2;
    const long long i = r % m, j = q % m, bi = r / m, bj = q / m;
    cuDoubleComplex h = (i <= j) ? A[i + j * m] : cuConj(A[j + i * m]);
    M[t] = (bi == bj) ? h.x : (bi == 1 ? h.y : -h.y);
  }
}

// The complex eigenvectors from those of the real embedding: an eigenpair
// (lambda, u + i v) of H gives M the two eigenvectors [u; v] and [-v; u], so
// the real spectrum holds each lambda twice.  Per cluster of equal real
// eigenvalues (2 q of them: q complex eigenvectors), the complex candidates
// u + i v of all 2 q real vectors span the complex eigenspace; q of them are
// chosen by Gram-Schmidt with pivoting on the largest remaining norm, so a
// pair (c, i c) is never taken twice.  vr: the real eigenvectors
// (column-major, 2m x 2m), wr: their eigenvalues ascending; out: column-major
// complex m x m and w (m).  Host arithmetic, O(m^2) per cluster member.
int embed_to_complex(long long m, const std::vector<double>& wr, const std::vector<double>& vr,
                     std::vector<cuDoubleComplex>& out, std::vector<double>& w) {
  const long long n2 = 2 * m;
  double scale = 1.0;
  for (double x : wr) scale = std::max(scale, std::fabs(x));
  const double tol = 1e-10 * scale;
  out.assign((size_t)(m * m), make_cuDoubleComplex(0.0, 0.0));
  w.assign((size_t)m, 0.0);
  long long oc = 0;
  long long i = 0;
  std::vector<std::vector<double>> re, im;
  while (i < n2) {
    long long j = i + 1;
    while (j < n2 && std::fabs(wr[(size_t)j] - wr[(size_t)j - 1]) <= tol) ++j;
    const long long size = j - i, want = size / 2;
    re.assign((size_t)size, std::vector<double>((size_t)m));
    im.assign((size_t)size, std::vector<double>((size_t)m));
    for (long long t = 0; t < size; ++t)
      for (long long r = 0; r < m; ++r) {
        re[(size_t)t][(size_t)r] = vr[(size_t)((i + t) * n2 + r)];
        im[(size_t)t][(size_t)r] = vr[(size_t)((i + t) * n2 + m + r)];
      }
    std::vector<bool> used((size_t)size, false);
    for (long long s = 0; s < want; ++s) {
      long long best = -1;
      double bn = -1.0;
      for (long long t = 0; t < size; ++t) {
        if (used[(size_t)t]) continue;
        double nn = 0.0;
        for (long long r = 0; r < m; ++r)
          nn += re[(size_t)t][(size_t)r] * re[(size_t)t][(size_t)r] +
                im[(size_t)t][(size_t)r] * im[(size_t)t][(size_t)r];
        if (nn > bn) {
          bn = nn;
          best = t;
        }
      }
      if (best < 0 || !(bn > 1e-12) || oc >= m) {
        set_error("spinor path: the real embedding's eigenvectors do not pair up");
        return kErrNumeric;
      }
      used[(size_t)best] = true;
      const double inv = 1.0 / std::sqrt(bn);
      std::vector<double>& qr = re[(size_t)best];
      std::vector<double>& qi = im[(size_t)best];
      for (long long r = 0; r < m; ++r) {
        qr[(size_t)r] *= inv;
        qi[(size_t)r] *= inv;
        out[(size_t)(r + oc * m)] = make_cuDoubleComplex(qr[(size_t)r], qi[(size_t)r]);
      }
      w[(size_t)oc] = wr[(size_t)(i + 2 * s)];
      ++oc;
      // remove q from the others: x -= q <q|x>
      for (long long t = 0; t < size; ++t) {
        if (used[(size_t)t]) continue;
        double pr = 0.0, pi = 0.0;
        for (long long r = 0; r < m; ++r) {
          const double xr = re[(size_t)t][(size_t)r], xi = im[(size_t)t][(size_t)r];
          pr += qr[(size_t)r] * xr + qi[(size_t)r] * xi;
          pi += qr[(size_t)r] * xi - qi[(size_t)r] * xr;
        }
        for (long long r = 0; r < m; ++r) {
          re[(size_t)t][(size_t)r] -= pr * qr[(size_t)r] - pi * qi[(size_t)r];
          im[(size_t)t][(size_t)r] -= pr * qi[(size_t)r] + pi * qr[(size_t)r];
        }
      }
    }
    i = j;
  }
  if (oc != m) {
    set_error("spinor path: the real embedding's eigenvalues do not come in pairs");
    return kErrNumeric;
  }
  return kOk;
}

// complex Hermitian eigensolve (column-major, in place, upper triangle read),
// w ascending.  c->eigensolver 1: the library's solver on the real embedding;
// 0: cuSOLVER's Zheevd.
int heevd(sep_ctx* c, cuDoubleComplex* A, long long m, double* w) {
  if (c->eigensolver == 1) {
    const long long n2 = 2 * m;
    const size_t wd = eigh::work_doubles(n2);
    RET(grow(c, c->w_eigh, sizeof(double) * (wd + (size_t)(n2 * n2) + (size_t)n2)));
    double* work = c->w_eigh.as<double>();
    double* M = work + wd;
    double* wr = M + n2 * n2;
    k_embed<<<blocks(n2 * n2), kT, 0, c->stream>>>(A, m, M);
    CK(cudaGetLastError());
    int bad = 0;
    CK(eigh::solve(M, (int)n2, wr, work, c->stream, &bad));
    if (bad) {
      set_error("spinor path: the QL iteration of a leaf did not converge");
      return kErrSolver;
    }
    std::vector<double> hw((size_t)n2), hv((size_t)(n2 * n2));
    CK(cudaMemcpyAsync(hw.data(), wr, sizeof(double) * n2, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(hv.data(), M, sizeof(double) * n2 * n2, cudaMemcpyDeviceToHost,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
    std::vector<cuDoubleComplex> hc;
    std::vector<double> hwc;
    RET(embed_to_complex(m, hw, hv, hc, hwc));
    CK(cudaMemcpyAsync(A, hc.data(), sizeof(cuDoubleComplex) * m * m, cudaMemcpyHostToDevice,
                       c->stream));
    CK(cudaMemcpyAsync(w, hwc.data(), sizeof(double) * m, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return kOk;
  }
  int lwork = 0;
  if (cusolverDnZheevd_bufferSize(c->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER,
                                  (int)m, A, (int)m, w, &lwork) != CUSOLVER_STATUS_SUCCESS) {
    set_error("spinor path: Hermitian eigensolver workspace query failed");
    return kErrSolver;
  }
  RET(grow(c, c->w_solver, sizeof(cuDoubleComplex) * ((size_t)lwork + 8)));
  cuDoubleComplex* work = c->w_solver.as<cuDoubleComplex>();
  int* info = reinterpret_cast<int*>(work + lwork);
  if (cusolverDnZheevd(c->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, (int)m, A,
                       (int)m, w, work, lwork, info) != CUSOLVER_STATUS_SUCCESS) {
    set_error("spinor path: Hermitian eigensolver failed to start");
    return kErrSolver;
  }
  int h = 0;
  CK(cudaMemcpyAsync(&h, info, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (h != 0) {
    char b[128];
    snprintf(b, sizeof b, "spinor path: Hermitian eigensolver info = %d", h);
    set_error(b);
    return kErrSolver;
  }
  return kOk;
}

// Workspace of the complex subspace steps for up to m spinor rows
struct Cplx {
  sep_ctx* c;
  long long L;
  double* T;             // m x L scratch (i Y, or the stacked [X; i X] second half)
  double* re;            // m x m
  double* im;            // m x m
  cuDoubleComplex* A;    // m x m column-major
  double* lam;           // m
  double* W;             // m x 2m rotation weights
};

int cplx_space(sep_ctx* c, long long m, long long L, Cplx& w) {
  RET(grow(c, c->w_so2, sizeof(double) * (size_t)(2 * m * L)));
  const size_t small = (size_t)m * m * 2 + (size_t)m * m * 2 + m + (size_t)m * 2 * m + 64;
  RET(grow(c, c->w_small, sizeof(double) * small));
  w.c = c;
  w.L = L;
  w.T = c->w_so2.as<double>();
  w.re = c->w_small.as<double>();
  w.im = w.re + (size_t)m * m;
  w.A = reinterpret_cast<cuDoubleComplex*>(w.im + (size_t)m * m);
  w.lam = reinterpret_cast<double*>(w.A + (size_t)m * m);
  w.W = w.lam + m;
  return kOk;
}

// G (mx x my, column-major complex in w.A) = <X_i|Y_j> dv
int cgram(Cplx& w, const double* X, long long mx, const double* Y, long long my, double dv) {
  sep_ctx* c = w.c;
  const bool same = X == Y;
  RET(sub_gemm_nt(c, X, Y, mx, my, w.L, dv, w.re, same));
  k_times_i<<<blocks(my * w.L / 2), kT, 0, c->stream>>>(Y, w.T, my * w.L / 2);
  CK(cudaGetLastError());
  RET(sub_gemm_nt(c, X, w.T, mx, my, w.L, -dv, w.im, false));
  k_pack_colmajor<<<blocks(mx * my), kT, 0, c->stream>>>(w.re, w.im, mx, my, w.A);
  CK(cudaGetLastError());
  return detail::oz_check(c);
}

// out (k rows) = W X with W (k x 2m real: [Re | Im]) and X (m rows); out may
// not alias X.  [X; i X] is stacked in w.T (2 m x L).
int crotate(Cplx& w, const double* Wd, long long k, const double* X, long long m, double* out) {
  sep_ctx* c = w.c;
  const long long L = w.L;
  CK(cudaMemcpyAsync(w.T, X, sizeof(double) * (size_t)(m * L), cudaMemcpyDeviceToDevice,
                     c->stream));
  k_times_i<<<blocks(m * L / 2), kT, 0, c->stream>>>(X, w.T + m * L, m * L / 2);
  CK(cudaGetLastError());
  long long cols = (long long)((size_t)1 << 27) / (sizeof(double) * std::max<long long>(k, 1));
  cols = std::max<long long>(64, std::min<long long>(cols, L));
  RET(grow(c, c->w_tmp, sizeof(double) * (size_t)k * cols));
  for (long long g0 = 0; g0 < L; g0 += cols) {
    const long long wd = std::min<long long>(cols, L - g0);
    RET(sub_gemm_nn_ld(c, Wd, w.T + g0, k, wd, 2 * m, L, c->w_tmp.as<double>()));
    CK(cudaMemcpy2DAsync(out + g0, sizeof(double) * L, c->w_tmp.p, sizeof(double) * wd,
                         sizeof(double) * wd, k, cudaMemcpyDeviceToDevice, c->stream));
  }
  return detail::oz_check(c);
}

int host_lam(sep_ctx* c, const double* d, long long m, std::vector<double>& h) {
  h.resize((size_t)m);
  CK(cudaMemcpyAsync(h.data(), d, sizeof(double) * m, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return kOk;
}

// rows of Q (k x L) <- an orthonormal basis of their span: the eigenvectors
// of Q^H Q dv scaled by lam^-1/2 (all k kept; the rows are linearly
// independent by construction).  Q is overwritten through scratch S (k x L).
int canonical(Cplx& w, double* Q, long long k, double dv, double* S) {
  sep_ctx* c = w.c;
  RET(cgram(w, Q, k, Q, k, dv));
  RET(heevd(c, w.A, k, w.lam));
  k_weights<<<blocks(k * k), kT, 0, c->stream>>>(w.A, w.lam, k, k, 1, w.W);
  CK(cudaGetLastError());
  RET(crotate(w, w.W, k, Q, k, S));
  CK(cudaMemcpyAsync(Q, S, sizeof(double) * (size_t)(k * w.L), cudaMemcpyDeviceToDevice,
                     c->stream));
  return kOk;
}

// X (m rows) -= P^T Q with P = Q X^H dv (k x m): removes span(Q) from X's rows.
// Out-of-place through S (m x L).
int cproject_out(Cplx& w, double* X, long long m, const double* Q, long long k, double dv,
                 double* S) {
  sep_ctx* c = w.c;
  RET(cgram(w, Q, k, X, m, dv));  // P_li = <Q_l|X_i>, column-major k x m in w.A
  k_proj_weights<<<blocks(m * k), kT, 0, c->stream>>>(w.A, k, m, w.W);
  CK(cudaGetLastError());
  RET(crotate(w, w.W, m, Q, k, S));
  k_axpy<<<blocks(m * w.L), kT, 0, c->stream>>>(X, S, -1.0, m * w.L);
  CK(cudaGetLastError());
  return kOk;
}

}  // namespace

// ---------------------------------------------------------------------------
int spinor_set_operator(sep_ctx* c, long natom, long nnlc, const sep_nlc* nlc, const long* nl,
                        double sigma, int flagkb, const double* elkb) {
  if (natom < 0 || nnlc < 0 || (natom > 0 && (!nlc || !nl)) || (flagkb && natom > 0 && !elkb) ||
      (!flagkb && !(sigma > 0.0)) || natom > 0x7fffffff)
    return arg_fail("sep_spinor_set_operator: bad arguments");
  for (long a = 0; a < natom; ++a) {
    if (nl[a] < 0 || nl[a] > nnlc)
      return arg_fail("sep_spinor_set_operator: a neighbour count is outside [0, nnlc]");
    for (long j = 0; j < nl[a]; ++j) {
      const long g = nlc[(size_t)a * nnlc + j].jxyz;
      if (g < 0 || g >= c->n)
        return arg_fail("sep_spinor_set_operator: a neighbour-list point lies outside the grid");
    }
  }
  CK(cudaStreamSynchronize(c->stream));
  RET(grow(c, c->w_nlc, sizeof(sep_nlc) * (size_t)std::max<long>(1, natom * nnlc)));
  RET(grow(c, c->w_nl, sizeof(long) * (size_t)std::max<long>(1, natom)));
  RET(grow(c, c->w_elkb, sizeof(double) * (size_t)std::max<long>(2, 2 * natom)));
  if (natom > 0) {
    CK(cudaMemcpy(c->w_nlc.p, nlc, sizeof(sep_nlc) * (size_t)natom * nnlc,
                  cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->w_nl.p, nl, sizeof(long) * (size_t)natom, cudaMemcpyHostToDevice));
    if (flagkb)
      CK(cudaMemcpy(c->w_elkb.p, elkb, sizeof(double) * 2 * (size_t)natom,
                    cudaMemcpyHostToDevice));
  }
  c->so_natom = natom;
  c->so_nnlc = nnlc;
  c->so_sigma = sigma;
  c->so_flagkb = flagkb ? 1 : 0;
  c->so_ready = true;
  return kOk;
}

int spinor_hamiltonian_device(sep_ctx* c, const double* psi, double* hpsi, long nsp) {
  if (!c->so_ready) return arg_fail("spinor path: no spin-orbit operator set");
  return spinor_h(c, psi, hpsi, nsp);
}

// filterSpinors/energy.c:49-109.  starts: 4 component grids (real, n each):
// the Emin spinor, then the Emax spinor.  One H apply per iteration: H of
// the new iterate serves both its energy and the next step.
int spinor_energy_range_device(sep_ctx* c, const double* starts_host, double tau, double* vmin,
                               double* dE, long* iters) {
  if (!c->so_ready) return arg_fail("spinor path: no spin-orbit operator set");
  const long long n = c->n, L = 4 * n;
  RET(grow(c, c->w_states, sizeof(double) * (size_t)(2 * L)));
  RET(grow(c, c->w_states2, sizeof(double) * (size_t)(2 * L)));
  RET(grow(c, c->w_red, sizeof(double) * (reduce_partial_doubles(1) + 64)));
  double* psi = c->w_states.as<double>();
  double* hp = c->w_states2.as<double>();
  double* part = c->w_red.as<double>();
  double* scal = part + reduce_partial_doubles(1);
  std::vector<double> z((size_t)L, 0.0);
  auto load = [&](int first) -> int {
    for (long long g = 0; g < n; ++g) {
      z[(size_t)(2 * g)] = starts_host[(size_t)(first * n + g)];
      z[(size_t)(2 * (n + g))] = starts_host[(size_t)((first + 1) * n + g)];
    }
    CK(cudaMemcpyAsync(psi, z.data(), sizeof(double) * L, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return kOk;
  };
  auto dot = [&](const double* a, const double* b, double* out) -> int {
    CK(row_dots<double>(a, b, 1, L, c->dv, scal, part, c->stream));
    CK(cudaMemcpyAsync(out, scal, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return kOk;
  };
  auto normalize = [&](double* x) -> int {
    CK(normalize_rows<double>(x, 1, L, c->dv, part, scal, c->stream));
    return kOk;
  };
  long it_total = 0;
  // Emin: phi <- normalise(psi - tau H psi), energy of phi
  RET(load(0));
  double emin = 0.1, old = 0.0;
  long i = 0;
  RET(spinor_h(c, psi, hp, 1));
  while (std::fabs((emin - old) / emin) > 1.0e-6 && i < 500) {
    k_axpy<<<blocks(L), kT, 0, c->stream>>>(psi, hp, -tau, L);  // psi - tau H psi
    CK(cudaGetLastError());
    RET(normalize(psi));
    RET(spinor_h(c, psi, hp, 1));
    old = emin;
    RET(dot(psi, hp, &emin));
    ++i;
  }
  it_total += i;
  // Emax: psi <- normalise(H psi), energy of psi
  RET(load(2));
  double emax = 0.1;
  old = 0.0;
  i = 0;
  RET(spinor_h(c, psi, hp, 1));
  while (std::fabs((emax - old) / emax) > 1.0e-6 && i < 500) {
    CK(cudaMemcpyAsync(psi, hp, sizeof(double) * L, cudaMemcpyDeviceToDevice, c->stream));
    RET(normalize(psi));
    RET(spinor_h(c, psi, hp, 1));
    old = emax;
    RET(dot(psi, hp, &emax));
    ++i;
  }
  it_total += i;
  emax *= 1.2;
  emin -= 0.2 * std::fabs(emin);
  if (!std::isfinite(emin) || !std::isfinite(emax)) {
    set_error("spinor energy range: non-finite energy");
    return kErrNumeric;
  }
  *vmin = emin;
  *dE = emax - emin;
  if (iters) *iters = it_total;
  return kOk;
}

// filterSpinors/filter.c:48-80 for ns spinors (device, 4 n doubles each):
// out (ns x ms x 4 n) = sum_j an[e][j] psi_j.
int spinor_filter_device(sep_ctx* c, const double* d_start, long ns, const double* an_re,
                         const double* an_im, const double* zn, long ms, long nc, double dE_1,
                         double vmin, double* d_out) {
  if (!c->so_ready) return arg_fail("spinor path: no spin-orbit operator set");
  if (ns < 1 || ms < 1 || ms > 16 || nc < 1)
    return arg_fail("spinor filter: need ns, nc >= 1 and 1 <= ms <= 16");
  const long long n = c->n, L = 4 * n;
  int K = std::max(1, std::min<int>(c->block_steps, (int)nc));
  const long ms2 = 2 * ms;
  // per spinor: 2 slots of (K history grids + 1 transform grid), 2 x 2 ms2
  // accumulators per point, and Vso psi
  const size_t per_sp = 2 * (sizeof(cx<double>) * (size_t)n * (K + 1) +
                             sizeof(double) * 2 * (size_t)ms2 * n) +
                        sizeof(double) * (size_t)L;
  const size_t have = c->w_hist.bytes + c->w_fft.bytes + c->w_acc.bytes + c->w_so.bytes;
  long long Bs = (long long)(((size_t)(0.6 * (double)free_device_bytes()) + have) / per_sp);
  if (Bs < 1) return arg_fail("spinor filter: not enough device memory for one spinor");
  Bs = std::min<long long>({Bs, (long long)ns, 32767LL});
  const long long Bc = 2 * Bs;  // complex grids (slots) per chunk
  RET(grow(c, c->w_hist, sizeof(cx<double>) * (size_t)n * K * Bc));
  RET(grow(c, c->w_fft, sizeof(cx<double>) * (size_t)n * Bc));
  RET(grow(c, c->w_acc, sizeof(double) * 2 * (size_t)ms2 * n * Bc));
  RET(grow(c, c->w_so, sizeof(double) * (size_t)L * Bs));
  RET(grow(c, c->w_coef, sizeof(double) * (size_t)ms2 * nc));
  RET(grow(c, c->w_steps, sizeof(double) * 2 * (size_t)nc));
  {
    std::vector<double> a((size_t)ms2 * nc), st(2 * (size_t)nc, 0.0);
    std::memcpy(a.data(), an_re, sizeof(double) * (size_t)ms * nc);
    std::memcpy(a.data() + (size_t)ms * nc, an_im, sizeof(double) * (size_t)ms * nc);
    for (long j = 1; j < nc; ++j) {  // filterSpinors/hnorm.c:5-17
      st[2 * j] = dE_1;
      st[2 * j + 1] = -(2.0 + zn[j - 1] + vmin * dE_1);
    }
    CK(cudaMemcpyAsync(c->w_coef.p, a.data(), sizeof(double) * a.size(), cudaMemcpyHostToDevice,
                       c->stream));
    CK(cudaMemcpyAsync(c->w_steps.p, st.data(), sizeof(double) * st.size(),
                       cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  GridDev<double>& g = c->g64;
  cx<double>* hist = c->w_hist.as<cx<double>>();
  double* acc = c->w_acc.as<double>();
  const double* an = c->w_coef.as<double>();
  for (long long s0 = 0; s0 < ns; s0 += Bs) {
    const long long nsp = std::min<long long>(Bs, ns - s0);
    const int bc = (int)(2 * nsp);
    // slot 0 of the history: the start spinors (component grids in order)
    CK(cudaMemcpyAsync(hist, d_start + s0 * L, sizeof(double) * (size_t)(nsp * L),
                       cudaMemcpyDeviceToDevice, c->stream));
    PassIO<double> io;
    io.data = c->w_fft.as<cx<double>>();
    io.src = hist;
    CK(run_pass<double>(0, kFwd, g, io, bc, c->stream));
    io.src = nullptr;
    io.coefs = c->w_steps.as<double>();
    for (long j = 1; j < nc; ++j) {
      const cx<double>* prev = hist + (long long)((j - 1) % K) * bc * n;
      RET(vso(c, reinterpret_cast<const double*>(prev), nsp, c->w_so.as<double>()));
      CK(run_pass<double>(1, kFwd, g, io, bc, c->stream));
      CK(run_pass<double>(2, kFwdKInv, g, io, bc, c->stream));
      CK(run_pass<double>(1, kInv, g, io, bc, c->stream));
      io.psi_in = prev;
      io.extra = c->w_so.as<cx<double>>();
      io.psi_out = hist + (long long)(j % K) * bc * n;
      io.step = (int)j;
      CK(run_pass<double>(0, (j + 1 < nc) ? kInvEpiFwd : kInvEpi, g, io, bc, c->stream));
      io.extra = nullptr;
      if ((j + 1) % K == 0 || j == nc - 1) {
        const long count = j % K + 1;
        const long j0 = j - count + 1;
        CK(newton_accumulate<double, double>(hist, K, bc, n, j0, (int)count, an, nc, (int)ms2,
                                             acc, 2LL * bc, j0 == 0, c->stream));
      }
    }
    if (nc == 1)
      CK(newton_accumulate<double, double>(hist, K, bc, n, 0, 1, an, nc, (int)ms2, acc,
                                           2LL * bc, true, c->stream));
    k_unpack_spinor<<<blocks((long long)bc * n), kT, 0, c->stream>>>(acc, bc, n, (int)ms,
                                                                    d_out + s0 * ms * L);
    CK(cudaGetLastError());
  }
  return kOk;
}

// filterSpinors/ortho.c:5-40: orthonormalise m spinors in place, keeping the
// directions with singular-value ratio >= 1e-10 (two Gram levels, as the real
// path's ortho).  *mkept rows of psi on return.
int spinor_ortho_device(sep_ctx* c, double* psi, long m, long* mkept) {
  const long long L = 4 * c->n;
  const double dv = c->dv;
  Cplx w;
  RET(cplx_space(c, m, L, w));
  RET(grow(c, c->w_states, sizeof(double) * (size_t)(m * L)));   // Q
  RET(grow(c, c->w_so3, sizeof(double) * (size_t)(m * L)));       // scratch rows
  double* Q = c->w_states.as<double>();
  double* S = c->w_so3.as<double>();
  RET(cgram(w, psi, m, psi, m, dv));
  RET(heevd(c, w.A, m, w.lam));
  std::vector<double> hl;
  RET(host_lam(c, w.lam, m, hl));
  const double top = hl[(size_t)m - 1];
  if (!(top > 0.0) || !std::isfinite(top)) {
    set_error("spinor ortho: the states are zero or not finite");
    return kErrNumeric;
  }
  long k0 = 0;
  while (k0 < m && !(std::sqrt(std::max(hl[(size_t)k0], 0.0) / top) >= kLevel1)) ++k0;
  const long k1 = m - k0;
  k_weights<<<blocks((long long)k1 * m), kT, 0, c->stream>>>(w.A, w.lam, m, k1, 1, w.W);
  CK(cudaGetLastError());
  RET(crotate(w, w.W, k1, psi, m, Q));
  RET(canonical(w, Q, k1, dv, S));
  long k2 = 0;
  if (k0 > 0) {
    // level 2: the part of psi outside span(Q1), projected twice
    RET(cproject_out(w, psi, m, Q, k1, dv, S));
    RET(cproject_out(w, psi, m, Q, k1, dv, S));
    RET(cgram(w, psi, m, psi, m, dv));
    RET(heevd(c, w.A, m, w.lam));
    RET(host_lam(c, w.lam, m, hl));
    long r0 = m;
    while (r0 > 0 && m - r0 < k0 && std::sqrt(std::max(hl[(size_t)r0 - 1], 0.0) / top) >= kRatio)
      --r0;
    k2 = m - r0;
    if (k2 > 0) {
      // the k2 largest of the remainder (kept rows m-1 .. r0), into Q's tail
      k_weights<<<blocks((long long)k2 * m), kT, 0, c->stream>>>(w.A, w.lam, m, k2, 1, w.W);
      CK(cudaGetLastError());
      double* Q2 = Q + (size_t)k1 * L;
      RET(crotate(w, w.W, k2, psi, m, Q2));
      RET(cproject_out(w, Q2, k2, Q, k1, dv, S));
      RET(canonical(w, Q2, k2, dv, S));
    }
  }
  const long k = k1 + k2;
  CK(cudaMemcpyAsync(psi, Q, sizeof(double) * (size_t)(k * L), cudaMemcpyDeviceToDevice,
                     c->stream));
  *mkept = k;
  return kOk;
}

// filterSpinors/Hmat.c:5-75: H_ij = <psi_i|H psi_j> dv, its Hermitian part
// diagonalised, psi rotated onto the eigenvectors (eval ascending, host);
// hpsi (m x L, device) receives H psi of the rotated states.
int spinor_rr_device(sep_ctx* c, double* psi, long m, double* eval, double* hpsi) {
  const long long L = 4 * c->n;
  Cplx w;
  RET(cplx_space(c, m, L, w));
  RET(grow(c, c->w_so3, sizeof(double) * (size_t)(m * L)));
  double* S = c->w_so3.as<double>();
  RET(spinor_h(c, psi, hpsi, m));
  RET(cgram(w, psi, m, hpsi, m, c->dv));
  k_hermitize<<<blocks((long long)m * m), kT, 0, c->stream>>>(w.A, m);
  CK(cudaGetLastError());
  RET(heevd(c, w.A, m, w.lam));
  // new state j = sum_i V_ij psi_i (mode 0: all, ascending)
  k_weights<<<blocks((long long)m * m), kT, 0, c->stream>>>(w.A, w.lam, m, m, 0, w.W);
  CK(cudaGetLastError());
  RET(crotate(w, w.W, m, psi, m, S));
  CK(cudaMemcpyAsync(psi, S, sizeof(double) * (size_t)(m * L), cudaMemcpyDeviceToDevice,
                     c->stream));
  RET(crotate(w, w.W, m, hpsi, m, S));
  CK(cudaMemcpyAsync(hpsi, S, sizeof(double) * (size_t)(m * L), cudaMemcpyDeviceToDevice,
                     c->stream));
  CK(cudaMemcpyAsync(eval, w.lam, sizeof(double) * m, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return kOk;
}

// filterSpinors/main.c:84-175 from given start spinors (host, ns x 4 n).
int spinor_pipeline_device(sep_ctx* c, const double* start, long ns, const double* el, long ms,
                           long nc, double vmin, double dE, double* psi_out, double* eval,
                           double* sige, long* mkept, sep_timing* tm) {
  if (!c->so_ready) return arg_fail("spinor path: no spin-orbit operator set");
  const long long n = c->n, L = 4 * n;
  const long m = ns * ms;
  sep_timing t;
  std::memset(&t, 0, sizeof t);
  cudaEvent_t ev[6];
  for (auto& e : ev) CK(cudaEventCreate(&e));
  RET(grow(c, c->w_start, sizeof(double) * (size_t)(ns * L)));
  RET(grow(c, c->w_out, sizeof(double) * (size_t)(m * L)));
  CK(cudaMemcpyAsync(c->w_start.p, start, sizeof(double) * (size_t)(ns * L),
                     cudaMemcpyHostToDevice, c->stream));
  CK(cudaEventRecord(ev[0], c->stream));
  if (!(dE > 0.0)) {
    // init_psi draws four component grids from the fixed seed (energy.c:49-109)
    std::vector<double> starts((size_t)(4 * n));
    host::Rand r(-874917403);
    for (int q = 0; q < 4; ++q) host::init_psi(r, n, c->dv, starts.data() + (size_t)q * n);
    RET(spinor_energy_range_device(c, starts.data(), 0.025, &vmin, &dE, &t.power_iterations));
  }
  CK(cudaEventRecord(ev[1], c->stream));
  const double dt = ((double)nc / (2.5 * dE)) * ((double)nc / (2.5 * dE));  // main.c:95
  std::vector<double> an_re((size_t)ms * nc), an_im((size_t)ms * nc), zn((size_t)nc);
  host::coefficients(ms, nc, dE, vmin, dt, el, an_re.data(), an_im.data(), zn.data());
  double* psi = c->w_out.as<double>();
  RET(spinor_filter_device(c, c->w_start.as<double>(), ns, an_re.data(), an_im.data(),
                           zn.data(), ms, nc, 4.0 / dE, vmin, psi));
  RET(grow(c, c->w_red, sizeof(double) * (reduce_partial_doubles(m) + 2 * (size_t)m + 64)));
  double* part = c->w_red.as<double>();
  double* norms = part + reduce_partial_doubles(m);
  CK(normalize_rows<double>(psi, m, L, c->dv, part, norms, c->stream));  // filter.c:32
  CK(cudaEventRecord(ev[2], c->stream));
  long k = 0;
  RET(spinor_ortho_device(c, psi, m, &k));
  CK(normalize_rows<double>(psi, k, L, c->dv, part, norms, c->stream));  // main.c:143
  CK(cudaEventRecord(ev[3], c->stream));
  RET(grow(c, c->w_hpsi, sizeof(double) * (size_t)(k * L)));
  double* hpsi = c->w_hpsi.as<double>();
  RET(spinor_rr_device(c, psi, k, eval, hpsi));
  CK(normalize_rows<double>(psi, k, L, c->dv, part, norms, c->stream));  // main.c:154
  CK(scale_rows<double>(hpsi, k, L, norms, c->dv, c->stream));
  CK(cudaEventRecord(ev[4], c->stream));
  double* e = norms + m;
  CK(row_dots<double>(psi, hpsi, k, L, c->dv, e, part, c->stream));
  CK(residual_norms(psi, hpsi, e, k, L, c->dv, norms, part, c->stream));
  CK(cudaMemcpyAsync(sige, norms, sizeof(double) * k, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaEventRecord(ev[5], c->stream));
  if (psi_out)
    CK(cudaMemcpyAsync(psi_out, psi, sizeof(double) * (size_t)(k * L), cudaMemcpyDeviceToHost,
                       c->stream));
  CK(cudaStreamSynchronize(c->stream));
  float ms_[5];
  for (int i = 0; i < 5; ++i) CK(cudaEventElapsedTime(&ms_[i], ev[i], ev[i + 1]));
  for (auto& x : ev) cudaEventDestroy(x);
  t.energy_range_s = ms_[0] * 1e-3;
  t.filter_s = ms_[1] * 1e-3;
  t.ortho_s = ms_[2] * 1e-3;
  t.rayleigh_ritz_s = ms_[3] * 1e-3;
  t.sigma_s = ms_[4] * 1e-3;
  t.total_s = t.energy_range_s + t.filter_s + t.ortho_s + t.rayleigh_ritz_s + t.sigma_s;
  t.mkept = k;
  t.dE = dE;
  t.dt = dt;
  t.emax = vmin + dE;
  t.h_applies = (long)t.power_iterations + 2 + (long)ns * (nc - 1) + k;
  *mkept = k;
  if (tm) *tm = t;
  return kOk;
}

}  // namespace sep

// ---------------------------------------------------------------------------
// C ABI (include/sep_gb300.h): host arrays in and out.
namespace {

int spin_ctx(sep_ctx* c) {
  if (!c) return sep::arg_fail("null context");
  if (!c->have_pot) return sep::arg_fail("the context has no potential yet");
  SEP_CK(cudaSetDevice(c->device));
  return sep::kOk;
}

int spin_upload(sep_ctx* c, sep::DevBuf& b, const double* h, size_t count) {
  SEP_RET(sep::detail::grow(c, b, sizeof(double) * count));
  SEP_CK(cudaMemcpyAsync(b.p, h, sizeof(double) * count, cudaMemcpyHostToDevice, c->stream));
  return sep::kOk;
}

}  // namespace

extern "C" {

int sep_spinor_set_operator(sep_ctx* ctx, long natom, long nnlc, const sep_nlc* nlc,
                            const long* nl, double sigma, int flagkb, const double* elkb) {
  SEP_RET(spin_ctx(ctx));
  return sep::spinor_set_operator(ctx, natom, nnlc, nlc, nl, sigma, flagkb, elkb);
}

int sep_spinor_hamiltonian(sep_ctx* ctx, const double* psi, double* hpsi, long nspinors) {
  SEP_RET(spin_ctx(ctx));
  if (!psi || !hpsi || nspinors < 1) return sep::arg_fail("sep_spinor_hamiltonian: bad argument");
  const size_t cnt = 4 * (size_t)ctx->n * nspinors;
  SEP_RET(spin_upload(ctx, ctx->w_start, psi, cnt));
  SEP_RET(sep::detail::grow(ctx, ctx->w_out, sizeof(double) * cnt));
  SEP_RET(sep::spinor_hamiltonian_device(ctx, ctx->w_start.as<double>(), ctx->w_out.as<double>(),
                                         nspinors));
  SEP_CK(cudaMemcpyAsync(hpsi, ctx->w_out.p, sizeof(double) * cnt, cudaMemcpyDeviceToHost,
                         ctx->stream));
  SEP_CK(cudaStreamSynchronize(ctx->stream));
  return sep::kOk;
}

int sep_spinor_energy_range(sep_ctx* ctx, double* vmin, double* dE, long* iters) {
  SEP_RET(spin_ctx(ctx));
  if (!vmin || !dE) return sep::arg_fail("sep_spinor_energy_range: null argument");
  const long long n = ctx->n;
  std::vector<double> starts((size_t)(4 * n));
  sep::host::Rand r(-874917403);
  for (int q = 0; q < 4; ++q) sep::host::init_psi(r, n, ctx->dv, starts.data() + (size_t)q * n);
  return sep::spinor_energy_range_device(ctx, starts.data(), 0.025, vmin, dE, iters);
}

int sep_spinor_filter(sep_ctx* ctx, const double* start, long ns, const double* an_re,
                      const double* an_im, const double* zn, long ms, long nc, double dE_1,
                      double vmin, double* out) {
  SEP_RET(spin_ctx(ctx));
  if (!start || !an_re || !an_im || !zn || !out || ns < 1 || ms < 1 || nc < 1)
    return sep::arg_fail("sep_spinor_filter: bad argument");
  const size_t L = 4 * (size_t)ctx->n;
  SEP_RET(spin_upload(ctx, ctx->w_start, start, L * ns));
  SEP_RET(sep::detail::grow(ctx, ctx->w_out, sizeof(double) * L * ns * ms));
  SEP_RET(sep::spinor_filter_device(ctx, ctx->w_start.as<double>(), ns, an_re, an_im, zn, ms, nc,
                                    dE_1, vmin, ctx->w_out.as<double>()));
  SEP_CK(cudaMemcpyAsync(out, ctx->w_out.p, sizeof(double) * L * ns * ms,
                         cudaMemcpyDeviceToHost, ctx->stream));
  SEP_CK(cudaStreamSynchronize(ctx->stream));
  return sep::kOk;
}

int sep_spinor_pipeline(sep_ctx* ctx, const double* start, long ns, const double* el, long ms,
                        long nc, double vmin, double dE, double* psi_out, double* eval,
                        double* sige, long* mkept, sep_timing* timing) {
  SEP_RET(spin_ctx(ctx));
  if (!start || !el || !eval || !sige || !mkept || ns < 1 || ms < 1 || nc < 1)
    return sep::arg_fail("sep_spinor_pipeline: bad argument");
  return sep::spinor_pipeline_device(ctx, start, ns, el, ms, nc, vmin, dE, psi_out, eval, sige,
                                     mkept, timing);
}

}  // extern "C"
