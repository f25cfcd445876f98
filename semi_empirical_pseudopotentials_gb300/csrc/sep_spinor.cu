// sep_spinor.cu -- the non-local spin-orbit operator of the spinor filter
// (the reference's spinors/filterSpinors/), |psinl> = Vso |psi>, on the GPU.
//
// Spinors are 2 ngrid complex values, the spin-up grid then the spin-down
// grid (filterSpinors/hamiltonian.c:38-44).  Each atom acts on the grid
// points of its neighbour list (nlc_st entries, filterSpinors/fd.h:55-60;
// nl[a] used of nnlc per atom); the atoms' contributions add up.
//
// Gaussian form (filterSpinors/hamiltonian.c:81-190): for each point j1 of an
// atom, six sums over the atom's points j2 of
//   K(j1, j2) conj(Y_m(j2)) psi_s(j2),
//   K = (Vr1 + Vr2)/2 exp(-((r1 - r2) sigma_1)^2) / ((r2_1 + r2_2)/2),
// combined with tmp Y_m(j1), tmp = 0.5 dv / sqrt(2 pi sigma^2).  One CTA per
// atom; the j2 points are staged through shared memory in tiles of 256 with
// conj(Y) psi already formed, so each pair costs one exp and 12 FMAs.
// Kleinman-Bylander form (filterSpinors/hamiltonian.c:193-401): twelve
// projections per atom (block reduction), scaled by Elkb dv, then spread back
// over the atom's points with the reference's coefficients, term by term.
// Contributions of overlapping atoms are added with atomicAdd.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <string>

#include "../../include/sep_gb300.h"

namespace sep {
void set_error(const std::string& msg);
}

namespace {

constexpr int kT = 256;
constexpr double kTwoPi = 6.28318530717958647692;  // filterSpinors/fd.h TWOPI

int fail(int status, const std::string& msg) {
  sep::set_error(msg);
  return status;
}

#define SK(...)                                                                      \
  do {                                                                               \
    cudaError_t _e = (__VA_ARGS__);                                                  \
    if (_e != cudaSuccess) {                                                         \
      char _b[320];                                                                  \
      snprintf(_b, sizeof _b, "CUDA error %d (%s) at sep_spinor.cu:%d", (int)_e,     \
               cudaGetErrorString(_e), __LINE__);                                    \
      return fail(_e == cudaErrorMemoryAllocation ? SEP_ERR_NOMEM : SEP_ERR_CUDA, _b); \
    }                                                                                \
  } while (0)

struct C2 {
  double re, im;
};
__device__ __forceinline__ C2 ld(const double* p) { return {p[0], p[1]}; }
// conj(y) psi, as the reference forms it (hamiltonian.c:139-140)
__device__ __forceinline__ C2 conj_mul(C2 y, C2 p) {
  return {y.re * p.re + y.im * p.im, y.re * p.im - y.im * p.re};
}
__device__ __forceinline__ C2 mul(C2 a, C2 b) {
  return {a.re * b.re - a.im * b.im, a.im * b.re + a.re * b.im};
}
__device__ __forceinline__ C2 scale(double s, C2 a) { return {s * a.re, s * a.im}; }
__device__ __forceinline__ C2 add(C2 a, C2 b) { return {a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ C2 sub(C2 a, C2 b) { return {a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ void atomic_add(double* p, C2 v) {
  atomicAdd(p, v.re);
  atomicAdd(p + 1, v.im);
}

// sums index: 0 y11 up, 1 y10 up, 2 y1_1 up, 3 y11 dn, 4 y10 dn, 5 y1_1 dn
// grid: x = atom, y = spinor of the batch (spinors 4 ngrid doubles apart)
__global__ void __launch_bounds__(kT) k_vso_gauss(const double* __restrict__ psi, long ngrid,
                                                  long nnlc, const sep_nlc* __restrict__ nlc,
                                                  const long* __restrict__ nl, double tmp,
                                                  double sigma_1, double* __restrict__ out) {
  __shared__ double sr[kT], sr2[kT], svr[kT];
  __shared__ C2 sx[6][kT];
  const long a = blockIdx.x;
  psi += (size_t)blockIdx.y * 4 * (size_t)ngrid;
  out += (size_t)blockIdx.y * 4 * (size_t)ngrid;
  const long n = nl[a];
  const sep_nlc* base = nlc + a * nnlc;
  const int tid = threadIdx.x;
  const double sqrttwo = sqrt(2.0);
  for (long j1b = 0; j1b < n; j1b += kT) {
    const long j1 = j1b + tid;
    const bool act = j1 < n;
    double r1 = 0.0, r21 = 1.0, vr1 = 0.0;
    if (act) {
      r1 = base[j1].r;
      r21 = base[j1].r2;
      vr1 = base[j1].Vr;
    }
    C2 acc[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) acc[m] = {0.0, 0.0};
    for (long t0 = 0; t0 < n; t0 += kT) {
      __syncthreads();
      const long j2 = t0 + tid;
      if (j2 < n) {
        const sep_nlc& e = base[j2];
        const C2 up = ld(psi + 2 * e.jxyz), dn = ld(psi + 2 * (ngrid + e.jxyz));
        const C2 y11 = ld(e.y11), y10 = ld(e.y10), y1_1 = ld(e.y1_1);
        sr[tid] = e.r;
        sr2[tid] = e.r2;
        svr[tid] = e.Vr;
        sx[0][tid] = conj_mul(y11, up);
        sx[1][tid] = conj_mul(y10, up);
        sx[2][tid] = conj_mul(y1_1, up);
        sx[3][tid] = conj_mul(y11, dn);
        sx[4][tid] = conj_mul(y10, dn);
        sx[5][tid] = conj_mul(y1_1, dn);
      }
      __syncthreads();
      if (act) {
        const int cnt = (int)((n - t0) < kT ? (n - t0) : kT);
        for (int jj = 0; jj < cnt; ++jj) {
          const double d = (r1 - sr[jj]) * sigma_1;
          const double k = 0.5 * (vr1 + svr[jj]) * exp(-(d * d)) / (0.5 * (r21 + sr2[jj]));
#pragma unroll
          for (int m = 0; m < 6; ++m) {
            acc[m].re += k * sx[m][jj].re;
            acc[m].im += k * sx[m][jj].im;
          }
        }
      }
    }
    if (act) {
      const sep_nlc& e = base[j1];
      const C2 t11 = scale(tmp, ld(e.y11)), t10 = scale(tmp, ld(e.y10)),
               t1_1 = scale(tmp, ld(e.y1_1));
      // hamiltonian.c:167-186
      const C2 up = add(sub(mul(t11, acc[0]), mul(t1_1, acc[2])),
                        scale(sqrttwo, add(mul(t10, acc[3]), mul(t1_1, acc[4]))));
      const C2 dn = add(sub(scale(-1.0, mul(t11, acc[3])), mul(t1_1, acc[5])),
                        scale(sqrttwo, add(mul(t10, acc[2]), mul(t11, acc[1]))));
      atomic_add(out + 2 * e.jxyz, up);
      atomic_add(out + 2 * (ngrid + e.jxyz), dn);
    }
  }
}

// projections p[g][m][s] (g: 0 G1, 1 G_2; m: 0 y10, 1 y11, 2 y1_1; s: 0 up, 1 dn)
__global__ void __launch_bounds__(kT) k_vso_kb(const double* __restrict__ psi, long ngrid,
                                               long nnlc, const sep_nlc* __restrict__ nlc,
                                               const long* __restrict__ nl,
                                               const double* __restrict__ elkb, long natom,
                                               double dv, double* __restrict__ out) {
  __shared__ double red[kT / 32][24];
  __shared__ double proj[24];
  const long a = blockIdx.x;
  psi += (size_t)blockIdx.y * 4 * (size_t)ngrid;
  out += (size_t)blockIdx.y * 4 * (size_t)ngrid;
  const long n = nl[a];
  const sep_nlc* base = nlc + a * nnlc;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  double p[24];
#pragma unroll
  for (int i = 0; i < 24; ++i) p[i] = 0.0;
  for (long j = tid; j < n; j += kT) {
    const sep_nlc& e = base[j];
    const C2 s[2] = {ld(psi + 2 * e.jxyz), ld(psi + 2 * (ngrid + e.jxyz))};
    const C2 y[3] = {ld(e.y10), ld(e.y11), ld(e.y1_1)};
    const double g[2] = {e.Vs0G1, e.Vs0G_2};
#pragma unroll
    for (int gi = 0; gi < 2; ++gi)
#pragma unroll
      for (int m = 0; m < 3; ++m)
#pragma unroll
        for (int si = 0; si < 2; ++si) {
          const C2 v = conj_mul(y[m], s[si]);
          const int i = ((gi * 3 + m) * 2 + si) * 2;
          p[i] += g[gi] * v.re;
          p[i + 1] += g[gi] * v.im;
        }
  }
#pragma unroll
  for (int i = 0; i < 24; ++i) {
    double x = p[i];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][i] = x;
  }
  __syncthreads();
  if (tid < 24) {
    double x = 0.0;
    for (int w = 0; w < kT / 32; ++w) x += red[w][tid];
    const double el = (tid < 12 ? elkb[a] : elkb[a + natom]) * dv;  // hamiltonian.c:284-285
    proj[tid] = x * el;
  }
  __syncthreads();
  auto P = [&](int gi, int m, int si) {
    const int i = ((gi * 3 + m) * 2 + si) * 2;
    return C2{proj[i], proj[i + 1]};
  };
  const double s6 = sqrt(2.0) / 6.0, s3 = sqrt(2.0) / 3.0;
  const double o6 = 1.0 / 6.0, o3 = 1.0 / 3.0, t3 = 2.0 / 3.0;
  for (long j = tid; j < n; j += kT) {
    const sep_nlc& e = base[j];
    const C2 y10 = ld(e.y10), y11 = ld(e.y11), y1_1 = ld(e.y1_1);
    const double g1 = e.Vs0G1, g2 = e.Vs0G_2;
    // hamiltonian.c:318-353, in its order: G_2 terms, then G1 terms
    C2 up = scale(o6 * g2, mul(P(1, 2, 0), y1_1));
    up = add(up, scale(o3 * g2, mul(P(1, 0, 0), y10)));
    up = add(up, scale(0.5 * g2, mul(P(1, 1, 0), y11)));
    up = add(up, scale(s6 * g2, mul(P(1, 0, 1), y1_1)));
    up = add(up, scale(s6 * g2, mul(P(1, 1, 1), y10)));
    up = add(up, scale(-t3 * g1, mul(P(0, 2, 0), y1_1)));
    up = add(up, scale(-o3 * g1, mul(P(0, 0, 0), y10)));
    up = add(up, scale(s3 * g1, mul(P(0, 0, 1), y1_1)));
    up = add(up, scale(s3 * g1, mul(P(0, 1, 1), y10)));
    // hamiltonian.c:358-395
    C2 dn = scale(o6 * g2, mul(P(1, 1, 1), y11));
    dn = add(dn, scale(o3 * g2, mul(P(1, 0, 1), y10)));
    dn = add(dn, scale(-0.5 * g2, mul(P(1, 2, 1), y1_1)));
    dn = add(dn, scale(s6 * g2, mul(P(1, 2, 0), y10)));
    dn = add(dn, scale(s6 * g2, mul(P(1, 0, 0), y11)));
    dn = add(dn, scale(s3 * g1, mul(P(0, 2, 0), y10)));
    dn = add(dn, scale(s3 * g1, mul(P(0, 0, 0), y10)));
    dn = add(dn, scale(-o3 * g1, mul(P(0, 0, 1), y10)));
    dn = add(dn, scale(-t3 * g1, mul(P(0, 1, 1), y11)));
    atomic_add(out + 2 * e.jxyz, up);
    atomic_add(out + 2 * (ngrid + e.jxyz), dn);
  }
}

}  // namespace

namespace sep {
// Vso on nsp spinors (4 ngrid doubles apart) into psinl (zeroed first), on st;
// the arguments are already checked.  nsp <= 65535.
cudaError_t spinor_vso_launch(const double* psi, long ngrid, long nsp, long natom, long nnlc,
                              const sep_nlc* nlc, const long* nl, double sigma, double dv,
                              int flagkb, const double* elkb, double* psinl, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(psinl, 0, sizeof(double) * 4 * (size_t)ngrid * nsp, st);
  if (e != cudaSuccess || natom == 0) return e;
  const dim3 grid((unsigned)natom, (unsigned)nsp);
  if (flagkb) {
    k_vso_kb<<<grid, kT, 0, st>>>(psi, ngrid, nnlc, nlc, nl, elkb, natom, dv, psinl);
  } else {
    const double tmp = 0.5 / sqrt(kTwoPi * (sigma * sigma)) * dv;  // hamiltonian.c:89
    const double sigma_1 = sqrt(0.5) / sigma;                       // init.c:97
    k_vso_gauss<<<grid, kT, 0, st>>>(psi, ngrid, nnlc, nlc, nl, tmp, sigma_1, psinl);
  }
  return cudaGetLastError();
}
}  // namespace sep

extern "C" {

int sep_spinor_vso_dev(const double* psi, long ngrid, long natom, long nnlc, const sep_nlc* nlc,
                       const long* nl, double sigma, double dv, int flagkb, const double* elkb,
                       double* psinl, void* cuda_stream) {
  if (!psi || !psinl || !nlc || !nl || ngrid < 1 || natom < 0 || nnlc < 0 ||
      (flagkb && !elkb) || (!flagkb && !(sigma > 0.0)))
    return fail(SEP_ERR_ARG, "sep_spinor_vso: bad arguments");
  cudaStream_t st = (cudaStream_t)cuda_stream;
  SK(sep::spinor_vso_launch(psi, ngrid, 1, natom, nnlc, nlc, nl, sigma, dv, flagkb, elkb, psinl,
                            st));
  return SEP_OK;
}

int sep_spinor_vso(const double* psi, long ngrid, long natom, long nnlc, const sep_nlc* nlc,
                   const long* nl, double sigma, double dv, int flagkb, const double* elkb,
                   double* psinl) {
  if (!psi || !psinl || !nlc || !nl || ngrid < 1 || natom < 0 || nnlc < 0 || (flagkb && !elkb))
    return fail(SEP_ERR_ARG, "sep_spinor_vso: bad arguments");
  for (long a = 0; a < natom; ++a)
    if (nl[a] < 0 || nl[a] > nnlc) return fail(SEP_ERR_ARG, "sep_spinor_vso: nl[a] > nnlc");
  for (long a = 0; a < natom; ++a)
    for (long j = 0; j < nl[a]; ++j) {
      const long g = nlc[a * nnlc + j].jxyz;
      if (g < 0 || g >= ngrid) return fail(SEP_ERR_ARG, "sep_spinor_vso: jxyz outside the grid");
    }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return fail(SEP_ERR_NO_DEVICE, "sep_spinor_vso: no CUDA device");
  }
  double *d_psi = nullptr, *d_out = nullptr, *d_el = nullptr;
  sep_nlc* d_nlc = nullptr;
  long* d_nl = nullptr;
  cudaStream_t st = nullptr;
  int r = SEP_OK;
  auto done = [&](int status) {
    if (st) cudaStreamSynchronize(st);
    cudaFree(d_psi);
    cudaFree(d_out);
    cudaFree(d_el);
    cudaFree(d_nlc);
    cudaFree(d_nl);
    if (st) cudaStreamDestroy(st);
    return status;
  };
  const size_t nbytes = sizeof(double) * 4 * ngrid;
  const size_t lbytes = sizeof(sep_nlc) * (size_t)(natom * nnlc > 0 ? natom * nnlc : 1);
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&d_psi, nbytes) != cudaSuccess || cudaMalloc(&d_out, nbytes) != cudaSuccess ||
      cudaMalloc(&d_nlc, lbytes) != cudaSuccess ||
      cudaMalloc(&d_nl, sizeof(long) * (natom > 0 ? natom : 1)) != cudaSuccess ||
      cudaMalloc(&d_el, sizeof(double) * (natom > 0 ? 2 * natom : 1)) != cudaSuccess)
    return done(fail(SEP_ERR_NOMEM, "sep_spinor_vso: device allocation failed"));
  if (cudaMemcpyAsync(d_psi, psi, nbytes, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      (natom > 0 && cudaMemcpyAsync(d_nlc, nlc, sizeof(sep_nlc) * natom * nnlc,
                                    cudaMemcpyHostToDevice, st) != cudaSuccess) ||
      (natom > 0 && cudaMemcpyAsync(d_nl, nl, sizeof(long) * natom, cudaMemcpyHostToDevice,
                                    st) != cudaSuccess) ||
      (flagkb && natom > 0 && cudaMemcpyAsync(d_el, elkb, sizeof(double) * 2 * natom,
                                              cudaMemcpyHostToDevice, st) != cudaSuccess))
    return done(fail(SEP_ERR_CUDA, "sep_spinor_vso: upload failed"));
  r = sep_spinor_vso_dev(d_psi, ngrid, natom, nnlc, d_nlc, d_nl, sigma, dv, flagkb, d_el, d_out,
                         st);
  if (r != SEP_OK) return done(r);
  if (cudaMemcpyAsync(psinl, d_out, nbytes, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return done(fail(SEP_ERR_CUDA, "sep_spinor_vso: download failed"));
  return done(SEP_OK);
}

}  // extern "C"
