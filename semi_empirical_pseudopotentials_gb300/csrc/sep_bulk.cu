// sep_bulk.cu -- bulk band structures of the empirical-pseudopotential fit
// (the reference's pseudopotFitting/ program) and their gradients with
// respect to the form-factor parameters.
//
// Per crystal (one sep_bulk): plane-wave basis G_j (|G|^2/2 < maxKE,
// states.c:10-61), atoms tau_a with a type each, and nk k-points.  One call
// of sep_bulk_bands
//   1. builds V_jl = sum_a v_t(a)(|G_j - G_l|) exp(-i (G_j - G_l).tau_a) / natom
//      (hamiltonian.c:55-83, v(q) = a0 (q^2 - a1) / (a2 exp(a3 q^2) + 1),
//      hamiltonian.c:91-94) on the GPU, once for all k-points;
//   2. assembles H_k = V + diag(s |k + G_j|^2 / 2) for every k-point at once
//      (hamiltonian.c:11-52), column-major nbv x nbv complex;
//   3. finds the lowest nev (+ 16, for degenerate clusters that reach past
//      band nev) eigenpairs of all nk matrices at once with the library's
//      batched Hermitian solver (sep_heevb.cu: one CTA per matrix), in place
//      of one zheev per k-point (diag.c:12-48); cuSOLVER's batched routine
//      (cusolverDnXsyevBatched, or Zheevd per matrix where it declines the
//      size) stays selectable;
//   4. keeps the lowest nev eigenvalues of each in eV (fit.c:86-88).
// The reference's fit searches the parameters by Monte Carlo (fit.c:9-69);
// sep_bulk_bands_backward gives the gradient instead:
//   dL/dtheta = sum_{k,n} dL/dE_kn <u_kn| dV/dtheta |u_kn>   (Hellmann-Feynman)
//             = Re sum_jl W_jl dV_jl/dtheta,  W_jl = sum_{k,n} g_kn conj(U_k(j,n)) U_k(l,n),
// with dV/dtheta from the analytic derivatives of v(q).
#include <cuda_runtime.h>
#include <cuComplex.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/sep_gb300.h"
#include "sep_heevb.cuh"

namespace sep {
void set_error(const std::string& msg);
}

struct sep_bulk {
  int device = 0;
  cudaStream_t stream = nullptr;
  cusolverDnHandle_t solver = nullptr;
  cusolverDnParams_t sparams = nullptr;
  long nbv = 0, natom = 0, nk = 0, nev = 0, ntype = 0;
  double ke_scale = 1.0;
  double* g = nullptr;        // nbv x 3
  double* tau = nullptr;      // natom x 3
  int* types = nullptr;       // natom
  double* kpts = nullptr;     // nk x 3
  double* params = nullptr;   // ntype x 4
  cuDoubleComplex* v = nullptr;   // nbv x nbv
  cuDoubleComplex* h = nullptr;   // nk x nbv x nbv
  cuDoubleComplex* wmat = nullptr;  // nbv x nbv
  double* w = nullptr;        // nk x nbv eigenvalues
  double* bands = nullptr;    // nk x nev
  double* dlde = nullptr;     // nk x nev_cap (dL/dE per band, clusters widened past nev)
  long nev_cap = 0;
  // degenerate clusters with unequal dL/dE (sep_bulk_bands_backward)
  int* clu = nullptr;                 // per cluster: k, first band, size
  cuDoubleComplex* cluy = nullptr;    // per cluster and parameter: dV/dtheta U_c (nbv x c)
  cuDoubleComplex* clum = nullptr;    // per cluster and parameter: U_c^H dV/dtheta U_c (c x c)
  long clu_cap = 0;
  double* partials = nullptr; // grad blocks x 4 ntype
  double* grad = nullptr;     // 4 ntype
  int* info = nullptr;        // nk
  void* dwork = nullptr;
  size_t dwork_bytes = 0;
  std::vector<char> hwork;
  int batched = -1;           // -1 untried, 1 batched routine, 0 per-matrix
  int native = 1;             // 1: the library's batched solver (sep_heevb.cu), 0: cuSOLVER
  int path = -1;              // last solve: 2 library, 1 cuSOLVER batched, 0 per matrix
  void* hbwork = nullptr;
  size_t hbwork_bytes = 0;
  // the last solve: its parameters, and whether b->h holds its eigenvectors
  // (a backward call with the same parameters reuses them)
  std::vector<double> last_params;
  bool last_vectors = false;
};

namespace {

constexpr double kAutoEv = 27.2114;                // fit.h AUTOEV
constexpr double kTwoPi = 6.28318530717958647692;  // fit.h TWOPI
constexpr int kThreads = 256;
constexpr int kMaxTypes = 8;
constexpr int kRetry = 1;  // eig_all: run the assembly and the eigensolver again

int fail(int status, const std::string& msg) {
  sep::set_error(msg);
  return status;
}

#define BK(...)                                                                      \
  do {                                                                               \
    cudaError_t _e = (__VA_ARGS__);                                                  \
    if (_e != cudaSuccess) {                                                         \
      char _b[320];                                                                  \
      snprintf(_b, sizeof _b, "CUDA error %d (%s) at sep_bulk.cu:%d", (int)_e,       \
               cudaGetErrorString(_e), __LINE__);                                    \
      return fail(_e == cudaErrorMemoryAllocation ? SEP_ERR_NOMEM : SEP_ERR_CUDA, _b); \
    }                                                                                \
  } while (0)
#define BS(...)                                                                      \
  do {                                                                               \
    cusolverStatus_t _s = (__VA_ARGS__);                                             \
    if (_s != CUSOLVER_STATUS_SUCCESS) {                                             \
      char _b[256];                                                                  \
      snprintf(_b, sizeof _b, "cusolver status %d at sep_bulk.cu:%d", (int)_s,       \
               __LINE__);                                                            \
      return fail(SEP_ERR_SOLVER, _b);                                               \
    }                                                                                \
  } while (0)

struct V3 {
  double x, y, z;
};
// retCrossProduct / retDotProduct of vector.c
V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

__device__ __forceinline__ double dot_rn(double ax, double ay, double az, double bx, double by,
                                         double bz) {
  return __dadd_rn(__dadd_rn(__dmul_rn(ax, bx), __dmul_rn(ay, by)), __dmul_rn(az, bz));
}

// V_jl, column-major (v[j + l nbv]); the atoms are summed in input order
__global__ void k_bulk_potential(const double* __restrict__ g, const double* __restrict__ tau,
                                 const int* __restrict__ types, const double* __restrict__ prm,
                                 int natom, long nbv, cuDoubleComplex* __restrict__ v) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nbv * nbv) return;
  const long j = t % nbv, l = t / nbv;
  const double dx = g[3 * j] - g[3 * l], dy = g[3 * j + 1] - g[3 * l + 1],
               dz = g[3 * j + 2] - g[3 * l + 2];
  const double q = sqrt(dot_rn(dx, dy, dz, dx, dy, dz));
  const double q2 = __dmul_rn(q, q);
  const double inv = 1.0 / (double)natom;
  double re = 0.0, im = 0.0;
  for (int a = 0; a < natom; ++a) {
    const double* p = prm + 4 * types[a];
    const double ph = dot_rn(dx, dy, dz, tau[3 * a], tau[3 * a + 1], tau[3 * a + 2]);
    double s, c;
    sincos(ph, &s, &c);
    const double ff = p[0] * (q2 - p[1]) / (p[2] * exp(p[3] * q2) + 1.0);
    re += ff * (inv * c);
    im += ff * (-inv * s);
  }
  v[t] = make_cuDoubleComplex(re, im);
}

// H_k = V + diag(s |k + G_j|^2 / 2) for every k-point
__global__ void k_bulk_assemble(const cuDoubleComplex* __restrict__ v,
                                const double* __restrict__ g, const double* __restrict__ kp,
                                double pre, long nbv, long nk, cuDoubleComplex* __restrict__ h) {
  const long n2 = nbv * nbv;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nk * n2;
       t += (long)gridDim.x * blockDim.x) {
    const long k = t / n2, e = t - k * n2;
    const long j = e % nbv, l = e / nbv;
    cuDoubleComplex x = v[e];
    if (j == l) {
      const double px = g[3 * j] + kp[3 * k], py = g[3 * j + 1] + kp[3 * k + 1],
                   pz = g[3 * j + 2] + kp[3 * k + 2];
      const double mag = sqrt(dot_rn(px, py, pz, px, py, pz));
      x.x += __dmul_rn(__dmul_rn(mag, mag), pre);
    }
    h[t] = x;
  }
}

__global__ void k_bulk_take(const double* __restrict__ w, long nbv, long nk, long nev,
                            double* __restrict__ bands) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nk * nev) return;
  const long k = t / nev, n = t - k * nev;
  bands[t] = w[k * nbv + n] * kAutoEv;
}

// W_jl = sum_{k,n} g_kn conj(U_k(j,n)) U_k(l,n); U_k(j,n) = h[k nbv^2 + j + n nbv]
__global__ void k_bulk_density(const cuDoubleComplex* __restrict__ h,
                               const double* __restrict__ gkn, long nbv, long nk, long nev,
                               cuDoubleComplex* __restrict__ wm) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nbv * nbv) return;
  const long j = t % nbv, l = t / nbv;
  double re = 0.0, im = 0.0;
  for (long k = 0; k < nk; ++k) {
    const cuDoubleComplex* u = h + k * nbv * nbv;
    for (long n = 0; n < nev; ++n) {
      const double wgt = gkn[k * nev + n];
      if (wgt == 0.0) continue;
      const cuDoubleComplex a = u[j + n * nbv], b = u[l + n * nbv];
      // conj(a) b
      re += wgt * (a.x * b.x + a.y * b.y);
      im += wgt * (a.x * b.y - a.y * b.x);
    }
  }
  wm[t] = make_cuDoubleComplex(re, im);
}

// per block: sum over its (j, l) of Re(W_jl dV_jl / da_{t,p}) for every type t and p
__global__ void k_bulk_grad(const double* __restrict__ g, const double* __restrict__ tau,
                            const int* __restrict__ types, const double* __restrict__ prm,
                            int natom, int ntype, long nbv,
                            const cuDoubleComplex* __restrict__ wm,
                            double* __restrict__ partials) {
  __shared__ double red[kThreads / 32];
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  double acc[4 * kMaxTypes];
#pragma unroll
  for (int i = 0; i < 4 * kMaxTypes; ++i) acc[i] = 0.0;
  if (t < nbv * nbv) {
    const long j = t % nbv, l = t / nbv;
    const double dx = g[3 * j] - g[3 * l], dy = g[3 * j + 1] - g[3 * l + 1],
                 dz = g[3 * j + 2] - g[3 * l + 2];
    const double q = sqrt(dot_rn(dx, dy, dz, dx, dy, dz));
    const double q2 = __dmul_rn(q, q);
    const double inv = 1.0 / (double)natom;
    const cuDoubleComplex wv = wm[t];
    for (int a = 0; a < natom; ++a) {
      const int ty = types[a];
      const double* p = prm + 4 * ty;
      const double ph = dot_rn(dx, dy, dz, tau[3 * a], tau[3 * a + 1], tau[3 * a + 2]);
      double s, c;
      sincos(ph, &s, &c);
      // Re(W (sr + i si)) with the structure factor (c, -s) / natom
      const double proj = wv.x * (inv * c) - wv.y * (-inv * s);
      const double e = exp(p[3] * q2);
      const double den = p[2] * e + 1.0;
      const double num = q2 - p[1];
      const double f_den2 = p[0] * num * e / (den * den);
      double d[4];
      d[0] = num / den;
      d[1] = -p[0] / den;
      d[2] = -f_den2;
      d[3] = -f_den2 * p[2] * q2;
#pragma unroll
      for (int i = 0; i < kMaxTypes; ++i)
        if (i == ty) {
#pragma unroll
          for (int m = 0; m < 4; ++m) acc[4 * i + m] += d[m] * proj;
        }
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int i = 0; i < 4 * ntype; ++i) {
    double x = acc[0];
#pragma unroll
    for (int r = 0; r < 4 * kMaxTypes; ++r)
      if (r == i) x = acc[r];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int k = 0; k < kThreads / 32; ++k) s += red[k];
      partials[(long)blockIdx.x * 4 * ntype + i] = s;
    }
    __syncthreads();
  }
}

constexpr int kMaxCluster = 16;  // bands in one degenerate cluster handled exactly

// dV_jl/da_{t,m} = sum_{a of type t} (cos - i sin)(G_jl . tau_a) / natom * dv_t/da_m(|G_jl|)
__device__ __forceinline__ void dv_dparam(const double* __restrict__ g,
                                          const double* __restrict__ tau,
                                          const int* __restrict__ types,
                                          const double* __restrict__ prm, int natom, long j,
                                          long l, int ty, int m, double* re, double* im) {
  const double dx = g[3 * j] - g[3 * l], dy = g[3 * j + 1] - g[3 * l + 1],
               dz = g[3 * j + 2] - g[3 * l + 2];
  const double q = sqrt(dot_rn(dx, dy, dz, dx, dy, dz));
  const double q2 = __dmul_rn(q, q);
  const double* p = prm + 4 * ty;
  const double e = exp(p[3] * q2);
  const double den = p[2] * e + 1.0;
  const double num = q2 - p[1];
  const double f_den2 = p[0] * num * e / (den * den);
  const double d = m == 0 ? num / den : m == 1 ? -p[0] / den : m == 2 ? -f_den2
                                                                        : -f_den2 * p[2] * q2;
  const double inv = 1.0 / (double)natom;
  double sr = 0.0, si = 0.0;
  for (int a = 0; a < natom; ++a) {
    if (types[a] != ty) continue;
    const double ph = dot_rn(dx, dy, dz, tau[3 * a], tau[3 * a + 1], tau[3 * a + 2]);
    double sn, cs;
    sincos(ph, &sn, &cs);
    sr += inv * cs;
    si -= inv * sn;
  }
  *re = d * sr;
  *im = d * si;
}

// Y = dV/da_{t,m} U_c for cluster c (grid: clusters x parameters; rows j over threads)
__global__ void k_bulk_cluster_y(const double* __restrict__ g, const double* __restrict__ tau,
                                 const int* __restrict__ types, const double* __restrict__ prm,
                                 int natom, int nparam, long nbv,
                                 const cuDoubleComplex* __restrict__ h,
                                 const int* __restrict__ clu, cuDoubleComplex* __restrict__ y) {
  const int item = blockIdx.x / nparam, par = blockIdx.x % nparam;
  const int k = clu[3 * item], n0 = clu[3 * item + 1], c = clu[3 * item + 2];
  const cuDoubleComplex* u = h + (long)k * nbv * nbv;
  cuDoubleComplex* out = y + ((long)item * nparam + par) * nbv * kMaxCluster;
  for (long j = threadIdx.x; j < nbv; j += blockDim.x) {
    double ar[kMaxCluster], ai[kMaxCluster];
#pragma unroll
    for (int i = 0; i < kMaxCluster; ++i) ar[i] = ai[i] = 0.0;
    for (long l = 0; l < nbv; ++l) {
      double dr, di;
      dv_dparam(g, tau, types, prm, natom, j, l, par / 4, par % 4, &dr, &di);
#pragma unroll
      for (int i = 0; i < kMaxCluster; ++i)
        if (i < c) {
          const cuDoubleComplex b = u[l + (long)(n0 + i) * nbv];
          ar[i] += dr * b.x - di * b.y;
          ai[i] += dr * b.y + di * b.x;
        }
    }
#pragma unroll
    for (int i = 0; i < kMaxCluster; ++i)
      if (i < c) out[j * kMaxCluster + i] = make_cuDoubleComplex(ar[i], ai[i]);
  }
}

// M = U_c^H Y (c x c per cluster and parameter; one thread per entry)
__global__ void k_bulk_cluster_m(int nparam, long nbv, const cuDoubleComplex* __restrict__ h,
                                 const int* __restrict__ clu,
                                 const cuDoubleComplex* __restrict__ y,
                                 cuDoubleComplex* __restrict__ mm) {
  const int item = blockIdx.x / nparam, par = blockIdx.x % nparam;
  const int k = clu[3 * item], n0 = clu[3 * item + 1], c = clu[3 * item + 2];
  const int i = threadIdx.x / kMaxCluster, i2 = threadIdx.x % kMaxCluster;
  if (i >= c || i2 >= c) return;
  const cuDoubleComplex* u = h + (long)k * nbv * nbv + (long)(n0 + i) * nbv;
  const cuDoubleComplex* yy = y + ((long)item * nparam + par) * nbv * kMaxCluster;
  double re = 0.0, im = 0.0;
  for (long j = 0; j < nbv; ++j) {
    const cuDoubleComplex a = u[j], b = yy[j * kMaxCluster + i2];
    re += a.x * b.x + a.y * b.y;  // conj(a) b
    im += a.x * b.y - a.y * b.x;
  }
  mm[((long)item * nparam + par) * kMaxCluster * kMaxCluster + i * kMaxCluster + i2] =
      make_cuDoubleComplex(re, im);
}

// eigenvalues (ascending) of a c x c Hermitian matrix: cyclic Jacobi on its
// real symmetric embedding [[Re, -Im], [Im, Re]], whose eigenvalues are those
// of M, each twice
void hermitian_eigvals(int c, const cuDoubleComplex* m, int ld, double* out) {
  const int n = 2 * c;
  std::vector<double> a((size_t)n * n);
  for (int i = 0; i < c; ++i)
    for (int j = 0; j < c; ++j) {
      const double re = 0.5 * (m[i * ld + j].x + m[j * ld + i].x);
      const double im = 0.5 * (m[i * ld + j].y - m[j * ld + i].y);
      a[(size_t)i * n + j] = re;
      a[(size_t)(i + c) * n + (j + c)] = re;
      a[(size_t)i * n + (j + c)] = -im;
      a[(size_t)(i + c) * n + j] = im;
    }
  for (int sweep = 0; sweep < 64; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        tot += a[(size_t)i * n + j] * a[(size_t)i * n + j];
        if (i != j) off += a[(size_t)i * n + j] * a[(size_t)i * n + j];
      }
    if (off <= 1e-30 * tot || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = a[(size_t)p * n + q];
        if (apq == 0.0) continue;
        const double app = a[(size_t)p * n + p], aqq = a[(size_t)q * n + q];
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) /
                         (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double cs = 1.0 / std::sqrt(t * t + 1.0), sn = t * cs;
        for (int r = 0; r < n; ++r) {  // columns p, q
          const double x = a[(size_t)r * n + p], yv = a[(size_t)r * n + q];
          a[(size_t)r * n + p] = cs * x - sn * yv;
          a[(size_t)r * n + q] = sn * x + cs * yv;
        }
        for (int r = 0; r < n; ++r) {  // rows p, q
          const double x = a[(size_t)p * n + r], yv = a[(size_t)q * n + r];
          a[(size_t)p * n + r] = cs * x - sn * yv;
          a[(size_t)q * n + r] = sn * x + cs * yv;
        }
      }
  }
  std::vector<double> ev(n);
  for (int i = 0; i < n; ++i) ev[i] = a[(size_t)i * n + i];
  std::sort(ev.begin(), ev.end());
  for (int i = 0; i < c; ++i) out[i] = 0.5 * (ev[2 * i] + ev[2 * i + 1]);
}

__global__ void k_bulk_grad_sum(const double* __restrict__ partials, long nblocks, int nval,
                                double* __restrict__ grad) {
  const int i = threadIdx.x;
  if (i >= nval) return;
  double s = 0.0;
  for (long b = 0; b < nblocks; ++b) s += partials[b * nval + i];
  grad[i] = s;
}

unsigned blocks_for(long n) { return (unsigned)((n + kThreads - 1) / kThreads); }

// eigenvalues (and eigenvectors when vectors != 0) of the nk matrices in b->h
int eig_all(sep_bulk* b, bool vectors) {
  // the library's solver: the lowest nev + kMaxCluster eigenpairs (NaN after
  // them in b->w), enough for the bands and for any cluster of up to
  // kMaxCluster bands that starts below band nev
  const int nwant = (int)std::min<long>(b->nbv, b->nev + kMaxCluster);
  if (b->native && sep::hb::supported((int)b->nbv, nwant)) {
    const size_t need = sep::hb::work_bytes((int)b->nbv, (int)b->nk, nwant);
    if (need > b->hbwork_bytes) {
      if (b->hbwork) cudaFree(b->hbwork);
      b->hbwork = nullptr;
      b->hbwork_bytes = 0;
      BK(cudaMalloc(&b->hbwork, need));
      b->hbwork_bytes = need;
    }
    BK(sep::hb::lowest(reinterpret_cast<double2*>(b->h), (int)b->nbv, (int)b->nk, nwant, vectors,
                       b->w, b->hbwork, b->stream));
    b->path = 2;
    if (vectors) {
      int bad = 0;
      BK(sep::hb::failed_vectors(b->hbwork, (int)b->nbv, (int)b->nk, nwant, &bad, b->stream));
      if (bad)
        return fail(SEP_ERR_SOLVER, "sep_bulk: inverse iteration did not converge for " +
                                        std::to_string(bad) + " eigenvector(s)");
    }
    return SEP_OK;
  }
  const cusolverEigMode_t jobz = vectors ? CUSOLVER_EIG_MODE_VECTOR : CUSOLVER_EIG_MODE_NOVECTOR;
  const cublasFillMode_t uplo = CUBLAS_FILL_MODE_LOWER;
  const int64_t n = b->nbv;
  if (b->batched != 0) {
    size_t dbytes = 0, hbytes = 0;
    const cusolverStatus_t s = cusolverDnXsyevBatched_bufferSize(
        b->solver, b->sparams, jobz, uplo, n, CUDA_C_64F, b->h, n, CUDA_R_64F, b->w, CUDA_C_64F,
        &dbytes, &hbytes, (int64_t)b->nk);
    if (s == CUSOLVER_STATUS_SUCCESS) {
      if (dbytes > b->dwork_bytes) {
        if (b->dwork) cudaFree(b->dwork);
        b->dwork = nullptr;
        b->dwork_bytes = 0;
        BK(cudaMalloc(&b->dwork, dbytes));
        b->dwork_bytes = dbytes;
      }
      if (b->hwork.size() < hbytes) b->hwork.resize(hbytes);
      const cusolverStatus_t r = cusolverDnXsyevBatched(
          b->solver, b->sparams, jobz, uplo, n, CUDA_C_64F, b->h, n, CUDA_R_64F, b->w,
          CUDA_C_64F, b->dwork, b->dwork_bytes, hbytes ? b->hwork.data() : nullptr, hbytes,
          b->info, (int64_t)b->nk);
      if (r == CUSOLVER_STATUS_SUCCESS) {
        b->batched = 1;
        b->path = 1;
        return SEP_OK;
      }
      if (b->batched == 1) BS(r);
      b->batched = 0;  // declined at run time: the matrices are assembled again
      return kRetry;
    } else if (b->batched == 1) {
      BS(s);
    }
    b->batched = 0;  // the batched routine declined this size: one matrix per call
  }
  int lwork = 0;
  BS(cusolverDnZheevd_bufferSize(b->solver, jobz, uplo, (int)n, b->h, (int)n, b->w, &lwork));
  const size_t want = (size_t)lwork * sizeof(cuDoubleComplex);
  if (want > b->dwork_bytes) {
    if (b->dwork) cudaFree(b->dwork);
    b->dwork = nullptr;
    b->dwork_bytes = 0;
    BK(cudaMalloc(&b->dwork, want));
    b->dwork_bytes = want;
  }
  for (long k = 0; k < b->nk; ++k)
    BS(cusolverDnZheevd(b->solver, jobz, uplo, (int)n, b->h + k * n * n, (int)n, b->w + k * n,
                        (cuDoubleComplex*)b->dwork, lwork, b->info + k));
  b->path = 0;
  return SEP_OK;
}

int check_info(sep_bulk* b) {
  std::vector<int> info(b->nk);
  BK(cudaMemcpyAsync(info.data(), b->info, sizeof(int) * b->nk, cudaMemcpyDeviceToHost,
                     b->stream));
  BK(cudaStreamSynchronize(b->stream));
  for (long k = 0; k < b->nk; ++k)
    if (info[k] != 0) {
      char m[160];
      snprintf(m, sizeof m, "eigensolver info %d at k-point %ld (reference: zheev info, "
               "diag.c:37-41)", info[k], k);
      return fail(SEP_ERR_SOLVER, m);
    }
  return SEP_OK;
}

// potential, assembly and the eigensolver for params (ntype x 4, host)
int solve(sep_bulk* b, const double* params, bool vectors) {
  BK(cudaSetDevice(b->device));
  const size_t np = (size_t)(4 * b->ntype);
  if (b->last_params.size() == np && (b->last_vectors || !vectors) &&
      std::equal(params, params + np, b->last_params.begin()))
    return SEP_OK;  // b->w (and b->h) already hold this solve
  b->last_params.clear();
  BK(cudaMemcpyAsync(b->params, params, sizeof(double) * 4 * b->ntype, cudaMemcpyHostToDevice,
                     b->stream));
  const long n2 = b->nbv * b->nbv;
  k_bulk_potential<<<blocks_for(n2), kThreads, 0, b->stream>>>(b->g, b->tau, b->types, b->params,
                                                                (int)b->natom, b->nbv, b->v);
  BK(cudaGetLastError());
  const long tot = n2 * b->nk;
  const unsigned grid = (unsigned)std::min<long>(blocks_for(tot), 152L * 16);
  int r = kRetry;
  for (int attempt = 0; attempt < 2 && r == kRetry; ++attempt) {
    k_bulk_assemble<<<grid, kThreads, 0, b->stream>>>(b->v, b->g, b->kpts, 0.5 * b->ke_scale,
                                                       b->nbv, b->nk, b->h);
    BK(cudaGetLastError());
    r = eig_all(b, vectors);
  }
  if (r != SEP_OK) return r == kRetry ? fail(SEP_ERR_SOLVER, "sep_bulk: eigensolver retry") : r;
  if (b->path != 2 && (r = check_info(b)) != SEP_OK) return r;
  b->last_params.assign(params, params + np);
  b->last_vectors = vectors;
  return SEP_OK;
}

template <typename T> int dalloc(T** p, size_t count) {
  BK(cudaMalloc((void**)p, sizeof(T) * std::max<size_t>(count, 1)));
  return SEP_OK;
}

}  // namespace

extern "C" {

int sep_bulk_basis(const double cell[9], double max_ke, long cap, long* nbv, double* g) {
  if (!cell || !nbv || !(max_ke > 0.0)) return fail(SEP_ERR_ARG, "sep_bulk_basis: bad arguments");
  const V3 a0{cell[0], cell[1], cell[2]}, a1{cell[3], cell[4], cell[5]}, a2{cell[6], cell[7], cell[8]};
  // init.c:21-45
  const double vol = dot(a0, cross(a1, a2));
  if (!(std::fabs(vol) > 0.0)) return fail(SEP_ERR_ARG, "sep_bulk_basis: singular cell");
  const double pre = kTwoPi / vol;
  V3 b[3] = {cross(a1, a2), cross(a2, a0), cross(a0, a1)};
  for (V3& v : b) v = {v.x * pre, v.y * pre, v.z * pre};
  // states.c:10-61
  double gmin = 100000.0;
  for (const V3& v : b) gmin = std::min(gmin, std::sqrt(dot(v, v)));
  const int n = (int)(std::sqrt(max_ke / (gmin * gmin))) + 1;
  struct Gv {
    double x, y, z, mag;
  };
  std::vector<Gv> keep;
  for (int i = -n; i < n + 1; ++i)
    for (int j = -n; j < n + 1; ++j)
      for (int k = -n; k < n + 1; ++k) {
        Gv v;
        v.x = i * b[0].x + j * b[1].x + k * b[2].x;
        v.y = i * b[0].y + j * b[1].y + k * b[2].y;
        v.z = i * b[0].z + j * b[1].z + k * b[2].z;
        v.mag = std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
        if (1.0 * 0.5 * (v.mag * v.mag) / 1.0 < max_ke) keep.push_back(v);
      }
  // ordered by |G| (the reference's quicksort, states.c:78-110, leaves the
  // order inside a shell to its pivoting; the spectrum does not depend on it)
  std::stable_sort(keep.begin(), keep.end(), [](const Gv& p, const Gv& q) { return p.mag < q.mag; });
  *nbv = (long)keep.size();
  if (g) {
    if (cap < (long)keep.size()) return fail(SEP_ERR_ARG, "sep_bulk_basis: g holds fewer than nbv vectors");
    for (size_t i = 0; i < keep.size(); ++i) {
      g[3 * i] = keep[i].x;
      g[3 * i + 1] = keep[i].y;
      g[3 * i + 2] = keep[i].z;
    }
  }
  return SEP_OK;
}

int sep_bulk_create(long nbv, const double* g, long natom, const double* tau, const int* types,
                    long ntype, long nk, const double* kpts, double ke_scale, long nev,
                    sep_bulk** out) {
  if (!out || !g || !tau || !types || !kpts || nbv < 1 || natom < 1 || nk < 1 || nev < 1 ||
      nev > nbv || ntype < 1 || ntype > kMaxTypes)
    return fail(SEP_ERR_ARG, "sep_bulk_create: bad arguments (1 <= nev <= nbv, 1 <= ntype <= 8)");
  for (long a = 0; a < natom; ++a)
    if (types[a] < 0 || types[a] >= ntype) return fail(SEP_ERR_ARG, "sep_bulk_create: type out of range");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return fail(SEP_ERR_NO_DEVICE, "sep_bulk_create: no CUDA device");
  }
  sep_bulk* b = new sep_bulk();
  b->nbv = nbv;
  b->natom = natom;
  b->nk = nk;
  b->nev = nev;
  b->nev_cap = nev;
  b->ntype = ntype;
  b->ke_scale = ke_scale;
  auto bail = [&](int r) {
    sep_bulk_destroy(b);
    return r;
  };
  if (cudaGetDevice(&b->device) != cudaSuccess) return bail(fail(SEP_ERR_CUDA, "cudaGetDevice"));
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(fail(SEP_ERR_CUDA, "sep_bulk_create: stream"));
  if (cusolverDnCreate(&b->solver) != CUSOLVER_STATUS_SUCCESS ||
      cusolverDnSetStream(b->solver, b->stream) != CUSOLVER_STATUS_SUCCESS ||
      cusolverDnCreateParams(&b->sparams) != CUSOLVER_STATUS_SUCCESS)
    return bail(fail(SEP_ERR_SOLVER, "sep_bulk_create: cusolver set-up failed"));
  const size_t n2 = (size_t)nbv * nbv;
  int r = SEP_OK;
  if ((r = dalloc(&b->g, 3 * nbv)) || (r = dalloc(&b->tau, 3 * natom)) ||
      (r = dalloc(&b->types, natom)) || (r = dalloc(&b->kpts, 3 * nk)) ||
      (r = dalloc(&b->params, 4 * ntype)) || (r = dalloc(&b->v, n2)) ||
      (r = dalloc(&b->h, n2 * nk)) || (r = dalloc(&b->wmat, n2)) ||
      (r = dalloc(&b->w, (size_t)nbv * nk)) || (r = dalloc(&b->bands, (size_t)nk * nev)) ||
      (r = dalloc(&b->dlde, (size_t)nk * nev)) ||
      (r = dalloc(&b->partials, (size_t)blocks_for((long)n2) * 4 * ntype)) ||
      (r = dalloc(&b->grad, 4 * ntype)) || (r = dalloc(&b->info, nk)))
    return bail(r);
  if (cudaMemcpy(b->g, g, sizeof(double) * 3 * nbv, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->tau, tau, sizeof(double) * 3 * natom, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->types, types, sizeof(int) * natom, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(b->kpts, kpts, sizeof(double) * 3 * nk, cudaMemcpyHostToDevice) != cudaSuccess)
    return bail(fail(SEP_ERR_CUDA, "sep_bulk_create: upload"));
  *out = b;
  return SEP_OK;
}

static int bands_impl(sep_bulk* b, const double* params, double* bands, bool vectors) {
  if (!b || !params || !bands) return fail(SEP_ERR_ARG, "sep_bulk_bands: bad arguments");
  int r = solve(b, params, vectors);
  if (r != SEP_OK) return r;
  k_bulk_take<<<blocks_for(b->nk * b->nev), kThreads, 0, b->stream>>>(b->w, b->nbv, b->nk, b->nev,
                                                                       b->bands);
  BK(cudaGetLastError());
  BK(cudaMemcpyAsync(bands, b->bands, sizeof(double) * b->nk * b->nev, cudaMemcpyDeviceToHost,
                     b->stream));
  BK(cudaStreamSynchronize(b->stream));
  return SEP_OK;
}

int sep_bulk_bands(sep_bulk* b, const double* params, double* bands) {
  return bands_impl(b, params, bands, false);
}

int sep_bulk_bands_keep(sep_bulk* b, const double* params, double* bands) {
  return bands_impl(b, params, bands, true);
}

int sep_bulk_bands_backward(sep_bulk* b, const double* params, const double* dl_de, double* bands,
                            double* dl_dparams) {
  if (!b || !params || !dl_de || !dl_dparams)
    return fail(SEP_ERR_ARG, "sep_bulk_bands_backward: bad arguments");
  int r = solve(b, params, true);
  if (r != SEP_OK) return r;
  if (bands) {
    k_bulk_take<<<blocks_for(b->nk * b->nev), kThreads, 0, b->stream>>>(b->w, b->nbv, b->nk,
                                                                         b->nev, b->bands);
    BK(cudaGetLastError());
    BK(cudaMemcpyAsync(bands, b->bands, sizeof(double) * b->nk * b->nev, cudaMemcpyDeviceToHost,
                       b->stream));
  }
  // Degenerate clusters.  Inside a cluster of equal eigenvalues the
  // eigenvectors are any basis of its subspace, so sum_n g_n <u_n|dV|u_n>
  // depends on that basis unless the g_n are equal, and the sorted bands are
  // not differentiable there.  Each cluster's g is split into its mean, which
  // enters the density (a trace: basis-free), and the rest, whose part of
  // the derivative is taken from the cluster's first-order splitting: with
  // mu the eigenvalues of M = U_c^H dV/dtheta U_c ascending, band n0 + i
  // moves by +h mu_i for theta + h and by -h mu_{c-1-i} for theta - h, so
  // the limit of central differences is sum_i g_i (mu_i + mu_{c-1-i}) / 2.
  // A cluster that reaches past band nev takes its higher bands with g = 0.
  const long nbv = b->nbv, nk = b->nk, nev = b->nev;
  std::vector<double> wh((size_t)nk * nbv);
  BK(cudaMemcpyAsync(wh.data(), b->w, sizeof(double) * wh.size(), cudaMemcpyDeviceToHost,
                     b->stream));
  BK(cudaStreamSynchronize(b->stream));
  struct Cluster {
    int k, n0, c;
    std::vector<double> dg;  // g minus the cluster mean
  };
  std::vector<Cluster> split;
  long ncols = nev;  // bands that carry a g (nev, or more where a cluster reaches past it)
  std::vector<std::vector<double>> gk((size_t)nk);
  for (long k = 0; k < nk; ++k) {
    const double* lam = wh.data() + k * nbv;
    std::vector<double>& gg = gk[(size_t)k];
    gg.assign((size_t)nbv, 0.0);
    // bands are eV = AUTOEV x eigenvalue: dL/dlambda = AUTOEV dL/dE
    for (long n = 0; n < nev; ++n) gg[(size_t)n] = dl_de[k * nev + n] * kAutoEv;
    long n = 0;
    while (n < nev) {
      long e = n + 1;
      while (e < nbv && std::fabs(lam[e] - lam[e - 1]) <=
                            1e-10 * std::max(1.0, std::fabs(lam[e])))
        ++e;
      const long c = e - n;
      if (c > 1) {
        double mean = 0.0;
        for (long i = n; i < e; ++i) mean += gg[(size_t)i];
        mean /= (double)c;
        bool equal = true;
        for (long i = n; i < e; ++i) equal = equal && gg[(size_t)i] == mean;
        // a cluster of more than kMaxCluster bands keeps only its mean g (a
        // basis-free choice, without the splitting term)
        if (!equal && c <= kMaxCluster) {
          Cluster cl{(int)k, (int)n, (int)c, std::vector<double>((size_t)c)};
          for (long i = 0; i < c; ++i) cl.dg[(size_t)i] = gg[(size_t)(n + i)] - mean;
          split.push_back(std::move(cl));
        }
        if (!equal)
          for (long i = n; i < e; ++i) gg[(size_t)i] = mean;
        ncols = std::max(ncols, e);
      }
      n = e;
    }
  }
  if (ncols > b->nev_cap) {
    if (b->dlde) cudaFree(b->dlde);
    b->dlde = nullptr;
    b->nev_cap = 0;
    BK(cudaMalloc((void**)&b->dlde, sizeof(double) * (size_t)nk * ncols));
    b->nev_cap = ncols;
  }
  std::vector<double> g((size_t)nk * ncols);
  for (long k = 0; k < nk; ++k)
    for (long n = 0; n < ncols; ++n) g[(size_t)(k * ncols + n)] = gk[(size_t)k][(size_t)n];
  BK(cudaMemcpyAsync(b->dlde, g.data(), sizeof(double) * g.size(), cudaMemcpyHostToDevice,
                     b->stream));
  const long n2 = b->nbv * b->nbv;
  k_bulk_density<<<blocks_for(n2), kThreads, 0, b->stream>>>(b->h, b->dlde, b->nbv, b->nk, ncols,
                                                              b->wmat);
  BK(cudaGetLastError());
  const unsigned nblk = blocks_for(n2);
  k_bulk_grad<<<nblk, kThreads, 0, b->stream>>>(b->g, b->tau, b->types, b->params, (int)b->natom,
                                                 (int)b->ntype, b->nbv, b->wmat, b->partials);
  BK(cudaGetLastError());
  k_bulk_grad_sum<<<1, 32, 0, b->stream>>>(b->partials, nblk, (int)(4 * b->ntype), b->grad);
  BK(cudaGetLastError());
  const int nparam = (int)(4 * b->ntype);
  BK(cudaMemcpyAsync(dl_dparams, b->grad, sizeof(double) * nparam, cudaMemcpyDeviceToHost,
                     b->stream));
  BK(cudaStreamSynchronize(b->stream));
  if (!split.empty()) {
    const long ns = (long)split.size();
    if (ns > b->clu_cap) {
      for (void* q : {(void*)b->clu, (void*)b->cluy, (void*)b->clum})
        if (q) cudaFree(q);
      b->clu = nullptr;
      b->cluy = b->clum = nullptr;
      b->clu_cap = 0;
      BK(cudaMalloc((void**)&b->clu, sizeof(int) * 3 * ns));
      BK(cudaMalloc((void**)&b->cluy,
                    sizeof(cuDoubleComplex) * (size_t)ns * nparam * nbv * kMaxCluster));
      BK(cudaMalloc((void**)&b->clum, sizeof(cuDoubleComplex) * (size_t)ns * nparam *
                                          kMaxCluster * kMaxCluster));
      b->clu_cap = ns;
    }
    std::vector<int> desc((size_t)(3 * ns));
    for (long i = 0; i < ns; ++i) {
      desc[(size_t)(3 * i)] = split[(size_t)i].k;
      desc[(size_t)(3 * i + 1)] = split[(size_t)i].n0;
      desc[(size_t)(3 * i + 2)] = split[(size_t)i].c;
    }
    BK(cudaMemcpyAsync(b->clu, desc.data(), sizeof(int) * desc.size(), cudaMemcpyHostToDevice,
                       b->stream));
    k_bulk_cluster_y<<<(unsigned)(ns * nparam), 128, 0, b->stream>>>(
        b->g, b->tau, b->types, b->params, (int)b->natom, nparam, nbv, b->h, b->clu, b->cluy);
    BK(cudaGetLastError());
    k_bulk_cluster_m<<<(unsigned)(ns * nparam), kMaxCluster * kMaxCluster, 0, b->stream>>>(
        nparam, nbv, b->h, b->clu, b->cluy, b->clum);
    BK(cudaGetLastError());
    std::vector<cuDoubleComplex> mh((size_t)ns * nparam * kMaxCluster * kMaxCluster);
    BK(cudaMemcpyAsync(mh.data(), b->clum, sizeof(cuDoubleComplex) * mh.size(),
                       cudaMemcpyDeviceToHost, b->stream));
    BK(cudaStreamSynchronize(b->stream));
    std::vector<double> mu(kMaxCluster);
    for (long i = 0; i < ns; ++i) {
      const Cluster& cl = split[(size_t)i];
      for (int par = 0; par < nparam; ++par) {
        hermitian_eigvals(cl.c, mh.data() + ((size_t)i * nparam + par) * kMaxCluster * kMaxCluster,
                          kMaxCluster, mu.data());
        double add = 0.0;
        for (int r = 0; r < cl.c; ++r)
          add += cl.dg[(size_t)r] * 0.5 * (mu[(size_t)r] + mu[(size_t)(cl.c - 1 - r)]);
        dl_dparams[par] += add;
      }
    }
  }
  return SEP_OK;
}

int sep_bulk_solver_path(sep_bulk* b, int* batched) {
  if (!b || !batched) return fail(SEP_ERR_ARG, "sep_bulk_solver_path: bad arguments");
  *batched = b->path;
  return SEP_OK;
}

int sep_hermitian_lowest(const double* a, long n, long nmat, long nw, int vectors, double* w,
                         double* v) {
  if (!a || !w || (vectors && !v) || nmat < 1 || !sep::hb::supported((int)n, (int)nw))
    return fail(SEP_ERR_ARG, "sep_hermitian_lowest: 2 <= n <= 512, 1 <= nw <= min(n, 64), nmat >= 1");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return fail(SEP_ERR_NO_DEVICE, "sep_hermitian_lowest: no CUDA device");
  }
  const size_t nn = (size_t)n * n * nmat;
  double2* dA = nullptr;
  double* dw = nullptr;
  void* work = nullptr;
  cudaStream_t s = nullptr;
  auto done = [&](int r) {
    if (s) cudaStreamSynchronize(s);
    cudaFree(dA);
    cudaFree(dw);
    cudaFree(work);
    if (s) cudaStreamDestroy(s);
    return r;
  };
  const size_t wb = sep::hb::work_bytes((int)n, (int)nmat, (int)nw);
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&dA, sizeof(double2) * nn) != cudaSuccess ||
      cudaMalloc(&dw, sizeof(double) * n * nmat) != cudaSuccess || cudaMalloc(&work, wb) != cudaSuccess) {
    cudaGetLastError();
    return done(fail(SEP_ERR_NOMEM, "sep_hermitian_lowest: device allocation"));
  }
  cudaError_t e = cudaMemcpyAsync(dA, a, sizeof(double2) * nn, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = sep::hb::lowest(dA, (int)n, (int)nmat, (int)nw, vectors != 0, dw, work, s);
  for (long m = 0; e == cudaSuccess && m < nmat; ++m) {
    e = cudaMemcpyAsync(w + m * nw, dw + m * n, sizeof(double) * nw, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && vectors)
      e = cudaMemcpyAsync(v + 2 * m * nw * n, dA + (size_t)m * n * n, sizeof(double2) * nw * n,
                          cudaMemcpyDeviceToHost, s);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    char m[200];
    snprintf(m, sizeof m, "sep_hermitian_lowest: CUDA error %d (%s)", (int)e, cudaGetErrorString(e));
    return done(fail(SEP_ERR_CUDA, m));
  }
  if (vectors) {
    int bad = 0;
    if (sep::hb::failed_vectors(work, (int)n, (int)nmat, (int)nw, &bad, s) != cudaSuccess)
      return done(fail(SEP_ERR_CUDA, "sep_hermitian_lowest: status read"));
    if (bad) return done(fail(SEP_ERR_SOLVER, "sep_hermitian_lowest: inverse iteration did not converge"));
  }
  return done(SEP_OK);
}

int sep_bulk_set_eigensolver(sep_bulk* b, int mode) {
  if (!b || mode < 0 || mode > 1)
    return fail(SEP_ERR_ARG, "sep_bulk_set_eigensolver: mode 0 (cuSOLVER) or 1 (library)");
  b->native = mode;
  b->last_params.clear();
  return SEP_OK;
}

int sep_bulk_set_solver(sep_bulk* b, int batched) {
  if (!b || batched < 0 || batched > 1) return fail(SEP_ERR_ARG, "sep_bulk_set_solver: mode 0 or 1");
  b->batched = batched ? -1 : 0;
  b->last_params.clear();
  return SEP_OK;
}

int sep_bulk_destroy(sep_bulk* b) {
  if (!b) return SEP_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  void* bufs[] = {b->g, b->tau, b->types, b->kpts, b->params, b->v, b->h, b->wmat, b->w,
                  b->bands, b->dlde, b->partials, b->grad, b->info, b->dwork, b->clu,
                  b->cluy, b->clum, b->hbwork};
  for (void* p : bufs)
    if (p) cudaFree(p);
  if (b->sparams) cusolverDnDestroyParams(b->sparams);
  if (b->solver) cusolverDnDestroy(b->solver);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return SEP_OK;
}

}  // extern "C"
