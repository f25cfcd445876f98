// sep_heevb.cu -- the lowest eigenpairs of many small Hermitian matrices at
// once (the bulk fit's per-k-point problems, pseudopotFitting/diag.c:12-48,
// where the reference calls zheev for every k-point and keeps the lowest
// bands, fit.c:86-88).
//
// One CTA per matrix (n <= 512, column-major, both triangles stored):
//  1. k_hetrd: Householder reduction to real symmetric tridiagonal form with
//     LAPACK zhetd2's conventions (lower triangle; H_j = I - tau_j v_j v_j^H
//     with v_j(j+1) = 1 and a real beta_j, so T = Q^H A Q has a real
//     diagonal d and off-diagonal e).  Per step: the reflector of the next
//     column, p = tau A22 v, w = p - (tau/2)(p^H v) v and the rank-2 update
//     A22 -= v w^H + w v^H of the lower triangle.  Warps take columns (lanes
//     on consecutive rows: coalesced); for p each column adds A_ik v_k to
//     its rows' per-lane sums (scatter) and sum_{i>k} conj(A_ik) v_i to p_k
//     (gather), and the warps' scatter sums are added in a fixed order, so
//     the result does not depend on timing.  The reflectors stay below the
//     subdiagonal for the back-transformation.
//  2. k_stebz: the lowest nw eigenvalues of T by bisection on Sturm counts
//     (one thread per eigenvalue; the counts by the division-free continuant
//     recursion with exact power-of-two rescaling).
//  3. k_stein: their eigenvectors by inverse iteration (LAPACK dstein's
//     scheme): Gaussian elimination with partial pivoting of T - lambda I,
//     eigenvalues closer than 1e-3 ||T||_1 form a group whose vectors are
//     orthogonalised against each other (modified Gram-Schmidt), eigenvalues
//     inside a group closer than 10 eps |lambda| are moved apart by that much.
//  4. k_unmtr: x = H_0 H_1 ... H_{n-2} z for each vector (a warp per vector,
//     the vector in registers).
// On GB300 every FP64 operation goes through the FP64 pipe (about 2 FMAs per
// clock per SM); the reduction costs 8 n^3 / 3 FMAs per matrix.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <vector>

#include "sep_heevb.cuh"

namespace sep {
namespace hb {
namespace {

using Z = double2;
constexpr int kWarps = 16;
constexpr int kThreads = 32 * kWarps;

__device__ __forceinline__ Z zmk(double a, double b) {
  Z r;
  r.x = a;
  r.y = b;
  return r;
}
__device__ __forceinline__ Z zadd(Z a, Z b) { return zmk(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ Z zmul(Z a, Z b) { return zmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
// acc + a * b
__device__ __forceinline__ Z zfma(Z a, Z b, Z acc) {
  return zmk(fma(a.x, b.x, fma(-a.y, b.y, acc.x)), fma(a.x, b.y, fma(a.y, b.x, acc.y)));
}
// acc + conj(a) * b
__device__ __forceinline__ Z zfmac(Z a, Z b, Z acc) {
  return zmk(fma(a.x, b.x, fma(a.y, b.y, acc.x)), fma(a.x, b.y, fma(-a.y, b.x, acc.y)));
}
// acc - a * conj(b), four FMAs
__device__ __forceinline__ Z zfnmsc(Z a, Z b, Z acc) {
  return zmk(fma(-a.x, b.x, fma(-a.y, b.y, acc.x)), fma(-a.y, b.x, fma(a.x, b.y, acc.y)));
}
// acc - a * b, four FMAs
__device__ __forceinline__ Z zfnms(Z a, Z b, Z acc) {
  return zmk(fma(-a.x, b.x, fma(a.y, b.y, acc.x)), fma(-a.x, b.y, fma(-a.y, b.x, acc.y)));
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// 1. tridiagonal reduction; shared memory: v, w, p, gather sums (4 n complex)
//    and the warps' scatter sums (kWarps x n complex)
template <int MAXR>
__global__ void __launch_bounds__(kThreads, 1)
    k_hetrd(Z* __restrict__ Aall, int n, double* __restrict__ dall, double* __restrict__ eall,
            Z* __restrict__ tauall) {
  extern __shared__ __align__(16) unsigned char hb_smem[];
  Z* v = reinterpret_cast<Z*>(hb_smem);
  Z* w = v + n;
  Z* gs = w + n;                 // gather part of p per column
  Z* pw = gs + n;                // scatter parts: kWarps x n
  __shared__ double red[2 * kWarps];
  __shared__ Z sh_tau, sh_scale;
  __shared__ int sh_skip;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  Z* A = Aall + (size_t)blockIdx.x * n * n;
  double* d = dall + (size_t)blockIdx.x * n;
  double* e = eall + (size_t)blockIdx.x * n;
  Z* tau = tauall + (size_t)blockIdx.x * n;

  for (int j = 0; j < n - 1; ++j) {
    const int r0 = j + 1;
    // ---- reflector of column j (rows r0 .. n-1), warp 0
    if (warp == 0) {
      double part = 0.0;
      for (int i = r0 + 1 + lane; i < n; i += 32) {
        const Z x = A[(size_t)j * n + i];
        part = fma(x.x, x.x, fma(x.y, x.y, part));
      }
      const double xn2 = warp_sum(part);
      if (lane == 0) {
        d[j] = A[(size_t)j * n + j].x;
        const Z al = A[(size_t)j * n + r0];
        if (xn2 == 0.0 && al.y == 0.0) {  // already reduced: H_j = I
          sh_skip = 1;
          e[j] = al.x;
          tau[j] = zmk(0.0, 0.0);
        } else {
          const double beta = -copysign(sqrt(al.x * al.x + al.y * al.y + xn2), al.x);
          const Z t = zmk((beta - al.x) / beta, -al.y / beta);
          const double dx = al.x - beta, dy = al.y, dd = dx * dx + dy * dy;
          sh_scale = zmk(dx / dd, -dy / dd);  // 1 / (alpha - beta)
          sh_tau = t;
          sh_skip = 0;
          e[j] = beta;
          tau[j] = t;
        }
      }
    }
    __syncthreads();
    if (sh_skip) {  // uniform; the barrier keeps sh_skip until every thread has read it
      __syncthreads();
      continue;
    }
    const Z sc = sh_scale, tj = sh_tau;
    for (int i = r0 + tid; i < n; i += kThreads) {
      Z vi = zmk(1.0, 0.0);
      if (i > r0) {
        vi = zmul(A[(size_t)j * n + i], sc);
        A[(size_t)j * n + i] = vi;  // kept for the back-transformation
      }
      v[i] = vi;
    }
    __syncthreads();
    // ---- p = tau A22 v: warps on columns k, lanes on rows i >= k (each FP64
    // instruction of the loop has every lane working: on this part an FP64
    // warp instruction costs the same however many lanes are active); the
    // scatter sums of each warp in shared memory
    Z* mine = pw + (size_t)warp * n;
    for (int i = r0 + lane; i < n; i += 32) mine[i] = zmk(0.0, 0.0);
    __syncwarp();
    for (int k = r0 + warp; k < n; k += kWarps) {
      const Z vk = v[k];
      const Z* col = A + (size_t)k * n;
      Z g = zmk(0.0, 0.0);
      for (int i = k + lane; i < n; i += 32) {
        const Z a = col[i];
        mine[i] = zfma(a, vk, mine[i]);
        if (i > k) g = zfmac(a, v[i], g);
      }
      g.x = warp_sum(g.x);
      g.y = warp_sum(g.y);
      if (lane == 0) gs[k] = g;
    }
    __syncthreads();
    // p_i = tau (gather_i + sum_w scatter_w,i), then p^H v
    double px = 0.0, py = 0.0;
    for (int i = r0 + tid; i < n; i += kThreads) {
      Z s = gs[i];
#pragma unroll
      for (int q = 0; q < kWarps; ++q) s = zadd(s, pw[(size_t)q * n + i]);
      const Z pi = zmul(tj, s);
      w[i] = pi;
      const Z c = zfmac(pi, v[i], zmk(0.0, 0.0));  // conj(p_i) v_i
      px += c.x;
      py += c.y;
    }
    px = warp_sum(px);
    py = warp_sum(py);
    if (lane == 0) {
      red[warp] = px;
      red[kWarps + warp] = py;
    }
    __syncthreads();
    double dx = 0.0, dy = 0.0;
#pragma unroll
    for (int q = 0; q < kWarps; ++q) {
      dx += red[q];
      dy += red[kWarps + q];
    }
    // w = p + alpha v, alpha = -tau (p^H v) / 2
    const Z alpha = zmul(zmk(-0.5 * tj.x, -0.5 * tj.y), zmk(dx, dy));
    for (int i = r0 + tid; i < n; i += kThreads) w[i] = zfma(alpha, v[i], w[i]);
    __syncthreads();
    // ---- A22 -= v w^H + w v^H, lower triangle (v_i, w_i from shared memory)
    for (int k = r0 + warp; k < n; k += kWarps) {
      const Z vk = v[k], wk = w[k];
      Z* col = A + (size_t)k * n;
      for (int i = k + lane; i < n; i += 32) {
        Z a = zfnmsc(v[i], wk, col[i]);
        a = zfnmsc(w[i], vk, a);
        if (i == k) a.y = 0.0;  // the diagonal stays real
        col[i] = a;
      }
    }
    __syncthreads();
  }
  if (tid == 0) {
    d[n - 1] = A[(size_t)(n - 1) * n + n - 1].x;
    e[n - 1] = 0.0;
  }
}

// ---------------------------------------------------------------------------
// Sturm count: eigenvalues of T below x = sign changes in the leading
// principal minors p_i = (d_i - x) p_{i-1} - e_{i-1}^2 p_{i-2} (p_{-1} = 1),
// two FP64 operations per step and no division.  When the larger of the two
// current minors leaves [2^-400, 2^400], both are multiplied by the same
// exact power of two (integer work on the exponent fields) that brings the
// larger near 1; a smaller one that would underflow becomes 0.  A minor that
// is exactly zero counts as having the sign opposite to its predecessor (as
// LAPACK's dlaebz, whose zero pivots count as negative).
__device__ __forceinline__ int expo_field(double v) {
  return (int)((__double_as_longlong(v) >> 52) & 0x7ff);
}
__device__ __forceinline__ double scale_pow2(double v, int k) {  // v 2^k
  const int ex = expo_field(v);
  if (ex == 0) return v;                 // zero
  if (ex + k <= 0) return copysign(0.0, v);  // underflow
  return __longlong_as_double(__double_as_longlong(v) + ((long long)k << 52));
}
__device__ int sturm_count(const double* d, const double* e2, int n, double x) {
  double pm = 1.0, p = d[0] - x;
  int c = 0;
  bool sprev = false;  // p_{-1} = 1 is positive
  for (int i = 0;; ++i) {
    // sign and zero tests on the bits (integer work, not the FP64 pipe)
    const long long pb = __double_as_longlong(p);
    const bool sn = (pb < 0 && (pb << 1) != 0) || ((pb << 1) == 0 && !sprev);
    c += (sn != sprev);
    sprev = sn;
    if (i == n - 1) break;
    const double q = fma(d[i + 1] - x, p, -e2[i] * pm);
    pm = p;
    p = q;
    const int emx = max(expo_field(p), expo_field(pm));
    if (emx > 1023 + 400 || emx < 1023 - 400) {
      const int k = 1023 - emx;
      p = scale_pow2(p, k);
      pm = scale_pow2(pm, k);
    }
  }
  return c;
}

// 2. lowest nw eigenvalues, one thread each; w[nw .. n-1] = NaN
__global__ void k_stebz(const double* __restrict__ dall, const double* __restrict__ eall, int n,
                        int nw, double* __restrict__ wall, double* __restrict__ tnorm) {
  extern __shared__ double sb[];
  double* d = sb;
  double* e2 = sb + n;
  __shared__ double sh_lo, sh_hi, sh_piv;
  const double* dg = dall + (size_t)blockIdx.x * n;
  const double* eg = eall + (size_t)blockIdx.x * n;
  double* w = wall + (size_t)blockIdx.x * n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    d[i] = dg[i];
    e2[i] = (i < n - 1) ? eg[i] * eg[i] : 0.0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double lo = d[0], hi = d[0], emax = 0.0, onenrm = 0.0;
    for (int i = 0; i < n; ++i) {
      const double r = (i > 0 ? fabs(eg[i - 1]) : 0.0) + (i < n - 1 ? fabs(eg[i]) : 0.0);
      lo = fmin(lo, d[i] - r);
      hi = fmax(hi, d[i] + r);
      onenrm = fmax(onenrm, fabs(d[i]) + r);
      emax = fmax(emax, e2[i]);
    }
    const double span = fmax(hi - lo, DBL_MIN);
    sh_lo = lo - 2.1 * DBL_EPSILON * span - 1e-300;
    sh_hi = hi + 2.1 * DBL_EPSILON * span + 1e-300;
    sh_piv = DBL_MIN * fmax(1.0, emax);
    tnorm[blockIdx.x] = onenrm;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    if (t >= nw) {
      w[t] = __longlong_as_double(0x7ff8000000000000LL);  // NaN: not computed
      continue;
    }
    double lo = sh_lo, hi = sh_hi;
    for (int it = 0; it < 200; ++it) {
      const double mid = 0.5 * (lo + hi);
      if (hi - lo <= 2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)) + sh_piv || mid <= lo ||
          mid >= hi)
        break;
      if (sturm_count(d, e2, n, mid) > t)
        hi = mid;
      else
        lo = mid;
    }
    w[t] = 0.5 * (lo + hi);
  }
}

// ---------------------------------------------------------------------------
// 3. eigenvectors of T by inverse iteration.  Thread 0 splits the nw
//    eigenvalues into groups; each group's vectors are made by one thread.
//    Scratch per thread: the LU of T - lambda I (4 n) and two vectors.
constexpr int kSteinThreads = 64;

__device__ double lcg_uniform(unsigned long long& s) {  // (-1, 1)
  s = s * 6364136223846793005ULL + 1442695040888963407ULL;
  return (double)(s >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

// The LU rows, the iterate and the vectors live in global scratch that this
// thread both writes and reads back in the same loops (x[k + 1] after x[k]):
// no __restrict__ on those pointers, and the recurrences are not unrolled, so
// that no load is hoisted above the store it depends on.  (With restrict
// qualifiers here the compiled forward elimination read every x[k] from before
// the loop.)
__global__ void __launch_bounds__(kSteinThreads)
    k_stein(const double* dall, const double* eall, const double* wall, const double* tnorm,
            int n, int nw, double* zall, double* scratch, int* info) {
  __shared__ int gstart[kMaxWanted + 1];
  __shared__ int ngroups;
  const int m = blockIdx.x;
  const double* d = dall + (size_t)m * n;
  const double* e = eall + (size_t)m * n;
  const double* w = wall + (size_t)m * n;
  double* Zm = zall + (size_t)m * n * nw;
  const double onenrm = tnorm[m];
  const double ortol = 1e-3 * onenrm;
  if (threadIdx.x == 0) {
    int g = 0;
    gstart[g++] = 0;
    for (int i = 1; i < nw; ++i)
      if (w[i] - w[i - 1] > ortol) gstart[g++] = i;
    gstart[g] = nw;
    ngroups = g;
  }
  __syncthreads();
  const double eps = DBL_EPSILON;
  const double dtpcrt = sqrt(0.1 / n);
  for (int grp = threadIdx.x; grp < ngroups; grp += blockDim.x) {
    double* sc = scratch + ((size_t)m * kSteinThreads + threadIdx.x) * 6 * n;
    double* u0 = sc;          // U diagonal
    double* u1 = sc + n;      // first superdiagonal
    double* u2 = sc + 2 * n;  // second superdiagonal
    double* lm = sc + 3 * n;  // multipliers
    double* x = sc + 4 * n;
    char* piv = reinterpret_cast<char*>(sc + 5 * n);
    double xjm = 0.0;
    for (int jj = gstart[grp]; jj < gstart[grp + 1]; ++jj) {
      double xj = w[jj];
      if (jj > gstart[grp]) {
        const double pertol = 10.0 * fabs(eps * xj);
        if (xj - xjm < pertol) xj = xjm + pertol;
      }
      xjm = xj;
      // T - xj I = P L U (partial pivoting): row k holds (u0, u1, u2)
      double a = d[0] - xj, c = (n > 1) ? e[0] : 0.0;
      for (int k = 0; k < n - 1; ++k) {
        const double b = e[k];                     // subdiagonal (k+1, k)
        const double an = d[k + 1] - xj;          // next row's diagonal
        const double cn = (k + 1 < n - 1) ? e[k + 1] : 0.0;
        if (fabs(a) >= fabs(b)) {
          const double l = (a != 0.0) ? b / a : 0.0;
          u0[k] = a;
          u1[k] = c;
          u2[k] = 0.0;
          lm[k] = l;
          piv[k] = 0;
          a = an - l * c;
          c = cn;
        } else {
          const double l = a / b;
          u0[k] = b;
          u1[k] = an;
          u2[k] = cn;
          lm[k] = l;
          piv[k] = 1;
          a = c - l * an;
          c = -l * cn;
        }
      }
      u0[n - 1] = a;
      // small pivots are perturbed (dlagts with a tolerance)
      const double tol = fmax(eps * onenrm, DBL_MIN);
      for (int k = 0; k < n; ++k)
        if (fabs(u0[k]) < tol) u0[k] = (u0[k] < 0.0) ? -tol : tol;
      unsigned long long seed = 0x9E3779B97F4A7C15ULL * (unsigned long long)(m * 4096 + jj + 1);
      for (int i = 0; i < n; ++i) x[i] = lcg_uniform(seed);
      int nrmchk = 0;
      for (int its = 0; its < 5; ++its) {
        double asum = 0.0;
        for (int i = 0; i < n; ++i) asum += fabs(x[i]);
        const double scl = n * onenrm * fmax(eps, fabs(u0[n - 1])) / fmax(asum, DBL_MIN);
        for (int i = 0; i < n; ++i) x[i] *= scl;
        // solve P L U y = x: forward with the row interchanges, then U
#pragma unroll 1
        for (int k = 0; k < n - 1; ++k) {
          if (piv[k]) {
            const double t = x[k];
            x[k] = x[k + 1];
            x[k + 1] = t - lm[k] * x[k];
          } else {
            x[k + 1] -= lm[k] * x[k];
          }
        }
#pragma unroll 1
        for (int k = n - 1; k >= 0; --k) {
          double s = x[k];
          if (k + 1 < n) s -= u1[k] * x[k + 1];
          if (k + 2 < n) s -= u2[k] * x[k + 2];
          x[k] = s / u0[k];
        }
        // orthogonalise against the group's earlier vectors
        for (int q = gstart[grp]; q < jj; ++q) {
          const double* zq = Zm + (size_t)q * n;
          double dot = 0.0;
          for (int i = 0; i < n; ++i) dot += zq[i] * x[i];
          for (int i = 0; i < n; ++i) x[i] -= dot * zq[i];
        }
        double nrm = 0.0;
        for (int i = 0; i < n; ++i) nrm = fmax(nrm, fabs(x[i]));
        if (nrm < dtpcrt) continue;
        if (++nrmchk < 3) continue;
        break;
      }
      if (nrmchk == 0 && info) atomicAdd(info + m, 1);  // no growth: not accepted by dstein
      double s2 = 0.0;
      int jmax = 0;
      for (int i = 0; i < n; ++i) {
        s2 += x[i] * x[i];
        if (fabs(x[i]) > fabs(x[jmax])) jmax = i;
      }
      double scl = 1.0 / sqrt(s2);
      if (x[jmax] < 0.0) scl = -scl;
      double* zj = Zm + (size_t)jj * n;
      for (int i = 0; i < n; ++i) zj[i] = x[i] * scl;
    }
  }
}

// ---------------------------------------------------------------------------
// 4. X = Q Z: warps on vectors, the vector in shared memory, lanes on the
//    rows of each reflector
template <int MAXR>
__global__ void __launch_bounds__(kThreads)
    k_unmtr(const Z* __restrict__ Aall, const Z* __restrict__ tauall,
            const double* __restrict__ zall, int n, int nw, Z* __restrict__ xall) {
  extern __shared__ __align__(16) unsigned char hb_smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int m = blockIdx.x;
  const Z* A = Aall + (size_t)m * n * n;
  const Z* tau = tauall + (size_t)m * n;
  Z* x = reinterpret_cast<Z*>(hb_smem) + (size_t)warp * n;
  for (int c = warp; c < nw; c += kWarps) {
    const double* z = zall + ((size_t)m * nw + c) * n;
    for (int i = lane; i < n; i += 32) x[i] = zmk(z[i], 0.0);
    __syncwarp();
    for (int j = n - 2; j >= 0; --j) {
      const Z tj = tau[j];
      if (tj.x == 0.0 && tj.y == 0.0) continue;
      const Z* col = A + (size_t)j * n;
      Z s = zmk(0.0, 0.0);  // v^H x
      for (int i = j + 1 + lane; i < n; i += 32)
        s = zfmac(i == j + 1 ? zmk(1.0, 0.0) : col[i], x[i], s);
      s.x = warp_sum(s.x);
      s.y = warp_sum(s.y);
      const Z f = zmul(tj, s);
      for (int i = j + 1 + lane; i < n; i += 32) {
        const Z vi = (i == j + 1) ? zmk(1.0, 0.0) : col[i];
        x[i] = zfnms(f, vi, x[i]);
      }
      __syncwarp();
    }
    Z* xo = xall + ((size_t)m * nw + c) * n;
    for (int i = lane; i < n; i += 32) xo[i] = x[i];
    __syncwarp();
  }
}

// the vectors into the first nw columns of each matrix
__global__ void k_put_vectors(const Z* __restrict__ xall, int n, int nw, long nmat,
                              Z* __restrict__ Aall) {
  const long per = (long)n * nw;
  for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < nmat * per;
       t += (long)gridDim.x * blockDim.x) {
    const long m = t / per, r = t - m * per;
    Aall[m * (long)n * n + r] = xall[t];
  }
}

template <int MAXR> size_t hetrd_smem(int n) { return (size_t)(3 + kWarps) * n * sizeof(Z); }

template <int MAXR>
cudaError_t run_all(Z* A, int n, int nmat, int nw, bool vectors, double* w, const Work& wk,
                    cudaStream_t s) {
  // the shared-memory limits are set to what the largest n of this
  // instantiation needs, the same value from every thread: calls for
  // different n may run at once from several host threads
  const size_t smem = hetrd_smem<MAXR>(n);
  cudaError_t e = cudaFuncSetAttribute(k_hetrd<MAXR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)hetrd_smem<MAXR>(32 * MAXR));
  if (e != cudaSuccess) return e;
  k_hetrd<MAXR><<<nmat, kThreads, smem, s>>>(A, n, wk.d, wk.e, wk.tau);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  k_stebz<<<nmat, 128, 2 * n * sizeof(double), s>>>(wk.d, wk.e, n, nw, w, wk.tnorm);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (!vectors) return cudaSuccess;
  if ((e = cudaMemsetAsync(wk.info, 0, sizeof(int) * nmat, s)) != cudaSuccess) return e;
  k_stein<<<nmat, kSteinThreads, 0, s>>>(wk.d, wk.e, w, wk.tnorm, n, nw, wk.z, wk.scratch,
                                         wk.info);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const size_t usmem = (size_t)kWarps * n * sizeof(Z);
  if ((e = cudaFuncSetAttribute(k_unmtr<MAXR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)((size_t)kWarps * 32 * MAXR * sizeof(Z)))) != cudaSuccess)
    return e;
  k_unmtr<MAXR><<<nmat, kThreads, usmem, s>>>(A, wk.tau, wk.z, n, nw, wk.x);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const long tot = (long)nmat * n * nw;
  k_put_vectors<<<(unsigned)std::min<long>((tot + 255) / 256, 152L * 16), 256, 0, s>>>(
      wk.x, n, nw, nmat, A);
  return cudaGetLastError();
}

}  // namespace

size_t work_bytes(int n, int nmat, int nw) {
  const size_t nm = (size_t)nmat;
  return nm * n * sizeof(double) * 2       // d, e
         + nm * n * sizeof(Z)              // tau
         + nm * sizeof(double)             // |T|_1
         + nm * sizeof(int) + 64           // info
         + nm * n * nw * sizeof(double)    // tridiagonal eigenvectors
         + nm * n * nw * sizeof(Z)         // eigenvectors of A
         + nm * kSteinThreads * 6 * n * sizeof(double) + 8 * 256;
}

Work carve(void* base, int n, int nmat, int nw) {
  Work wk;
  char* p = static_cast<char*>(base);
  auto take = [&](size_t bytes) {
    char* q = p;
    p += (bytes + 255) & ~(size_t)255;
    return q;
  };
  const size_t nm = (size_t)nmat;
  wk.d = reinterpret_cast<double*>(take(nm * n * sizeof(double)));
  wk.e = reinterpret_cast<double*>(take(nm * n * sizeof(double)));
  wk.tau = reinterpret_cast<Z*>(take(nm * n * sizeof(Z)));
  wk.tnorm = reinterpret_cast<double*>(take(nm * sizeof(double)));
  wk.info = reinterpret_cast<int*>(take(nm * sizeof(int)));
  wk.z = reinterpret_cast<double*>(take(nm * n * nw * sizeof(double)));
  wk.x = reinterpret_cast<Z*>(take(nm * n * nw * sizeof(Z)));
  wk.scratch = reinterpret_cast<double*>(take(nm * kSteinThreads * 6 * n * sizeof(double)));
  return wk;
}

bool supported(int n, int nw) { return n >= 2 && n <= 512 && nw >= 1 && nw <= kMaxWanted && nw <= n; }

cudaError_t lowest(Z* A, int n, int nmat, int nw, bool vectors, double* w, void* work,
                   cudaStream_t s) {
  if (!supported(n, nw) || nmat < 1) return cudaErrorInvalidValue;
  const Work wk = carve(work, n, nmat, nw);
  if (n <= 128) return run_all<4>(A, n, nmat, nw, vectors, w, wk, s);
  if (n <= 256) return run_all<8>(A, n, nmat, nw, vectors, w, wk, s);
  return run_all<16>(A, n, nmat, nw, vectors, w, wk, s);
}

cudaError_t failed_vectors(const void* work, int n, int nmat, int nw, int* host_count,
                           cudaStream_t s) {
  const Work wk = carve(const_cast<void*>(work), n, nmat, nw);
  std::vector<int> h((size_t)nmat);
  cudaError_t e = cudaMemcpyAsync(h.data(), wk.info, sizeof(int) * nmat, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  int c = 0;
  for (int v : h) c += v;
  *host_count = c;
  return e;
}

}  // namespace hb
}  // namespace sep
