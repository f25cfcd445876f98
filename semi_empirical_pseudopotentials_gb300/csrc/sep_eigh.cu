// sep_eigh.cu -- FP64 symmetric eigensolver on the GPU, written for the
// subspace stages (the Gram matrices of ortho, filter/ortho.c:11-52, and the
// projected H of Rayleigh-Ritz, filter/Hmat.c:11-86, where the reference calls
// LAPACK dgesvd / dsyev).  A = V diag(w) V^T for a dense symmetric n x n A;
// eigenvalues ascending, eigenvectors as the columns of V (column-major,
// V[i + j n] = component i of vector j, in place of A).
//
// Three stages:
//  1. Householder tridiagonalisation A = Q T Q^T (LAPACK's dsytd2 scheme:
//     reflector H_k = I - tau v v^T with v[k+1] = 1 annihilates column k below
//     the subdiagonal; p = tau A22 v, w = p - (tau/2)(p.v) v,
//     A22 -= v w^T + w v^T).  One cooperative kernel runs all steps with one
//     grid barrier per step: each block forms the next reflector itself from
//     the next row updated on the fly, then one pass over the trailing rows
//     applies the update and accumulates the next step's p.  The rows of a
//     step are spread over all blocks: on this part the FP64 pipe (about 2
//     FMAs per clock per SM) is the scarce resource.
//  2. The eigenpairs of T by divide and conquer (Cuppen's method): T is
//     split recursively into leaves of at most 8 rows, T = diag(T1, T2) +
//     rho u u^T at each split; the leaves are solved by the implicit QL
//     iteration with Wilkinson shifts (EISPACK tql2, one warp per leaf);
//     each merge deflates negligible and near-equal components (Givens
//     rotations), finds the roots of the secular equation
//     1 + rho sum z_i^2 / (d_i - lambda) = 0 by safeguarded Newton steps in
//     the distance to the nearer pole (bisection of the bracket as fallback), recomputes z from the roots (Loewner's formula, which
//     keeps the merged eigenvectors orthogonal) and forms the eigenvectors
//     with one product per merge.  The deflation scan and the sorting run on
//     the host (O(n) per level).
//  3. Back-transformation V = Q Y: each column of Y passes through the
//     reflectors H_{n-3} .. H_0 (a warp per column).
// No library is called.  Every kernel's loop bounds are fixed; there are no
// spin-waits.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <vector>

#include "sep_eigh.cuh"

namespace sep {
namespace eigh {

namespace cg = cooperative_groups;

namespace {

constexpr int kLeaf = 8;   // rows of a leaf (one warp; the QL recurrence is serial FP64)
constexpr int kT = 256;    // threads per block
constexpr double kEps = 2.220446049250313e-16;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ double warp_prod(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v *= __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---- 1. tridiagonalisation -------------------------------------------------

// Block-wide reductions (blockDim.x = kT) through red[kT / 32].
__device__ __forceinline__ double block_max(double v, double* red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = warp_max(v);
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double m = 0.0;
  for (int q = 0; q < kT / 32; ++q) m = fmax(m, red[q]);
  return m;
}
__device__ __forceinline__ double block_sum(double v, double* red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double m = 0.0;
  for (int q = 0; q < kT / 32; ++q) m += red[q];
  return m;
}

// One grid barrier per step.  Every block keeps the current reflector v_k
// in shared memory (vk) and builds the next one itself: row k+1 after step
// k's rank-2 update, x_j = A[k+1][j] - (v_{k+1} p_j + u_{k+1} v_j), is
// formed on the fly from the stored row (rows and columns <= k+1 are not
// written back: later steps read only the trailing block), and the
// reflector of x (dlarfg's conventions, scaled by max |x| against
// over/underflow) goes to vn.  One pass over the trailing rows i >= k+2 then
// applies step k's update, A[i][j] -= v_i p_j + u_i v_j with
// u_i = p_i - 2 c v_i and c = tau_k (p.v) / 2, and accumulates step k+1's
// p_i = tau_{k+1} sum_j A[i][j] vn_j from the updated values.  Every block
// computes the reflectors identically; block 0 stores them (Vh, tau, d, e).
// Rows are owned by warps: row r by warp (r % G, (r / G) % 8), so that
// consecutive rows sit on different SMs.  p: 2 x n (by step parity);
// part: 2 x gridDim.x partial sums of p.v (deterministic order).
__global__ void __launch_bounds__(kT) k_sytrd(double* __restrict__ A, int n, double* d,
                                              double* e, double* tau, double* Vh,
                                              double* __restrict__ pbuf, double* part) {
  cg::grid_group grid = cg::this_grid();
  extern __shared__ double sm[];
  double* vbuf = sm;         // 2 x n: the reflectors of steps k (k & 1) and k + 1
  double* red = sm + 2 * n;  // kT / 32
  __shared__ double sc[4];   // tau, beta, scale of the reflector being built
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int W = gridDim.x * (kT / 32);
  const int gw = blockIdx.x + gridDim.x * wib;
  auto first = [&](int r0) { return r0 + ((gw - r0) % W + W) % W; };
  // the reflector of step s from x[j] (j in [s+1, n), held in vn): vn <- v
  auto reflector = [&](int s, double* vn) {
    // |x| unscaled; scaled by max |x| only when the sum of squares under- or
    // overflows
    double ss = 0.0;
    for (int j = s + 2 + threadIdx.x; j < n; j += kT) ss = fma(vn[j], vn[j], ss);
    ss = block_sum(ss, red);
    double xnorm = sqrt(ss);
    if (!(ss > 1e-290 && ss < 1e290)) {
      double amax = 0.0;
      for (int j = s + 2 + threadIdx.x; j < n; j += kT) amax = fmax(amax, fabs(vn[j]));
      amax = block_max(amax, red);
      xnorm = 0.0;
      if (amax > 0.0) {
        const double inv = 1.0 / amax;
        double sq = 0.0;
        for (int j = s + 2 + threadIdx.x; j < n; j += kT) {
          const double q = vn[j] * inv;
          sq += q * q;
        }
        xnorm = amax * sqrt(block_sum(sq, red));
      }
    }
    if (threadIdx.x == 0) {
      const double alpha = vn[s + 1];
      if (xnorm == 0.0) {
        sc[0] = 0.0;
        sc[1] = alpha;
        sc[2] = 0.0;
      } else {
        const double beta = -copysign(hypot(alpha, xnorm), alpha);
        sc[0] = (beta - alpha) / beta;
        sc[1] = beta;
        sc[2] = 1.0 / (alpha - beta);
      }
    }
    __syncthreads();
    const double scal = sc[2];
    for (int j = s + 2 + threadIdx.x; j < n; j += kT) vn[j] *= scal;
    if (threadIdx.x == 0) vn[s + 1] = 1.0;
    __syncthreads();
    if (blockIdx.x == 0) {
      for (int j = s + 1 + threadIdx.x; j < n; j += kT) Vh[(size_t)s * n + j] = vn[j];
      if (threadIdx.x == 0) {
        e[s] = sc[1];
        tau[s] = sc[0];
      }
    }
  };
  // step 0: the reflector of row 0 as stored, then p = tau_0 A v_0
  {
    double* v0 = vbuf;
    for (int j = 1 + threadIdx.x; j < n; j += kT) v0[j] = A[j];
    if (blockIdx.x == 0 && threadIdx.x == 0) d[0] = A[0];
    __syncthreads();
    reflector(0, v0);
    const double t0 = sc[0];
    double mine = 0.0;
    for (int i = first(1); i < n; i += W) {
      const double* row = A + (size_t)i * n;
      double s0 = 0.0;
      for (int j = 1 + lane; j < n; j += 32) s0 += row[j] * v0[j];
      const double pi = t0 * warp_sum(s0);
      if (lane == 0) pbuf[i] = pi;
      mine += pi * v0[i];
    }
    const double b = block_sum(lane == 0 ? mine : 0.0, red);
    if (threadIdx.x == 0) part[blockIdx.x] = b;
  }
  grid.sync();
  for (int k = 0; k <= n - 3; ++k) {
    const double* v = vbuf + (size_t)(k & 1) * n;
    double* vn = vbuf + (size_t)((k + 1) & 1) * n;
    const double* p = pbuf + (size_t)(k & 1) * n;
    double* pn = pbuf + (size_t)((k + 1) & 1) * n;
    const double t = sc[0];  // tau_k of this block's reflector
    double pv = 0.0;  // the block partials, summed by every warp in the same order
    for (int b = lane; b < (int)gridDim.x; b += 32) pv += part[(k & 1) * gridDim.x + b];
    pv = warp_sum(pv);
    const double c = 0.5 * t * pv;
    // row k+1 after step k's update, on the fly
    const double v1 = v[k + 1], u1 = p[k + 1] - 2.0 * c * v1;
    const double* row1 = A + (size_t)(k + 1) * n;
    for (int j = k + 1 + threadIdx.x; j < n; j += kT)
      vn[j] = row1[j] - fma(v1, p[j], u1 * v[j]);
    __syncthreads();
    if (blockIdx.x == 0 && threadIdx.x == 0) d[k + 1] = vn[k + 1];
    const bool last = k + 1 > n - 3;
    double tn = 0.0;
    if (!last) {
      reflector(k + 1, vn);
      tn = sc[0];
    } else if (blockIdx.x == 0 && threadIdx.x == 0) {
      // n - 2: no reflector; the last subdiagonal (row n-2 is not written
      // this step); the last diagonal comes from the owner of row n-1 below
      e[n - 2] = vn[n - 1];
      tau[n - 2] = 0.0;
      tau[n - 1] = 0.0;
    }
    // step k's update of rows i >= k+2 (columns >= k+2) and step k+1's p
    double mine = 0.0;
    for (int i = first(k + 2); i < n; i += W) {
      double* row = A + (size_t)i * n;
      const double vi = v[i], ui = p[i] - 2.0 * c * vi;
      double s0 = 0.0;
      for (int j = k + 2 + lane; j < n; j += 32) {
        const double a = row[j] - fma(vi, p[j], ui * v[j]);
        row[j] = a;
        s0 = fma(a, vn[j], s0);
        if (last && i == n - 1 && j == n - 1) d[n - 1] = a;
      }
      if (!last) {
        const double pi = tn * warp_sum(s0);
        if (lane == 0) pn[i] = pi;
        mine += pi * vn[i];
      }
    }
    if (!last) {
      const double b = block_sum(lane == 0 ? mine : 0.0, red);
      if (threadIdx.x == 0) part[((k + 1) & 1) * gridDim.x + blockIdx.x] = b;
    }
    grid.sync();
  }
}

// ---- 3. back-transformation --------------------------------------------------
// column j of Z (column-major, in place): Z[:, j] <- H_0 H_1 .. H_{n-3} Z[:, j]
__global__ void __launch_bounds__(kT) k_ormtr(double* __restrict__ Z, int n,
                                              const double* __restrict__ Vh,
                                              const double* __restrict__ tau) {
  const int lane = threadIdx.x & 31;
  const int j = blockIdx.x * (kT / 32) + (threadIdx.x >> 5);
  if (j >= n) return;
  double* z = Z + (size_t)j * n;
  for (int k = n - 3; k >= 0; --k) {
    const double t = tau[k];
    if (t == 0.0) continue;
    const double* v = Vh + (size_t)k * n;
    double s = 0.0;
    for (int i = k + 1 + lane; i < n; i += 32) s += v[i] * z[i];
    s = t * warp_sum(s);
    for (int i = k + 1 + lane; i < n; i += 32) z[i] -= s * v[i];
  }
}

// ---- 2. divide and conquer ----------------------------------------------------

// Leaves: the implicit QL iteration with Wilkinson shifts (EISPACK tql2, as
// restated in Numerical Recipes' tqli) on rows [lo, hi) of T, one warp each.
// d[i] and e[i] live in lane i's registers; the scalar recurrence reads them
// with shuffles and every lane computes it (identical values), the lane that
// owns an entry keeping the new value; lane r updates row r of the leaf's
// eigenvector matrix in shared memory.  Output: the leaf's eigenvalues
// ascending in lam[lo..hi), its eigenvectors in Q's diagonal block
// (column-major, leading dimension n).  status |= 1 when a leaf needs more
// than 64 iterations for one eigenvalue.
__global__ void __launch_bounds__(32) k_leaf_ql(const double* __restrict__ dmod,
                                               const double* __restrict__ e0,
                                               const int* __restrict__ leaf_lo, int nleaf,
                                               int n, double* __restrict__ lam,
                                               double* __restrict__ Q, int* status) {
  __shared__ double Z[32][kLeaf + 1];  // a row per lane (lanes >= s carry unused rows)
  const int leaf = blockIdx.x;
  if (leaf >= nleaf) return;
  const int lo = leaf_lo[leaf], hi = leaf_lo[leaf + 1], s = hi - lo;
  const int r = threadIdx.x;
  const unsigned full = 0xffffffffu;
  for (int c = 0; c < kLeaf; ++c) Z[r][c] = (r == c) ? 1.0 : 0.0;
  double dr = (r < s) ? dmod[lo + r] : 0.0;
  double er = (r < s - 1) ? e0[lo + r] : 0.0;
  auto D = [&](int i) { return __shfl_sync(full, dr, i); };
  auto E = [&](int i) { return __shfl_sync(full, er, i); };
  bool bad = false;
  for (int l = 0; l < s && !bad; ++l) {
    int iter = 0;
    for (;;) {
      int m = l;
      for (; m < s - 1; ++m) {
        const double dd = fabs(D(m)) + fabs(D(m + 1));
        if (fabs(E(m)) <= kEps * dd) break;
      }
      if (m == l) break;
      if (++iter > 64) {
        bad = true;
        break;
      }
      const double dl = D(l), el = E(l);
      double g = (D(l + 1) - dl) / (2.0 * el);
      double rr = hypot(g, 1.0);
      g = D(m) - dl + el / (g + copysign(rr, g));
      double sn = 1.0, cs = 1.0, p = 0.0;
      bool under = false;
      for (int i = m - 1; i >= l; --i) {
        const double ei = E(i);
        const double f = sn * ei, b = cs * ei;
        rr = hypot(f, g);
        if (r == i + 1) er = rr;  // e[i+1] = r
        if (rr == 0.0) {
          if (r == i + 1) dr -= p;
          if (r == m) er = 0.0;
          under = true;
          break;
        }
        sn = f / rr;
        cs = g / rr;
        const double di1 = D(i + 1), di = D(i);
        g = di1 - p;
        rr = (di - g) * sn + 2.0 * cs * b;
        p = sn * rr;
        if (r == i + 1) dr = g + p;
        g = cs * rr - b;
        const double z1 = Z[r][i + 1], z0 = Z[r][i];
        Z[r][i + 1] = sn * z0 + cs * z1;
        Z[r][i] = cs * z0 - sn * z1;
      }
      if (under) continue;
      if (r == l) {
        dr -= p;
        er = g;
      }
      if (r == m) er = 0.0;
    }
  }
  if (bad && r == 0) atomicOr(status, 1);
  __syncwarp();
  // ascending order: the rank of each lane's eigenvalue (ties by index)
  int rank = 0;
  for (int i = 0; i < s; ++i) {
    const double x = D(i);
    if (r < s && (x < dr || (x == dr && i < r))) ++rank;
  }
  if (r < s) {
    lam[lo + rank] = dr;
    for (int q = 0; q < s; ++q) Q[(size_t)(lo + rank) * n + (lo + q)] = Z[q][r];
  }
}

// z of every merge of one level: per merge, the last row of the left child's
// eigenvectors then sgn * the first row of the right child's, each / sqrt(2)
__global__ void k_merge_z(const double* __restrict__ Q, int n, const int* __restrict__ mlo,
                          const int* __restrict__ mmid, const int* __restrict__ mhi,
                          const double* __restrict__ sgn, int nmerge, double* __restrict__ z) {
  const int m = blockIdx.y;
  if (m >= nmerge) return;
  const int lo = mlo[m], mid = mmid[m], hi = mhi[m];
  const double r2 = 0.70710678118654752440;
  for (int j = lo + blockIdx.x * blockDim.x + threadIdx.x; j < hi; j += gridDim.x * blockDim.x)
    z[j] = (j < mid) ? Q[(size_t)j * n + (mid - 1)] * r2 : sgn[m] * Q[(size_t)j * n + mid] * r2;
}

// Givens rotations of columns of Q: rot[k] = (ci, cj, c, s): col_i <- c col_i
// + s col_j, col_j <- -s col_i + c col_j, in order, rows [lo, hi) of merge m
// (column indices global)
__global__ void k_rotate(double* __restrict__ Q, int n, const int* __restrict__ mlo,
                         const int* __restrict__ mhi, const int* __restrict__ rot_off,
                         const int* __restrict__ rot_idx, const double* __restrict__ rot_cs,
                         int nmerge) {
  const int m = blockIdx.y;
  if (m >= nmerge) return;
  const int lo = mlo[m], hi = mhi[m];
  const int r = lo + blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= hi) return;
  for (int k = rot_off[m]; k < rot_off[m + 1]; ++k) {
    const size_t ci = (size_t)rot_idx[2 * k], cj = (size_t)rot_idx[2 * k + 1];
    const double c = rot_cs[2 * k], s = rot_cs[2 * k + 1];
    const double a = Q[ci * n + r], b = Q[cj * n + r];
    Q[ci * n + r] = c * a + s * b;
    Q[cj * n + r] = -s * a + c * b;
  }
}

// secular roots: one warp per root.  Per merge m: kk = cnt[m] poles dn
// (ascending) and weights zn at off[m]; rho = rho[m].  Root j lies in
// (dn_j, dn_{j+1}) (the last in (dn_{kk-1}, dn_{kk-1} + rho sum z^2]); it is
// found in tau = lambda - dn_o, o the nearer pole, on
// f(tau) = 1 + rho sum_i z_i^2 / ((dn_i - dn_o) - tau).
__global__ void k_secular(const double* __restrict__ dn, const double* __restrict__ zn,
                          const int* __restrict__ off, const int* __restrict__ cnt,
                          const double* __restrict__ rho, const int* __restrict__ root_merge,
                          int nroots, int* __restrict__ orig, double* __restrict__ tau) {
  const int lane = threadIdx.x & 31;
  const int gr = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (gr >= nroots) return;
  const int m = root_merge[gr];
  const int o0 = off[m], kk = cnt[m];
  const int j = gr - o0;  // roots of merge m sit at the same offsets as its poles
  const double* d = dn + o0;
  const double* z = zn + o0;
  const double r = rho[m];
  auto f_at = [&](int o, double t) {
    double s = 0.0;
    for (int i = lane; i < kk; i += 32) s += z[i] * z[i] / ((d[i] - d[o]) - t);
    return 1.0 + r * warp_sum(s);
  };
  int o;
  double lo, hi;
  if (j < kk - 1) {
    const double half = 0.5 * (d[j + 1] - d[j]);
    if (f_at(j, half) >= 0.0) {
      o = j;
      lo = 0.0;
      hi = half;
    } else {
      o = j + 1;
      lo = -half;
      hi = 0.0;
    }
  } else {
    double s = 0.0;
    for (int i = lane; i < kk; i += 32) s += z[i] * z[i];
    o = j;
    lo = 0.0;
    hi = r * warp_sum(s) * (1.0 + 8.0 * kEps);
  }
  // safeguarded Newton on f (increasing in tau): the bracket [lo, hi] shrinks
  // with the sign of f at every iterate; a Newton step that leaves it is
  // replaced by bisection.  Ends when the step or the bracket is at the
  // rounding level of tau (at most 200 evaluations).
  double t = 0.5 * (lo + hi);
  for (int it = 0; it < 200; ++it) {
    double s = 0.0, ds = 0.0;
    for (int i = lane; i < kk; i += 32) {
      const double q = 1.0 / ((d[i] - d[o]) - t);
      const double zq = z[i] * q;
      s += z[i] * zq;
      ds += zq * zq;
    }
    s = warp_sum(s);
    ds = warp_sum(ds);
    const double f = 1.0 + r * s;
    if (f == 0.0) break;
    if (f < 0.0) lo = t;
    else hi = t;
    if (!(hi - lo > 2.0 * kEps * fmax(fabs(lo), fabs(hi)))) break;
    double tn = t - f / (r * ds);
    if (!(tn > lo && tn < hi)) tn = 0.5 * (lo + hi);
    if (fabs(tn - t) <= 2.0 * kEps * fabs(t)) {
      t = tn;
      break;
    }
    t = tn;
  }
  if (lane == 0) {
    orig[gr] = o;
    tau[gr] = t;
  }
}

// z recomputed from the roots (Loewner): one warp per pole i,
// zhat_i^2 = (lambda_{kk-1} - d_i) / rho * prod_{j < kk-1} (lambda_j - d_i) /
// (d_{j < i ? j : j+1} - d_i), lambda_j - d_i = (d_{o_j} - d_i) + tau_j
__global__ void k_loewner(const double* __restrict__ dn, const double* __restrict__ zn,
                          const int* __restrict__ off, const int* __restrict__ cnt,
                          const double* __restrict__ rho, const int* __restrict__ root_merge,
                          int nroots, const int* __restrict__ orig,
                          const double* __restrict__ tau, double* __restrict__ zhat) {
  const int lane = threadIdx.x & 31;
  const int gi = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (gi >= nroots) return;
  const int m = root_merge[gi];
  const int o0 = off[m], kk = cnt[m];
  const int i = gi - o0;
  const double* d = dn + o0;
  const int* og = orig + o0;
  const double* tg = tau + o0;
  double pr = 1.0;
  for (int j = lane; j < kk - 1; j += 32) {
    const double num = (d[og[j]] - d[i]) + tg[j];
    const double den = d[j < i ? j : j + 1] - d[i];
    pr *= num / den;
  }
  pr = warp_prod(pr);
  if (lane == 0) {
    const double last = (d[og[kk - 1]] - d[i]) + tg[kk - 1];
    const double v = fabs(pr * last / rho[m]);
    zhat[gi] = copysign(sqrt(v), zn[gi]);
  }
}

// secular eigenvectors, column-major per merge: S[i + j kk] = zhat_i /
// ((d_i - d_{o_j}) - tau_j), then each column normalised (one warp per column)
__global__ void k_secular_vectors(const double* __restrict__ dn, const int* __restrict__ off,
                                  const int* __restrict__ cnt, const int* __restrict__ soff,
                                  const int* __restrict__ root_merge, int nroots,
                                  const int* __restrict__ orig, const double* __restrict__ tau,
                                  const double* __restrict__ zhat, double* __restrict__ S) {
  const int lane = threadIdx.x & 31;
  const int gj = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (gj >= nroots) return;
  const int m = root_merge[gj];
  const int o0 = off[m], kk = cnt[m];
  const int j = gj - o0;
  const double* d = dn + o0;
  const double* zh = zhat + o0;
  const double dj = d[orig[gj]], tj = tau[gj];
  double* col = S + soff[m] + (size_t)j * kk;
  double ss = 0.0;
  for (int i = lane; i < kk; i += 32) {
    const double v = zh[i] / ((d[i] - dj) - tj);
    col[i] = v;
    ss += v * v;
  }
  const double inv = 1.0 / sqrt(warp_sum(ss));
  for (int i = lane; i < kk; i += 32) col[i] *= inv;
}

// G (k x kk, column-major per merge at goff[m]) = columns colN of Q's block
__global__ void k_gather(const double* __restrict__ Q, int n, const int* __restrict__ mlo,
                         const int* __restrict__ mhi, const int* __restrict__ off,
                         const int* __restrict__ cnt, const int* __restrict__ goff,
                         const int* __restrict__ colN, int nmerge, double* __restrict__ G) {
  const int m = blockIdx.y;
  if (m >= nmerge) return;
  const int lo = mlo[m], k = mhi[m] - lo, kk = cnt[m];
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (long long)k * kk;
       t += (long long)gridDim.x * blockDim.x) {
    const int j = (int)(t / k), r = (int)(t - (long long)j * k);
    G[goff[m] + t] = Q[(size_t)colN[off[m] + j] * n + lo + r];
  }
}

// C (k x kk) = G (k x kk) S (kk x kk), column-major, per merge (tiled FP64)
__global__ void __launch_bounds__(256) k_merge_gemm(const double* __restrict__ G,
                                                    const double* __restrict__ S,
                                                    const int* __restrict__ mlo,
                                                    const int* __restrict__ mhi,
                                                    const int* __restrict__ cnt,
                                                    const int* __restrict__ goff,
                                                    const int* __restrict__ soff, int nmerge,
                                                    double* __restrict__ Cout) {
  const int m = blockIdx.z;
  if (m >= nmerge) return;
  const int k = mhi[m] - mlo[m], kk = cnt[m];
  const int r0 = blockIdx.x * 64, c0 = blockIdx.y * 64;
  if (r0 >= k || c0 >= kk) return;
  const double* g = G + goff[m];
  const double* s = S + soff[m];
  double* out = Cout + goff[m];
  __shared__ double As[16][64 + 1], Bs[16][64 + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;  // 16 x 16 threads, 4 x 4 each
  double acc[4][4] = {};
  for (int p0 = 0; p0 < kk; p0 += 16) {
    for (int t = threadIdx.x; t < 16 * 64; t += 256) {
      const int pp = t / 64, rr = t % 64;
      const int gr = r0 + rr, gp = p0 + pp;
      As[pp][rr] = (gr < k && gp < kk) ? g[(size_t)gp * k + gr] : 0.0;
      const int gc = c0 + rr;
      Bs[pp][rr] = (gc < kk && gp < kk) ? s[(size_t)gc * kk + gp] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int pp = 0; pp < 16; ++pp) {
      double a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = As[pp][ty + 16 * q];
        b[q] = Bs[pp][tx + 16 * q];
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int w = 0; w < 4; ++w) acc[q][w] += a[q] * b[w];
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int w = 0; w < 4; ++w) {
      const int gr = r0 + ty + 16 * q, gc = c0 + tx + 16 * w;
      if (gr < k && gc < kk) out[(size_t)gc * k + gr] = acc[q][w];
    }
}

// Q's block columns in their final order: destination column dst[t] of merge
// m takes, for t < kk, column t of C (the merged vectors), else the deflated
// column colD[t - kk] of Q (copied first into X, a k-column scratch)
__global__ void k_scatter(double* __restrict__ Q, int n, const int* __restrict__ mlo,
                          const int* __restrict__ mhi, const int* __restrict__ cnt,
                          const int* __restrict__ goff, const int* __restrict__ dst_off,
                          const int* __restrict__ dst, const double* __restrict__ C,
                          const double* __restrict__ X, int nmerge) {
  const int m = blockIdx.y;
  if (m >= nmerge) return;
  const int lo = mlo[m], k = mhi[m] - lo, kk = cnt[m];
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (long long)k * k;
       t += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(t / k), r = (int)(t - (long long)c * k);
    const double v = (c < kk) ? C[goff[m] + (size_t)c * k + r] : X[(size_t)(lo + c) * n + lo + r];
    Q[(size_t)(lo + dst[dst_off[m] + c]) * n + lo + r] = v;
  }
}

// X's block columns [lo + kk, hi) = the deflated columns of Q (before the scatter)
__global__ void k_copy_deflated(const double* __restrict__ Q, int n,
                                const int* __restrict__ mlo, const int* __restrict__ mhi,
                                const int* __restrict__ cnt, const int* __restrict__ dcol_off,
                                const int* __restrict__ dcol, int nmerge,
                                double* __restrict__ X) {
  const int m = blockIdx.y;
  if (m >= nmerge) return;
  const int lo = mlo[m], k = mhi[m] - lo, kk = cnt[m], nd = k - kk;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (long long)nd * k;
       t += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(t / k), r = (int)(t - (long long)q * k);
    X[(size_t)(lo + kk + q) * n + lo + r] = Q[(size_t)(lo + dcol[dcol_off[m] + q]) * n + lo + r];
  }
}

unsigned gblocks(long long work, int per = kT) {
  long long b = (work + per - 1) / per;
  return (unsigned)std::max<long long>(1, std::min<long long>(b, 4096));
}

#define EK(...)                                          \
  do {                                                    \
    cudaError_t _e = (__VA_ARGS__);                       \
    if (_e != cudaSuccess) return _e;                     \
  } while (0)

// Page-locked host memory for the merges' small transfers, so that each copy
// is one asynchronous DMA instead of a staged pageable copy.  One buffer per
// host thread, grown on demand: an upload region (filled sequentially and
// rewound only after the stream has been synchronised, so that no queued copy
// reads a rewritten byte) and a download region.
struct Pinned {
  char* p = nullptr;
  size_t bytes = 0;
  ~Pinned() {
    if (p) cudaFreeHost(p);
  }
  cudaError_t ensure(size_t want) {
    if (want <= bytes) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMallocHost((void**)&p, want);
    if (e == cudaSuccess) bytes = want;
    return e;
  }
};
thread_local Pinned g_pinned;

struct Stager {
  char* base = nullptr;
  size_t cap = 0, used = 0;
  void rewind() { used = 0; }
  template <typename T>
  cudaError_t put(T* dev, const std::vector<T>& h, cudaStream_t s) {
    if (h.empty()) return cudaSuccess;
    const size_t b = sizeof(T) * h.size();
    used = (used + 15) & ~(size_t)15;
    if (used + b > cap) return cudaErrorMemoryAllocation;
    std::memcpy(base + used, h.data(), b);
    cudaError_t e = cudaMemcpyAsync(dev, base + used, b, cudaMemcpyHostToDevice, s);
    used += b;
    return e;
  }
};

}  // namespace

size_t work_doubles(long long n) {
  // Vh, Q, X, G, S, C (n^2 each); vectors; the integer arena (as doubles)
  return (size_t)6 * n * n + (size_t)24 * n + 4096 + (size_t)16 * n + 64;
}

cudaError_t solve(double* A, int n, double* w, double* work, cudaStream_t s, int* bad,
                  double* stage_ms) {
  *bad = 0;
  if (n < 1) return cudaSuccess;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  if (stage_ms)
    for (auto& x : ev) EK(cudaEventCreate(&x));
  auto mark = [&](int i) -> cudaError_t {
    return stage_ms ? cudaEventRecord(ev[i], s) : cudaSuccess;
  };
  EK(mark(0));
  const size_t nn = (size_t)n * n;
  double* Vh = work;
  double* Q = Vh + nn;
  double* X = Q + nn;
  double* G = X + nn;
  double* S = G + nn;
  double* C = S + nn;
  double* d = C + nn;
  double* e = d + n;
  double* tau = e + n;
  double* p = tau + n;        // 2 x n (by step parity)
  double* lam = p + 2 * (size_t)n;
  double* z = lam + n;
  double* dn = z + n;
  double* zn = dn + n;
  double* rho = zn + n;       // per merge (<= n)
  double* sgn = rho + n;      // per merge
  double* tauv = sgn + n;     // per root
  double* zhat = tauv + n;
  double* rot_cs = zhat + n;  // 2 per rotation (<= n rotations)
  double* part = rot_cs + 2 * (size_t)n;  // 2 x grid
  int* ib = reinterpret_cast<int*>(part + 4096);
  int* status = ib;
  int* mlo = ib + 16;
  int* mmid = mlo + n;
  int* mhi = mmid + n;
  int* off = mhi + n;
  int* cnt = off + n + 1;
  int* goff = cnt + n;
  int* soff = goff + n;
  int* root_merge = soff + n;
  int* orig = root_merge + n;
  int* colN = orig + n;
  int* dcol_off = colN + n;
  int* dcol = dcol_off + n + 1;
  int* dst_off = dcol + n;
  int* dst = dst_off + n + 1;
  int* rot_off = dst + n;
  int* rot_idx = rot_off + n + 1;  // 2 per rotation
  int* leaf_lo = rot_idx + 2 * n;
  EK(cudaMemsetAsync(status, 0, sizeof(int), s));
  // pinned host memory: uploads (at most ~40 n values between two
  // synchronisations) then downloads (d, e, lam, z, tau: doubles; orig: ints)
  const size_t up_bytes = (size_t)64 * 8 * (n + 64), down_doubles = (size_t)6 * n + 64;
  EK(g_pinned.ensure(up_bytes + sizeof(double) * down_doubles));
  Stager st;
  st.base = g_pinned.p;
  st.cap = up_bytes;
  double* h_down = reinterpret_cast<double*>(g_pinned.p + up_bytes);
  double* hd_p = h_down;            // n
  double* he_p = hd_p + n;          // n
  double* hz_p = he_p + n;          // n
  double* htau_p = hz_p + n;        // n
  int* horig_p = reinterpret_cast<int*>(htau_p + n);  // n ints
  double* hlam_p = htau_p + 2 * n;  // n

  // ---- 1. tridiagonalisation
  if (n >= 3) {
    int dev = 0, nsm = 0, per_sm = 0;
    EK(cudaGetDevice(&dev));
    EK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const size_t smem = sizeof(double) * (2 * (size_t)n + kT / 32);
    // the limit is the device's opt-in maximum, the same value from every
    // host thread (calls for different n may run at once)
    int optin = 0;
    cudaFuncAttributes fa;
    EK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    EK(cudaFuncGetAttributes(&fa, k_sytrd));
    const int dyn_max = optin - (int)fa.sharedSizeBytes;  // static shared memory counts too
    if (smem > (size_t)dyn_max) return cudaErrorInvalidValue;
    EK(cudaFuncSetAttribute(k_sytrd, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_max));
    EK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sytrd, kT, smem));
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    // one block per SM (the rows of a step spread over every SM's FP64
    // pipe), fewer when there are fewer rows than warps
    int grid = std::max(1, std::min(n / 2, nsm * per_sm));
    grid = std::min(grid, nsm);
    void* args[] = {&A, &n, &d, &e, &tau, &Vh, &p, &part};
    EK(cudaLaunchCooperativeKernel((void*)k_sytrd, dim3(grid), dim3(kT), args, smem, s));
  }
  EK(mark(1));
  std::vector<double> hd(n), he(n > 1 ? n - 1 : 1, 0.0);
  if (n >= 3) {
    EK(cudaMemcpyAsync(hd_p, d, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    EK(cudaMemcpyAsync(he_p, e, sizeof(double) * (n - 1), cudaMemcpyDeviceToHost, s));
    EK(cudaStreamSynchronize(s));
    std::memcpy(hd.data(), hd_p, sizeof(double) * n);
    std::memcpy(he.data(), he_p, sizeof(double) * (n - 1));
  } else {
    std::vector<double> ha(nn);
    EK(cudaMemcpyAsync(ha.data(), A, sizeof(double) * nn, cudaMemcpyDeviceToHost, s));
    EK(cudaStreamSynchronize(s));
    for (int i = 0; i < n; ++i) hd[i] = ha[(size_t)i * n + i];
    if (n == 2) he[0] = ha[1];
  }

  // ---- 2. divide and conquer on (hd, he)
  // tree: level L has 2^L nodes [ (c n) >> L, ((c + 1) n) >> L ); leaves at
  // the first L with every node <= kLeaf rows
  int L = 0;
  while ((n + (1 << L) - 1) >> L > kLeaf) ++L;
  std::vector<double> dmod = hd;
  // rank-one splits: d[mid-1] -= |beta|, d[mid] -= |beta|, beta = e[mid-1]
  for (int lev = 0; lev < L; ++lev)
    for (int c = 0; c < (1 << lev); ++c) {
      const long long lo = ((long long)c * n) >> lev, hi = ((long long)(c + 1) * n) >> lev;
      const long long mid = ((long long)(2 * c + 1) * n) >> (lev + 1);
      if (mid <= lo || mid >= hi) continue;
      const double b = he[mid - 1];
      dmod[mid - 1] -= std::fabs(b);
      dmod[mid] -= std::fabs(b);
    }
  {
    const int nleaf = 1 << L;
    std::vector<int> llo(nleaf + 1);
    for (int c = 0; c <= nleaf; ++c) llo[c] = (int)(((long long)c * n) >> L);
    EK(st.put(leaf_lo, llo, s));
    EK(st.put(dn, dmod, s));
    EK(st.put(zn, he, s));
    EK(cudaMemsetAsync(Q, 0, sizeof(double) * nn, s));
    k_leaf_ql<<<nleaf, 32, 0, s>>>(dn, zn, leaf_lo, nleaf, n, lam, Q, status);
    EK(cudaGetLastError());
  }
  std::vector<double> hlam(n);
  EK(cudaMemcpyAsync(hlam_p, lam, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  EK(cudaStreamSynchronize(s));
  st.rewind();
  std::memcpy(hlam.data(), hlam_p, sizeof(double) * n);
  for (int lev = L - 1; lev >= 0; --lev) {
    const int nm = 1 << lev;
    std::vector<int> hlo, hmid, hhi;
    std::vector<double> hs, hr;
    for (int c = 0; c < nm; ++c) {
      const int lo = (int)(((long long)c * n) >> lev), hi = (int)(((long long)(c + 1) * n) >> lev);
      const int mid = (int)(((long long)(2 * c + 1) * n) >> (lev + 1));
      if (mid <= lo || mid >= hi) continue;
      hlo.push_back(lo);
      hmid.push_back(mid);
      hhi.push_back(hi);
      const double b = he[mid - 1];
      hs.push_back(b < 0.0 ? -1.0 : 1.0);
      hr.push_back(2.0 * std::fabs(b));
    }
    const int nmerge = (int)hlo.size();
    if (nmerge == 0) continue;
    EK(st.put(mlo, hlo, s));
    EK(st.put(mmid, hmid, s));
    EK(st.put(mhi, hhi, s));
    EK(st.put(sgn, hs, s));
    int maxk = 0;
    for (int q = 0; q < nmerge; ++q) maxk = std::max(maxk, hhi[q] - hlo[q]);
    k_merge_z<<<dim3(gblocks(maxk), nmerge), kT, 0, s>>>(Q, n, mlo, mmid, mhi, sgn, nmerge, z);
    EK(cudaGetLastError());
    EK(cudaMemcpyAsync(hz_p, z, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    EK(cudaStreamSynchronize(s));
    st.rewind();
    const double* hz = hz_p;
    // deflation on the host, per merge
    std::vector<int> hoff(nmerge + 1, 0), hcnt(nmerge), hcolN, hdcoff(nmerge + 1, 0), hdcol,
        hroff(nmerge + 1, 0), hridx, hgoff(nmerge), hsoff(nmerge), hroot_merge;
    std::vector<double> hdn, hzn, hrcs, hdval;  // hdval: deflated values, in hdcol order
    long long gpos = 0, spos = 0;
    for (int q = 0; q < nmerge; ++q) {
      const int lo = hlo[q], hi = hhi[q], k = hi - lo;
      const double r = hr[q];
      std::vector<int> ord(k);
      std::iota(ord.begin(), ord.end(), 0);
      std::stable_sort(ord.begin(), ord.end(),
                       [&](int a, int b) { return hlam[lo + a] < hlam[lo + b]; });
      double dmax = 0.0, zmax = 0.0;
      for (int t = 0; t < k; ++t) {
        dmax = std::max(dmax, std::fabs(hlam[lo + t]));
        zmax = std::max(zmax, std::fabs(hz[lo + t]));
      }
      const double tol = 8.0 * kEps * std::max(dmax, r * zmax);
      int pend = -1;  // block-local column of the pending entry
      double pd = 0.0, pz = 0.0;
      for (int t = 0; t < k; ++t) {
        const int col = ord[t];
        const double dv = hlam[lo + col], zv = hz[lo + col];
        if (r * std::fabs(zv) <= tol) {  // negligible coupling: an eigenpair of D
          hdcol.push_back(col);
          hdval.push_back(dv);
          continue;
        }
        if (pend < 0) {
          pend = col;
          pd = dv;
          pz = zv;
          continue;
        }
        const double rr = std::hypot(pz, zv);
        const double c = zv / rr, sn = -pz / rr;
        const double tdiff = dv - pd;
        if (std::fabs(tdiff * c * sn) <= tol) {
          // rotate (pend, col): the pending direction deflates
          hridx.push_back(pend + lo);
          hridx.push_back(col + lo);
          hrcs.push_back(c);
          hrcs.push_back(sn);
          hdcol.push_back(pend);
          hdval.push_back(c * c * pd + sn * sn * dv);
          pd = sn * sn * pd + c * c * dv;
          pz = rr;
          pend = col;
          continue;
        }
        hcolN.push_back(lo + pend);
        hdn.push_back(pd);
        hzn.push_back(pz);
        pend = col;
        pd = dv;
        pz = zv;
      }
      if (pend >= 0) {
        hcolN.push_back(lo + pend);
        hdn.push_back(pd);
        hzn.push_back(pz);
      }
      hoff[q + 1] = (int)hdn.size();
      hcnt[q] = hoff[q + 1] - hoff[q];
      hdcoff[q + 1] = (int)hdcol.size();
      hroff[q + 1] = (int)(hrcs.size() / 2);
      hgoff[q] = (int)gpos;
      hsoff[q] = (int)spos;
      gpos += (long long)k * hcnt[q];
      spos += (long long)hcnt[q] * hcnt[q];
      for (int t = 0; t < hcnt[q]; ++t) hroot_merge.push_back(q);
    }
    const int nroots = (int)hdn.size();
    EK(st.put(off, hoff, s));
    EK(st.put(cnt, hcnt, s));
    EK(st.put(colN, hcolN, s));
    EK(st.put(dcol_off, hdcoff, s));
    EK(st.put(dcol, hdcol, s));
    EK(st.put(rot_off, hroff, s));
    EK(st.put(rot_idx, hridx, s));
    EK(st.put(rot_cs, hrcs, s));
    EK(st.put(goff, hgoff, s));
    EK(st.put(soff, hsoff, s));
    EK(st.put(root_merge, hroot_merge, s));
    EK(st.put(dn, hdn, s));
    EK(st.put(zn, hzn, s));
    EK(st.put(rho, hr, s));
    int maxkk = 0;
    for (int q = 0; q < nmerge; ++q) maxkk = std::max(maxkk, hcnt[q]);
    if (!hridx.empty()) {
      k_rotate<<<dim3(gblocks(maxk), nmerge), kT, 0, s>>>(Q, n, mlo, mhi, rot_off, rot_idx,
                                                          rot_cs, nmerge);
      EK(cudaGetLastError());
    }
    if (nroots > 0) {
      const unsigned wb = (unsigned)((nroots + 7) / 8);
      k_secular<<<wb, 256, 0, s>>>(dn, zn, off, cnt, rho, root_merge, nroots, orig, tauv);
      EK(cudaGetLastError());
      k_loewner<<<wb, 256, 0, s>>>(dn, zn, off, cnt, rho, root_merge, nroots, orig, tauv, zhat);
      EK(cudaGetLastError());
      k_secular_vectors<<<wb, 256, 0, s>>>(dn, off, cnt, soff, root_merge, nroots, orig, tauv,
                                           zhat, S);
      EK(cudaGetLastError());
      k_gather<<<dim3(gblocks((long long)maxk * maxkk), nmerge), kT, 0, s>>>(
          Q, n, mlo, mhi, off, cnt, goff, colN, nmerge, G);
      EK(cudaGetLastError());
      k_merge_gemm<<<dim3((maxk + 63) / 64, (maxkk + 63) / 64, nmerge), 256, 0, s>>>(
          G, S, mlo, mhi, cnt, goff, soff, nmerge, C);
      EK(cudaGetLastError());
    }
    // the merged eigenvalues: roots (lambda_j = dn_{o_j} + tau_j) and the
    // deflated values, sorted per merge; the new column order
    const int* horig = horig_p;
    const double* htau = htau_p;
    if (nroots > 0) {
      EK(cudaMemcpyAsync(horig_p, orig, sizeof(int) * nroots, cudaMemcpyDeviceToHost, s));
      EK(cudaMemcpyAsync(htau_p, tauv, sizeof(double) * nroots, cudaMemcpyDeviceToHost, s));
      EK(cudaStreamSynchronize(s));
      st.rewind();
    }
    std::vector<int> hdst, hdstoff(nmerge + 1, 0);
    for (int q = 0; q < nmerge; ++q) {
      const int lo = hlo[q], k = hhi[q] - lo, kk = hcnt[q];
      std::vector<double> val(k);
      for (int t = 0; t < kk; ++t) {
        const int g = hoff[q] + t;
        val[t] = hdn[hoff[q] + horig[g]] + htau[g];
      }
      for (int t = 0; t < k - kk; ++t) val[kk + t] = hdval[hdcoff[q] + t];
      std::vector<int> ord(k);
      std::iota(ord.begin(), ord.end(), 0);
      std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return val[a] < val[b]; });
      std::vector<int> pos(k);
      for (int t = 0; t < k; ++t) pos[ord[t]] = t;
      for (int t = 0; t < k; ++t) {
        hdst.push_back(pos[t]);
        hlam[lo + pos[t]] = val[t];
      }
      hdstoff[q + 1] = (int)hdst.size();
    }
    EK(st.put(dst_off, hdstoff, s));
    EK(st.put(dst, hdst, s));
    k_copy_deflated<<<dim3(gblocks((long long)maxk * maxk), nmerge), kT, 0, s>>>(
        Q, n, mlo, mhi, cnt, dcol_off, dcol, nmerge, X);
    EK(cudaGetLastError());
    k_scatter<<<dim3(gblocks((long long)maxk * maxk), nmerge), kT, 0, s>>>(
        Q, n, mlo, mhi, cnt, goff, dst_off, dst, C, X, nmerge);
    EK(cudaGetLastError());
  }
  EK(st.put(w, hlam, s));

  // ---- 3. back-transformation into A
  EK(mark(2));
  EK(cudaMemcpyAsync(A, Q, sizeof(double) * nn, cudaMemcpyDeviceToDevice, s));
  if (n >= 3) {
    k_ormtr<<<(unsigned)((n + kT / 32 - 1) / (kT / 32)), kT, 0, s>>>(A, n, Vh, tau);
    EK(cudaGetLastError());
  }
  EK(mark(3));
  int hb = 0;
  EK(cudaMemcpyAsync(&hb, status, sizeof(int), cudaMemcpyDeviceToHost, s));
  EK(cudaStreamSynchronize(s));
  *bad = hb;
  if (stage_ms) {
    for (int i = 0; i < 3; ++i) {
      float t = 0.f;
      EK(cudaEventElapsedTime(&t, ev[i], ev[i + 1]));
      stage_ms[i] = t;
    }
    for (auto& x : ev) cudaEventDestroy(x);
  }
  return cudaSuccess;
}

}  // namespace eigh
}  // namespace sep
