// sep_kernels.cu -- Newton accumulation, packing, reductions and FP64
// contractions (see sep_kernels.cuh).
#include "sep_kernels.cuh"

#include <type_traits>

namespace sep {

namespace {

constexpr int kThreads = 256;

inline unsigned blocks_for(long long work, int per_block, long long cap = 152LL * 32) {
  long long b = (work + per_block - 1) / per_block;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (unsigned)b;
}

// -------------------------------------------------------------------------
template <typename T, typename TR>
__global__ void k_pack(const TR* __restrict__ real, long long nstates, long long n,
                       cx<T>* __restrict__ out) {
  const long long B = (nstates + 1) / 2;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < B * n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long b = i / n, g = i - b * n;
    const T re = (T)real[(2 * b) * n + g];
    const T im = (2 * b + 1 < nstates) ? (T)real[(2 * b + 1) * n + g] : T(0);
    out[i] = mk<T>(re, im);
  }
}

template <typename T, typename TR>
__global__ void k_unpack(const cx<T>* __restrict__ in, long long nstates, long long n,
                         TR* __restrict__ real) {
  const long long B = (nstates + 1) / 2;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < B * n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long b = i / n, g = i - b * n;
    const cx<T> v = in[i];
    real[(2 * b) * n + g] = (TR)v.x;
    if (2 * b + 1 < nstates) real[(2 * b + 1) * n + g] = (TR)v.y;
  }
}

// -------------------------------------------------------------------------
constexpr int kMaxBlockSteps = 128;  // history grids per accumulation pass
constexpr int kLoadBatch = 8;       // history loads in flight per thread (ms > 4)

template <typename T, typename TA, int MSMAX>
__global__ void __launch_bounds__(kThreads)
k_accumulate(const cx<T>* __restrict__ hist, int slots, int B, long long n, long long j0,
             int count, const TA* __restrict__ an, long long nc, int ms, TA* __restrict__ acc,
             long long nstates, int init) {
  // grid.y = pair b; grid-stride over the grid points of that pair; the slot
  // offsets and coefficients are resolved once per block
  __shared__ TA cf[MSMAX * kMaxBlockSteps];
  __shared__ long long soff[kMaxBlockSteps];
  for (int i = threadIdx.x; i < ms * count; i += blockDim.x) {
    const int e = i / count, s = i - e * count;
    cf[e * kMaxBlockSteps + s] = an[e * nc + j0 + s];
  }
  const long long b = blockIdx.y;
  for (int s = threadIdx.x; s < count; s += blockDim.x)
    soff[s] = (long long)((j0 + s) % slots) * ((long long)B * n) + b * n;
  __syncthreads();
  (void)nstates;  // the imaginary half of an odd last pair is zero and unread
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n;
       g += (long long)gridDim.x * blockDim.x) {
    TA re[MSMAX], im[MSMAX];
#pragma unroll
    for (int e = 0; e < MSMAX; ++e) { re[e] = TA(0); im[e] = TA(0); }
    // LB history loads are issued before their products, so each thread
    // keeps that many grid loads in flight
    constexpr int LB = MSMAX >= 8 ? kLoadBatch : kLoadBatch / 2;
    int s = 0;
    for (; s + LB <= count; s += LB) {
      cx<T> h[LB];
#pragma unroll
      for (int u = 0; u < LB; ++u) h[u] = hist[soff[s + u] + g];
#pragma unroll
      for (int u = 0; u < LB; ++u) {
#pragma unroll
        for (int e = 0; e < MSMAX; ++e) {
          if (e < ms) {
            const TA c = cf[e * kMaxBlockSteps + s + u];
            re[e] += c * (TA)h[u].x;
            im[e] += c * (TA)h[u].y;
          }
        }
      }
    }
    for (; s < count; ++s) {
      const cx<T> h = hist[soff[s] + g];
#pragma unroll
      for (int e = 0; e < MSMAX; ++e) {
        if (e < ms) {
          const TA c = cf[e * kMaxBlockSteps + s];
          re[e] += c * (TA)h.x;
          im[e] += c * (TA)h.y;
        }
      }
    }
    // the 2 ms accumulators of (pair b, point g) are adjacent: targets of
    // state 2b, then of state 2b + 1
    TA* __restrict__ pa = acc + (b * n + g) * (2 * ms);
    bool stored = false;
    if constexpr (std::is_same<TA, float>::value) {
    if (MSMAX <= 16 && ms == MSMAX) {
      float4* p4 = reinterpret_cast<float4*>(pa);
#pragma unroll
      for (int q = 0; q < MSMAX / 2; ++q) {
        TA v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int k = 4 * q + u;
          v[u] = k < MSMAX ? re[k] : im[k - MSMAX];
        }
        float4 o = make_float4((float)v[0], (float)v[1], (float)v[2], (float)v[3]);
        if (!init) {
          const float4 old = p4[q];
          o = make_float4(old.x + o.x, old.y + o.y, old.z + o.z, old.w + o.w);
        }
        p4[q] = o;
      }
    } else if (ms % 2 == 0) {
      float2* q0 = reinterpret_cast<float2*>(pa);
      float2* q1 = reinterpret_cast<float2*>(pa + ms);
#pragma unroll
      for (int e = 0; e < MSMAX; e += 2) {
        if (e < ms) {
          float2 r = make_float2((float)re[e], (float)re[e + 1]);
          float2 i = make_float2((float)im[e], (float)im[e + 1]);
          if (!init) {
            const float2 r0 = q0[e / 2], i0 = q1[e / 2];
            r = make_float2(r0.x + r.x, r0.y + r.y);
            i = make_float2(i0.x + i.x, i0.y + i.y);
          }
          q0[e / 2] = r;
          q1[e / 2] = i;
        }
      }
    }
    stored = (MSMAX <= 16 && ms == MSMAX) || ms % 2 == 0;
    }
    if (!stored) {
#pragma unroll
      for (int e = 0; e < MSMAX; ++e) {
        if (e < ms) {
          pa[e] = init ? re[e] : pa[e] + re[e];
          pa[ms + e] = init ? im[e] : pa[ms + e] + im[e];
        }
      }
    }
  }
}

// Complex64 history, FP32 accumulators and exactly MS targets (the common
// case): as k_accumulate, with two adjacent grid points per thread (16-byte
// history loads) and the coefficients of four steps per 16-byte shared load,
// so that the shared-memory pipe issues a quarter of the loads per multiply-
// add.  Each point's sums take the same products in the same order as in
// k_accumulate, so the results are equal bit for bit.  n is even.
template <int MS>
__global__ void __launch_bounds__(kThreads)
k_accumulate_x2(const float4* __restrict__ hist, int slots, int B, long long n2, long long j0,
                int count, const float* __restrict__ an, long long nc,
                float* __restrict__ acc, int init) {
  __shared__ __align__(16) float cf[MS * kMaxBlockSteps];
  __shared__ long long soff[kMaxBlockSteps];  // in float4 (point pairs)
  for (int i = threadIdx.x; i < MS * count; i += blockDim.x) {
    const int e = i / count, s = i - e * count;
    cf[e * kMaxBlockSteps + s] = an[e * nc + j0 + s];
  }
  const long long b = blockIdx.y;
  for (int s = threadIdx.x; s < count; s += blockDim.x)
    soff[s] = (long long)((j0 + s) % slots) * ((long long)B * n2) + b * n2;
  __syncthreads();
  for (long long g2 = blockIdx.x * (long long)blockDim.x + threadIdx.x; g2 < n2;
       g2 += (long long)gridDim.x * blockDim.x) {
    float re0[MS], im0[MS], re1[MS], im1[MS];
#pragma unroll
    for (int e = 0; e < MS; ++e) re0[e] = im0[e] = re1[e] = im1[e] = 0.f;
    constexpr int LB = kLoadBatch;
    int s = 0;
    for (; s + LB <= count; s += LB) {
      float4 h[LB];  // (x, y) of point 2 g2, then of point 2 g2 + 1
#pragma unroll
      for (int u = 0; u < LB; ++u) h[u] = hist[soff[s + u] + g2];
#pragma unroll
      for (int e = 0; e < MS; ++e) {
        float c[LB];
#pragma unroll
        for (int q = 0; q < LB / 4; ++q) {
          const float4 c4 = *reinterpret_cast<const float4*>(&cf[e * kMaxBlockSteps + s + 4 * q]);
          c[4 * q] = c4.x;
          c[4 * q + 1] = c4.y;
          c[4 * q + 2] = c4.z;
          c[4 * q + 3] = c4.w;
        }
#pragma unroll
        for (int u = 0; u < LB; ++u) {
          re0[e] += c[u] * h[u].x;
          im0[e] += c[u] * h[u].y;
          re1[e] += c[u] * h[u].z;
          im1[e] += c[u] * h[u].w;
        }
      }
    }
    for (; s < count; ++s) {
      const float4 h = hist[soff[s] + g2];
#pragma unroll
      for (int e = 0; e < MS; ++e) {
        const float c = cf[e * kMaxBlockSteps + s];
        re0[e] += c * h.x;
        im0[e] += c * h.y;
        re1[e] += c * h.z;
        im1[e] += c * h.w;
      }
    }
    // the 2 MS accumulators of (pair b, point g): targets of state 2b, then
    // of state 2b + 1; points 2 g2 and 2 g2 + 1 are adjacent
    float4* p4 = reinterpret_cast<float4*>(acc + (b * 2 * n2 + 2 * g2) * (2 * MS));
#pragma unroll
    for (int pt = 0; pt < 2; ++pt) {
#pragma unroll
      for (int q = 0; q < MS / 2; ++q) {
        float v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int k = 4 * q + u;
          v[u] = pt == 0 ? (k < MS ? re0[k] : im0[k - MS]) : (k < MS ? re1[k] : im1[k - MS]);
        }
        float4 o = make_float4(v[0], v[1], v[2], v[3]);
        float4* dst = p4 + pt * (MS / 2) + q;
        if (!init) {
          const float4 old = *dst;
          o = make_float4(old.x + o.x, old.y + o.y, old.z + o.z, old.w + o.w);
        }
        *dst = o;
      }
    }
  }
}

// accumulators [B][n][2 ms] -> out[(2b + c) ms + e][g] (state-major, double)
template <typename TA>
__global__ void k_unpack_acc(const TA* __restrict__ acc, long long B, long long n, int ms,
                             long long nstates, double* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < B * n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long b = i / n, g = i - b * n;
    const TA* pa = acc + i * (2 * ms);
    for (int c = 0; c < 2; ++c) {
      const long long st = 2 * b + c;
      if (st >= nstates) break;
      for (int e = 0; e < ms; ++e) out[(st * ms + e) * n + g] = (double)pa[c * ms + e];
    }
  }
}

// -------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* out) {
  __shared__ double red[NV][kThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double t = warp_sum(v[k]);
    if (lane == 0) red[k][w] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double t = 0.0;
      for (int i = 0; i < kThreads / 32; ++i) t += red[k][i];
      out[k] = t;
    }
  }
}

constexpr int kPartials = 128;  // blocks per row in the first reduction level

template <typename T>
__global__ void __launch_bounds__(kThreads)
k_pair_dots1(const cx<T>* __restrict__ x, const cx<T>* __restrict__ y, long long n,
             double* __restrict__ partial) {
  const long long b = blockIdx.y;
  const cx<T>* xb = x + b * n;
  const cx<T>* yb = y + b * n;
  double v[2] = {0.0, 0.0};
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n;
       g += (long long)gridDim.x * blockDim.x) {
    const cx<T> p = xb[g], q = yb[g];
    v[0] += (double)p.x * (double)q.x;
    v[1] += (double)p.y * (double)q.y;
  }
  double o[2];
  block_sum<2>(v, o);
  if (threadIdx.x == 0) {
    partial[(b * gridDim.x + blockIdx.x) * 2 + 0] = o[0];
    partial[(b * gridDim.x + blockIdx.x) * 2 + 1] = o[1];
  }
}

__global__ void k_pair_dots2(const double* __restrict__ partial, int nblk, double w,
                             double2* __restrict__ out) {
  const int b = blockIdx.x;
  if (threadIdx.x == 0) {
    double a = 0.0, c = 0.0;
    for (int i = 0; i < nblk; ++i) {
      a += partial[(b * nblk + i) * 2 + 0];
      c += partial[(b * nblk + i) * 2 + 1];
    }
    out[b] = make_double2(a * w, c * w);
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
k_row_dots1(const T* __restrict__ x, const T* __restrict__ y, long long n,
            double* __restrict__ partial) {
  const long long m = blockIdx.y;
  const T* xm = x + m * n;
  const T* ym = y + m * n;
  double v[1] = {0.0};
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n;
       g += (long long)gridDim.x * blockDim.x)
    v[0] += (double)xm[g] * (double)ym[g];
  double o[1];
  block_sum<1>(v, o);
  if (threadIdx.x == 0) partial[m * gridDim.x + blockIdx.x] = o[0];
}

__global__ void k_row_dots2(const double* __restrict__ partial, int nblk, double w,
                            double* __restrict__ out) {
  const long long m = blockIdx.x;
  if (threadIdx.x == 0) {
    double a = 0.0;
    for (int i = 0; i < nblk; ++i) a += partial[m * nblk + i];
    out[m] = a * w;
  }
}

template <typename T>
__global__ void k_scale_rows(T* __restrict__ x, long long n, const double* __restrict__ norms,
                             double dv) {
  const long long m = blockIdx.y;
  const double s = norms[m];
  const double f = (s != 0.0) ? 1.0 / sqrt(s * dv) : 0.0;
  T* xm = x + m * n;
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n;
       g += (long long)gridDim.x * blockDim.x)
    xm[g] = (T)((double)xm[g] * f);
}

__global__ void __launch_bounds__(kThreads)
k_resid1(const double* __restrict__ x, const double* __restrict__ hx,
         const double* __restrict__ e, long long n, double* __restrict__ partial) {
  const long long m = blockIdx.y;
  const double em = e[m];
  double v[1] = {0.0};
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n;
       g += (long long)gridDim.x * blockDim.x) {
    const double r = hx[m * n + g] - em * x[m * n + g];
    v[0] += r * r;
  }
  double o[1];
  block_sum<1>(v, o);
  if (threadIdx.x == 0) partial[m * gridDim.x + blockIdx.x] = o[0];
}

__global__ void k_sqrt_scaled(double* __restrict__ v, long long m, double w) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < m) v[i] = sqrt(v[i] * w);
}

// -------------------------------------------------------------------------
// FP64 tiled contractions: 64 x 64 tile, 16-deep k slices, 256 threads each
// owning a 4 x 4 block of outputs.
constexpr int TM = 64, TN = 64, TK = 16;

__global__ void __launch_bounds__(256)
k_gemm_nt(const double* __restrict__ A, const double* __restrict__ B, long long M,
          long long Nn, long long K, long long kchunk, double* __restrict__ part, bool sym) {
  const long long m0 = (long long)blockIdx.y * TM, n0 = (long long)blockIdx.x * TN;
  if (sym && n0 + TN <= m0) return;  // strictly below the diagonal
  const long long k_begin = (long long)blockIdx.z * kchunk;
  long long k_end = k_begin + kchunk;
  if (k_end > K) k_end = K;
  __shared__ double As[TK][TM + 1];
  __shared__ double Bs[TK][TN + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double c[4][4] = {};
  for (long long k0 = k_begin; k0 < k_end; k0 += TK) {
    // load 64 x 16 of A and B: each thread 4 elements of each
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int li = threadIdx.x + r * 256;  // 0..1023
      const int row = li >> 4, kk = li & 15;
      const long long gk = k0 + kk;
      const long long ga = m0 + row, gb = n0 + row;
      As[kk][row] = (ga < M && gk < k_end) ? A[ga * K + gk] : 0.0;
      Bs[kk][row] = (gb < Nn && gk < k_end) ? B[gb * K + gk] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) c[i][j] = fma(a[i], b[j], c[i][j]);
    }
    __syncthreads();
  }
  double* P = part + (long long)blockIdx.z * M * Nn;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const long long gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const long long gn = n0 + tx * 4 + j;
      if (gn < Nn) P[gm * Nn + gn] = c[i][j];
    }
  }
}

__global__ void k_gemm_nt_reduce(const double* __restrict__ part, int splits, long long M,
                                 long long Nn, double alpha, double* __restrict__ C, bool sym) {
  const long long total = M * Nn;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long m = i / Nn, nn = i - m * Nn;
    long long src = i;
    if (sym) {
      // tiles strictly below the diagonal were skipped: read the mirror
      const long long tm = m / TM, tn = nn / TN;
      if (tn < tm) src = nn * Nn + m;
    }
    double s = 0.0;
    for (int k = 0; k < splits; ++k) s += part[(long long)k * total + src];
    C[i] = alpha * s;
  }
}

__global__ void __launch_bounds__(256)
k_gemm_nn(const double* __restrict__ A, const double* __restrict__ B, long long M,
          long long Nn, long long K, long long ldb, long long ldc, double* __restrict__ C) {
  const long long m0 = (long long)blockIdx.y * TM, n0 = (long long)blockIdx.x * TN;
  __shared__ double As[TK][TM + 1];
  __shared__ double Bs[TK][TN];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double c[4][4] = {};
  for (long long k0 = 0; k0 < K; k0 += TK) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int li = threadIdx.x + r * 256;
      {  // A tile: 64 rows x 16 k
        const int row = li >> 4, kk = li & 15;
        const long long gm = m0 + row, gk = k0 + kk;
        As[kk][row] = (gm < M && gk < K) ? A[gm * K + gk] : 0.0;
      }
      {  // B tile: 16 k x 64 columns (columns contiguous)
        const int kk = li >> 6, col = li & 63;
        const long long gk = k0 + kk, gn = n0 + col;
        Bs[kk][col] = (gk < K && gn < Nn) ? B[gk * ldb + gn] : 0.0;
      }
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < TK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) c[i][j] = fma(a[i], b[j], c[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const long long gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const long long gn = n0 + tx + 16 * j;
      if (gn < Nn) C[gm * ldc + gn] = c[i][j];
    }
  }
}

__global__ void k_transpose(const double* __restrict__ in, long long rows, long long cols,
                            double* __restrict__ out) {
  __shared__ double t[32][33];
  const long long c0 = (long long)blockIdx.x * 32, r0 = (long long)blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const long long r = r0 + k, c = c0 + threadIdx.x;
    if (r < rows && c < cols) t[k][threadIdx.x] = in[r * cols + c];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const long long c = c0 + k, r = r0 + threadIdx.x;
    if (r < rows && c < cols) out[c * rows + r] = t[threadIdx.x][k];
  }
}

__global__ void k_scale_eigvecs(const double* __restrict__ V, const double* __restrict__ lam,
                                long long M, long long k0, double* __restrict__ out) {
  const long long kept = M - k0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < kept * M;
       i += (long long)gridDim.x * blockDim.x) {
    const long long r = i / M, j = i - r * M;
    const long long col = M - 1 - r;
    out[i] = V[col * M + j] / sqrt(lam[col]);
  }
}

template <typename A, typename B>
__global__ void k_convert(const A* __restrict__ in, B* __restrict__ out, long long count) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = (B)in[i];
}

}  // namespace

// =========================================================================
template <typename T, typename TR>
cudaError_t pack_pairs(const TR* real, long long nstates, long long n, cx<T>* out,
                       cudaStream_t s) {
  const long long B = (nstates + 1) / 2;
  k_pack<T, TR><<<blocks_for(B * n, kThreads), kThreads, 0, s>>>(real, nstates, n, out);
  return cudaGetLastError();
}
template <typename T, typename TR>
cudaError_t unpack_pairs(const cx<T>* in, long long nstates, long long n, TR* real,
                         cudaStream_t s) {
  const long long B = (nstates + 1) / 2;
  k_unpack<T, TR><<<blocks_for(B * n, kThreads), kThreads, 0, s>>>(in, nstates, n, real);
  return cudaGetLastError();
}
template cudaError_t pack_pairs<double, double>(const double*, long long, long long, cx<double>*,
                                                cudaStream_t);
template cudaError_t pack_pairs<float, double>(const double*, long long, long long, cx<float>*,
                                               cudaStream_t);
template cudaError_t pack_pairs<float, float>(const float*, long long, long long, cx<float>*,
                                              cudaStream_t);
template cudaError_t unpack_pairs<double, double>(const cx<double>*, long long, long long,
                                                  double*, cudaStream_t);
template cudaError_t unpack_pairs<float, double>(const cx<float>*, long long, long long, double*,
                                                 cudaStream_t);
template cudaError_t unpack_pairs<float, float>(const cx<float>*, long long, long long, float*,
                                                cudaStream_t);
template cudaError_t pack_pairs<ddf, double>(const double*, long long, long long, cx<ddf>*,
                                             cudaStream_t);
template cudaError_t unpack_pairs<ddf, double>(const cx<ddf>*, long long, long long, double*,
                                               cudaStream_t);

template <typename T, typename TA>
cudaError_t newton_accumulate(const cx<T>* hist, int slots, int B, long long n, long long j0,
                              int count, const TA* an, long long nc, int ms, TA* acc,
                              long long nstates, bool init, cudaStream_t s) {
  if (count < 1 || count > kMaxBlockSteps || ms < 1 || ms > 32 || B > 65535)
    return cudaErrorInvalidValue;
  // each thread sees about 4 grid points of one pair (enough blocks to keep
  // 64 warps per SM resident while the history loads are in flight)
  long long per = (n + 4LL * kThreads - 1) / (4LL * kThreads);
  if (per > 65535) per = 65535;
  if (per < 1) per = 1;
  const dim3 g((unsigned)per, (unsigned)B);
  if constexpr (std::is_same<T, float>::value && std::is_same<TA, float>::value) {
    if (n % 2 == 0 && ms == 8) {  // two points per thread
      k_accumulate_x2<8><<<g, kThreads, 0, s>>>(reinterpret_cast<const float4*>(hist), slots,
                                                 B, n / 2, j0, count, an, nc, acc, init);
      return cudaGetLastError();
    }
  }
  if (ms <= 4)
    k_accumulate<T, TA, 4><<<g, kThreads, 0, s>>>(hist, slots, B, n, j0, count, an, nc, ms, acc,
                                                  nstates, init);
  else if (ms <= 8)
    k_accumulate<T, TA, 8><<<g, kThreads, 0, s>>>(hist, slots, B, n, j0, count, an, nc, ms, acc,
                                                  nstates, init);
  else if (ms <= 16)
    k_accumulate<T, TA, 16><<<g, kThreads, 0, s>>>(hist, slots, B, n, j0, count, an, nc, ms,
                                                   acc, nstates, init);
  else
    k_accumulate<T, TA, 32><<<g, kThreads, 0, s>>>(hist, slots, B, n, j0, count, an, nc, ms,
                                                   acc, nstates, init);
  return cudaGetLastError();
}
template cudaError_t newton_accumulate<double, double>(const cx<double>*, int, int, long long,
                                                       long long, int, const double*, long long,
                                                       int, double*, long long, bool,
                                                       cudaStream_t);
template cudaError_t newton_accumulate<float, float>(const cx<float>*, int, int, long long,
                                                     long long, int, const float*, long long,
                                                     int, float*, long long, bool,
                                                     cudaStream_t);
template cudaError_t newton_accumulate<ddf, ddf>(const cx<ddf>*, int, int, long long, long long,
                                                 int, const ddf*, long long, int, ddf*,
                                                 long long, bool, cudaStream_t);

template <typename TA>
cudaError_t unpack_accumulators(const TA* acc, long long B, long long n, int ms,
                                long long nstates, double* out, cudaStream_t s) {
  k_unpack_acc<TA><<<blocks_for(B * n, kThreads, 152LL * 16), kThreads, 0, s>>>(acc, B, n, ms,
                                                                                 nstates, out);
  return cudaGetLastError();
}
template cudaError_t unpack_accumulators<float>(const float*, long long, long long, int,
                                                long long, double*, cudaStream_t);
template cudaError_t unpack_accumulators<double>(const double*, long long, long long, int,
                                                 long long, double*, cudaStream_t);
template cudaError_t unpack_accumulators<ddf>(const ddf*, long long, long long, int, long long,
                                              double*, cudaStream_t);

size_t reduce_partial_doubles(long long rows) { return (size_t)rows * kPartials * 2; }

template <typename T>
cudaError_t pair_dots(const cx<T>* x, const cx<T>* y, int B, long long n, double w,
                      double2* out_dev, double* partial, cudaStream_t s) {
  if (B > 65535) return cudaErrorInvalidValue;
  k_pair_dots1<T><<<dim3(kPartials, B), kThreads, 0, s>>>(x, y, n, partial);
  k_pair_dots2<<<B, 32, 0, s>>>(partial, kPartials, w, out_dev);
  return cudaGetLastError();
}
template cudaError_t pair_dots<double>(const cx<double>*, const cx<double>*, int, long long,
                                       double, double2*, double*, cudaStream_t);
template cudaError_t pair_dots<float>(const cx<float>*, const cx<float>*, int, long long, double,
                                      double2*, double*, cudaStream_t);

template <typename T>
cudaError_t row_dots(const T* x, const T* y, long long M, long long n, double w,
                     double* out_dev, double* partial, cudaStream_t s) {
  if (M > 65535) return cudaErrorInvalidValue;
  k_row_dots1<T><<<dim3(kPartials, (unsigned)M), kThreads, 0, s>>>(x, y, n, partial);
  k_row_dots2<<<(unsigned)M, 32, 0, s>>>(partial, kPartials, w, out_dev);
  return cudaGetLastError();
}
template cudaError_t row_dots<double>(const double*, const double*, long long, long long, double,
                                      double*, double*, cudaStream_t);
template cudaError_t row_dots<float>(const float*, const float*, long long, long long, double,
                                     double*, double*, cudaStream_t);

template <typename T>
cudaError_t normalize_rows(T* x, long long M, long long n, double dv, double* partial,
                           double* norms_dev, cudaStream_t s) {
  cudaError_t e = row_dots<T>(x, x, M, n, 1.0, norms_dev, partial, s);
  if (e) return e;
  k_scale_rows<T><<<dim3(64, (unsigned)M), kThreads, 0, s>>>(x, n, norms_dev, dv);
  return cudaGetLastError();
}
template <typename T>
cudaError_t scale_rows(T* x, long long M, long long n, const double* norms_dev, double dv,
                       cudaStream_t s) {
  if (M > 65535) return cudaErrorInvalidValue;
  k_scale_rows<T><<<dim3(64, (unsigned)M), kThreads, 0, s>>>(x, n, norms_dev, dv);
  return cudaGetLastError();
}
template cudaError_t scale_rows<double>(double*, long long, long long, const double*, double,
                                        cudaStream_t);
template cudaError_t normalize_rows<double>(double*, long long, long long, double, double*,
                                            double*, cudaStream_t);
template cudaError_t normalize_rows<float>(float*, long long, long long, double, double*,
                                           double*, cudaStream_t);

size_t gemm_nt_work_doubles(long long M, long long Nn, long long K) {
  (void)K;
  return (size_t)M * Nn * 32;  // up to 32 K-splits
}

cudaError_t gemm_nt_f64(const double* A, const double* B, long long M, long long Nn,
                        long long K, double alpha, double* C, bool sym, double* work,
                        size_t work_doubles, cudaStream_t s) {
  const long long tm = (M + TM - 1) / TM, tn = (Nn + TN - 1) / TN;
  long long tiles = sym ? tm * (tm + 1) / 2 : tm * tn;
  // enough blocks to fill 152 SMs a few times over
  long long splits = (152LL * 4 + tiles - 1) / tiles;
  if (splits > 32) splits = 32;
  if (splits < 1) splits = 1;
  while (splits > 1 && (size_t)(splits * M * Nn) > work_doubles) --splits;
  long long kchunk = (K + splits - 1) / splits;
  kchunk = (kchunk + TK - 1) / TK * TK;
  splits = (K + kchunk - 1) / kchunk;
  if (splits < 1) splits = 1;
  if ((size_t)(splits * M * Nn) > work_doubles) return cudaErrorInvalidValue;
  if (tm > 65535 || splits > 65535) return cudaErrorInvalidValue;
  k_gemm_nt<<<dim3((unsigned)tn, (unsigned)tm, (unsigned)splits), 256, 0, s>>>(A, B, M, Nn, K,
                                                                             kchunk, work, sym);
  k_gemm_nt_reduce<<<blocks_for(M * Nn, kThreads), kThreads, 0, s>>>(work, (int)splits, M, Nn,
                                                                     alpha, C, sym);
  return cudaGetLastError();
}

cudaError_t gemm_nn_f64_ld(const double* A, const double* B, long long M, long long Nn,
                           long long K, long long ldb, double* C, cudaStream_t s) {
  const long long tm = (M + TM - 1) / TM, tn = (Nn + TN - 1) / TN;
  if (tm > 65535 || tn > 0x7fffffffLL) return cudaErrorInvalidValue;
  k_gemm_nn<<<dim3((unsigned)tn, (unsigned)tm), 256, 0, s>>>(A, B, M, Nn, K, ldb, Nn, C);
  return cudaGetLastError();
}

cudaError_t gemm_nn_f64(const double* A, const double* B, long long M, long long Nn,
                        long long K, double* C, cudaStream_t s) {
  return gemm_nn_f64_ld(A, B, M, Nn, K, Nn, C, s);
}

namespace {
__global__ void k_symmetrize(double* __restrict__ A, long long m) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < m * m;
       i += (long long)gridDim.x * blockDim.x) {
    const long long r = i / m, c = i - r * m;
    if (c > r) {
      const double v = 0.5 * (A[r * m + c] + A[c * m + r]);
      A[r * m + c] = v;
      A[c * m + r] = v;
    }
  }
}
__global__ void k_scale_rows_isqrt(const double* __restrict__ R, const double* __restrict__ lam,
                                   long long k, double* __restrict__ S) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < k * k;
       i += (long long)gridDim.x * blockDim.x) {
    const long long l = i / k;
    S[i] = R[i] / sqrt(lam[l]);
  }
}
template <typename T>
__global__ void k_scale_copy(const cx<T>* __restrict__ in, cx<T>* __restrict__ out,
                             long long count, double f) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    const cx<T> v = in[i];
    out[i] = mk<T>((T)(v.x * f), (T)(v.y * f));
  }
}
}  // namespace

namespace {
__global__ void k_sub_2d(double* __restrict__ dst, long long ld, const double* __restrict__ src,
                         long long rows, long long w) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < rows * w;
       i += (long long)gridDim.x * blockDim.x) {
    const long long r = i / w, c = i - r * w;
    dst[r * ld + c] -= src[i];
  }
}
}  // namespace

cudaError_t sub_2d_f64(double* dst, long long ld, const double* src, long long rows,
                       long long w, cudaStream_t s) {
  k_sub_2d<<<blocks_for(rows * w, kThreads), kThreads, 0, s>>>(dst, ld, src, rows, w);
  return cudaGetLastError();
}

namespace {
__global__ void k_weighted_density(const double* __restrict__ psi, const double* __restrict__ w,
                                   long long m, long long n, double dv,
                                   double* __restrict__ rho) {
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < n;
       g += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (long long k = 0; k < m; ++k) {
      const double p = psi[k * n + g];
      s += w[k] * p * p;
    }
    rho[g] = s * dv;
  }
}
}  // namespace

cudaError_t weighted_density(const double* psi, const double* w, long long m, long long n,
                             double dv, double* rho, cudaStream_t s) {
  k_weighted_density<<<blocks_for(n, kThreads), kThreads, 0, s>>>(psi, w, m, n, dv, rho);
  return cudaGetLastError();
}

cudaError_t symmetrize_f64(double* A, long long m, cudaStream_t s) {
  k_symmetrize<<<blocks_for(m * m, kThreads), kThreads, 0, s>>>(A, m);
  return cudaGetLastError();
}

cudaError_t scale_rows_isqrt(const double* R, const double* lam, long long k, double* S,
                             cudaStream_t s) {
  k_scale_rows_isqrt<<<blocks_for(k * k, kThreads), kThreads, 0, s>>>(R, lam, k, S);
  return cudaGetLastError();
}

template <typename T>
cudaError_t scale_copy(const cx<T>* in, cx<T>* out, long long count, double f, cudaStream_t s) {
  k_scale_copy<T><<<blocks_for(count, kThreads), kThreads, 0, s>>>(in, out, count, f);
  return cudaGetLastError();
}
template cudaError_t scale_copy<double>(const cx<double>*, cx<double>*, long long, double,
                                        cudaStream_t);
template cudaError_t scale_copy<float>(const cx<float>*, cx<float>*, long long, double,
                                       cudaStream_t);

cudaError_t transpose_f64(const double* in, long long rows, long long cols, double* out,
                          cudaStream_t s) {
  dim3 g((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32));
  k_transpose<<<g, dim3(32, 8), 0, s>>>(in, rows, cols, out);
  return cudaGetLastError();
}

cudaError_t scale_eigvecs(const double* V, const double* lam, long long M, long long k0,
                          double* out, cudaStream_t s) {
  k_scale_eigvecs<<<blocks_for((M - k0) * M, kThreads), kThreads, 0, s>>>(V, lam, M, k0, out);
  return cudaGetLastError();
}

cudaError_t residual_norms(const double* x, const double* hx, const double* e, long long M,
                           long long n, double dv, double* out_dev, double* partial,
                           cudaStream_t s) {
  if (M > 65535) return cudaErrorInvalidValue;
  k_resid1<<<dim3(kPartials, (unsigned)M), kThreads, 0, s>>>(x, hx, e, n, partial);
  k_row_dots2<<<(unsigned)M, 32, 0, s>>>(partial, kPartials, 1.0, out_dev);
  k_sqrt_scaled<<<(unsigned)((M + 255) / 256), 256, 0, s>>>(out_dev, M, dv);
  return cudaGetLastError();
}

__global__ void k_residual_rows(const double* __restrict__ x, const double* hx,
                                const double* __restrict__ e, long long M, long long n,
                                double* out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < M * n;
       i += (long long)gridDim.x * blockDim.x)
    out[i] = hx[i] - e[i / n] * x[i];
}

cudaError_t residual_rows(const double* x, const double* hx, const double* e, long long M,
                          long long n, double* out, cudaStream_t s) {
  k_residual_rows<<<blocks_for(M * n, kThreads), kThreads, 0, s>>>(x, hx, e, M, n, out);
  return cudaGetLastError();
}

cudaError_t convert_f32_to_f64(const float* in, double* out, long long count, cudaStream_t s) {
  k_convert<float, double><<<blocks_for(count, kThreads), kThreads, 0, s>>>(in, out, count);
  return cudaGetLastError();
}
cudaError_t convert_f64_to_f32(const double* in, float* out, long long count, cudaStream_t s) {
  k_convert<double, float><<<blocks_for(count, kThreads), kThreads, 0, s>>>(in, out, count);
  return cudaGetLastError();
}
cudaError_t convert_f64_to_dd(const double* in, ddf* out, long long count, cudaStream_t s) {
  k_convert<double, ddf><<<blocks_for(count, kThreads), kThreads, 0, s>>>(in, out, count);
  return cudaGetLastError();
}

}  // namespace sep
