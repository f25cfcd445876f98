// sep_xypass.cuh -- the x and y transforms of a Newton step on whole z-planes
// held in shared memory (complex64), fused with the epilogue.
//
// With the line passes a Newton step makes four passes over the grids (y
// forward, z forward*k^2*inverse, y inverse, x inverse+epilogue+forward).
// When an xy-plane of complex64 fits in shared memory (nx = ny <= 128: 132 KB)
// the step needs two: the z pass, then one pass per z-plane that does
//   y inverse, x inverse, psi_j = alpha (T + V psi_{j-1}) + beta psi_{j-1}
//   (filter/hnorm.c:11-39), x forward, y forward
// so the grid is read and written once less per step.
//
// Each 1-D transform is the four-step split of sep_fftpass.cuh, with the same
// register DFTs and twiddles in the same order, run in place on the plane:
// lines are the rows (x transforms) or the columns (y transforms).  The row
// stride is nx + 1 elements, so that 32 threads on 32 different rows, or on 32
// adjacent columns, touch 32 different bank pairs.
#pragma once

#include "sep_fftpass.cuh"

namespace sep {

constexpr int kXyThreads = 512;

// forward (SIGN -1) or inverse (SIGN +1) transform of NL lines of length L in
// place, natural order in and out; line l starts at l * LS, element e of a
// line at e * ES
template <int L, int SIGN, int NL, int LS, int ES>
__device__ __forceinline__ void plane_fft(cx<float>* pl, const cx<float>* tws) {
  using C = cx<float>;
  constexpr int N1 = Split<L>::n1, N2 = Split<L>::n2;
  constexpr int NA = NL * N1, NB = NL * N2;
  constexpr int NT = kXyThreads;
  const int tid = threadIdx.x;
  if constexpr (SIGN < 0) {
    // stage A: item (line, x1): elements x1 + N1 x2 -> DFT_N2, twiddle; the
    // results go back to the positions the item read
    for (int i = tid; i < NA; i += NT) {
      const int line = i % NL, x1 = i / NL;
      C* p = pl + line * LS;
      C v[N2];
#pragma unroll
      for (int x2 = 0; x2 < N2; ++x2) v[x2] = p[(x1 + N1 * x2) * ES];
      Dft<N2, -1, float>::run(v);
#pragma unroll
      for (int k2 = 1; k2 < N2; ++k2) v[k2] = mul<float>(v[k2], tws[(x1 * k2) % L]);
#pragma unroll
      for (int k2 = 0; k2 < N2; ++k2) p[(x1 + N1 * k2) * ES] = v[k2];
    }
    __syncthreads();
    // stage B: item (line, k2): positions x1 + N1 k2 -> DFT_N1 -> element k2 + N2 k1
    constexpr int IB = (NB + NT - 1) / NT;
    C w[IB][N1];
#pragma unroll
    for (int r = 0; r < IB; ++r) {
      const int i = tid + r * NT;
      if (NB % NT == 0 || i < NB) {
        const int line = i % NL, k2 = i / NL;
        const C* p = pl + line * LS;
#pragma unroll
        for (int x1 = 0; x1 < N1; ++x1) w[r][x1] = p[(x1 + N1 * k2) * ES];
        Dft<N1, -1, float>::run(w[r]);
      }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < IB; ++r) {
      const int i = tid + r * NT;
      if (NB % NT == 0 || i < NB) {
        const int line = i % NL, k2 = i / NL;
        C* p = pl + line * LS;
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) p[(k2 + N2 * k1) * ES] = w[r][k1];
      }
    }
    __syncthreads();
  } else {
    // stage B': item (line, k2): elements k2 + N2 k1 -> inverse DFT_N1,
    // conjugate twiddle; back to the positions the item read
    for (int i = tid; i < NB; i += NT) {
      const int line = i % NL, k2 = i / NL;
      C* p = pl + line * LS;
      C v[N1];
#pragma unroll
      for (int k1 = 0; k1 < N1; ++k1) v[k1] = p[(k2 + N2 * k1) * ES];
      Dft<N1, +1, float>::run(v);
#pragma unroll
      for (int n1 = 1; n1 < N1; ++n1) v[n1] = mulc<float>(v[n1], tws[(n1 * k2) % L]);
#pragma unroll
      for (int n1 = 0; n1 < N1; ++n1) p[(k2 + N2 * n1) * ES] = v[n1];
    }
    __syncthreads();
    // stage A': item (line, n1): positions k2 + N2 n1 -> inverse DFT_N2 ->
    // element n1 + N1 n2
    constexpr int IA = (NA + NT - 1) / NT;
    C u[IA][N2];
#pragma unroll
    for (int r = 0; r < IA; ++r) {
      const int i = tid + r * NT;
      if (NA % NT == 0 || i < NA) {
        const int line = i % NL, n1 = i / NL;
        const C* p = pl + line * LS;
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) u[r][k2] = p[(k2 + N2 * n1) * ES];
        Dft<N2, +1, float>::run(u[r]);
      }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < IA; ++r) {
      const int i = tid + r * NT;
      if (NA % NT == 0 || i < NA) {
        const int line = i % NL, n1 = i / NL;
        C* p = pl + line * LS;
#pragma unroll
        for (int n2 = 0; n2 < N2; ++n2) p[(n1 + N1 * n2) * ES] = u[r][n2];
      }
    }
    __syncthreads();
  }
}

// One block per (grid of the batch, z-plane), the grids of one plane adjacent
// so that the plane of V is read from L2 after its first use.  MODE: kFwd (x
// and y forward of src, or of data), kInvEpi (y and x inverse + epilogue),
// kInvEpiFwd (and the forward transforms of the result).  Global accesses
// move two neighbouring x values at a time, eight per thread in flight.
template <int LX, int LY, int MODE>
__global__ void __launch_bounds__(kXyThreads, 1) xy_plane_pass(PassArgs<float> a) {
  using C = cx<float>;
  constexpr int RS = LX + 1;
  static_assert(LX % 2 == 0, "pairs of neighbouring x values");
  constexpr int NP = LX * LY / 2;                  // pairs of x values in a plane
  constexpr bool WHOLE = NP % (8 * kXyThreads) == 0;  // batches of 8 pairs per thread
  extern __shared__ __align__(16) unsigned char xy_smem[];
  C* pl = reinterpret_cast<C*>(xy_smem);
  C* twx = pl + LY * RS;
  C* twy = twx + LX;
  const int tid = threadIdx.x;
  const long long N = (long long)LX * LY * a.nz;
  const long long goff = (long long)blockIdx.y * LX * LY;  // offset in one grid
  const long long off = (long long)blockIdx.x * N + goff;
  for (int m = tid; m < LX; m += kXyThreads) twx[m] = a.tw[m];
  for (int m = tid; m < LY; m += kXyThreads) twy[m] = a.tw2[m];
  const C* src = (MODE == kFwd && a.src) ? a.src : a.data;
  {
    const float4* s4 = reinterpret_cast<const float4*>(src + off);
    for (int q0 = tid; q0 < NP; q0 += 8 * kXyThreads) {
      float4 v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (WHOLE || q0 + u * kXyThreads < NP) v[u] = s4[q0 + u * kXyThreads];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        if (!WHOLE && q0 + u * kXyThreads >= NP) break;
        const int i = 2 * (q0 + u * kXyThreads);
        C* q = pl + (i / LX) * RS + (i % LX);
        q[0] = mk<float>(v[u].x, v[u].y);
        q[1] = mk<float>(v[u].z, v[u].w);
      }
    }
  }
  __syncthreads();
  if constexpr (MODE != kFwd) {
    plane_fft<LY, +1, LX, 1, RS>(pl, twy);  // y inverse: lines are the columns
    plane_fft<LX, +1, LY, RS, 1>(pl, twx);  // x inverse: lines are the rows
    float alpha = a.alpha, beta = a.beta;
    if (a.coefs) {
      alpha = a.coefs[2 * a.step];
      beta = a.coefs[2 * a.step + 1];
    }
    const float4* pin = a.psi_in ? reinterpret_cast<const float4*>(a.psi_in + off) : nullptr;
    const float2* pv = reinterpret_cast<const float2*>(a.pot + goff);
    float4* pout = reinterpret_cast<float4*>(a.psi_out + off);
    for (int q0 = tid; q0 < NP; q0 += 8 * kXyThreads) {
      float4 p[8];
      float2 v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        if (WHOLE || q0 + u * kXyThreads < NP) {
          p[u] = pin ? pin[q0 + u * kXyThreads] : make_float4(0.f, 0.f, 0.f, 0.f);
          v[u] = pv[q0 + u * kXyThreads];
        }
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        if (!WHOLE && q0 + u * kXyThreads >= NP) break;
        const int i = 2 * (q0 + u * kXyThreads);
        C* q = pl + (i / LX) * RS + (i % LX);
        const C o0 = newton_epi<float>(q[0], v[u].x, mk<float>(p[u].x, p[u].y), alpha, beta);
        const C o1 = newton_epi<float>(q[1], v[u].y, mk<float>(p[u].z, p[u].w), alpha, beta);
        pout[q0 + u * kXyThreads] = make_float4(o0.x, o0.y, o1.x, o1.y);
        q[0] = o0;
        q[1] = o1;
      }
    }
    __syncthreads();
  }
  if constexpr (MODE != kInvEpi) {
    plane_fft<LX, -1, LY, RS, 1>(pl, twx);  // x forward
    plane_fft<LY, -1, LX, 1, RS>(pl, twy);  // y forward
    float4* d4 = reinterpret_cast<float4*>(a.data + off);
    for (int q = tid; q < NP; q += kXyThreads) {
      const int i = 2 * q;
      const C* r = pl + (i / LX) * RS + (i % LX);
      d4[q] = make_float4(r[0].x, r[0].y, r[1].x, r[1].y);
    }
  }
}

}  // namespace sep
