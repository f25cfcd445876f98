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
// Transforms.  Each 1-D transform of length L = N1 N2 is the four-step split
// of sep_fftpass.cuh, with the same register DFTs and twiddles in the same
// order, done in place and self-sorting: every item writes its results back to
// the positions it read.  The forward transform then leaves element
//   k = k2 + N2 k1   at position   k1 + N1 k2
// and the inverse transform takes its input in that order and leaves natural
// order.  Between passes the grids are therefore kept with x and y in this
// digit-reversed position order (z natural); the z pass looks k^2 up through
// tables in the same order, so every element sees the same arithmetic as with
// the line passes.  The epilogue (psi_{j-1}, V, psi_j) runs in natural order.
//
// Passes over shared memory.  The first y stage reads the plane from global
// memory and the last one writes it there; x inverse stage A', the epilogue
// and x forward stage A work on the same items and share one pass.  In the
// step pass (inverse, epilogue, forward) the last y stage of a plane and the
// first y stage of the block's next plane also share one pass
// (col_fwd_b_inv_b_next), so that the next plane's loads are in flight while
// the current plane is written out.  The row stride is L + 1 elements, so
// that the threads of a half-warp on 16 different rows, or on 16 adjacent
// columns, touch different bank pairs.  Each block prefetches its next plane,
// psi_{j-1} and V into L2 while it transforms the current one.
#pragma once

#include "sep_fftpass.cuh"

namespace sep {

// the plane pass's launch shape per length: threads per block and blocks per
// SM.  A block needs about 128 registers per thread and its plane in shared
// memory (13 KB at 40^2, 19 KB at 48^2, 25 KB at 56^2, 33 KB at 64^2, 42 KB
// at 72^2, 52 KB at 80^2, 74 KB at 96^2, 102 KB at 112^2, 132 KB at 128^2).
// Several blocks per SM let one block's transforms run while another waits
// for memory; the shapes are the fastest measured per length (step pass on
// 0.5 GB of grids, fraction of the copy bandwidth: 40^2 0.79, 48^2 0.79, 56^2
// 0.75, 64^2 0.84, 72^2 0.79, 80^2 0.74, 96^2 0.76 against 0.57 with one
// block of 512, 112^2 0.64, 128^2 0.73).  Only one 128^2 plane fits per SM.
template <int L> struct XyTune {
  static constexpr int nt = 512;
  static constexpr int min_blocks = 1;
};
template <> struct XyTune<40> {
  static constexpr int nt = 64, min_blocks = 8;
};
template <> struct XyTune<56> {
  static constexpr int nt = 128, min_blocks = 4;
};
template <> struct XyTune<72> {
  static constexpr int nt = 128, min_blocks = 4;
};
template <> struct XyTune<48> {
  static constexpr int nt = 128, min_blocks = 4;
};
template <> struct XyTune<64> {
  static constexpr int nt = 256, min_blocks = 3;
};
template <> struct XyTune<80> {
  static constexpr int nt = 128, min_blocks = 4;
};
template <> struct XyTune<96> {
  static constexpr int nt = 192, min_blocks = 2;
};
template <> struct XyTune<112> {
  static constexpr int nt = 128, min_blocks = 2;
};

template <int L, int NT> struct XyShape {
  static constexpr int n1 = Split<L>::n1, n2 = Split<L>::n2;
  static constexpr int rs = L + 1;  // row stride (elements)
  static constexpr int nt = NT;     // threads per block
  static_assert(n1 == 8 && L % 8 == 0, "row groups of the epilogue step");
  static constexpr size_t smem_bytes = ((size_t)L * rs + L) * sizeof(cx<float>);
};

namespace xy {

using C = cx<float>;

// bulk L2 prefetch of [p, p + bytes) (16-byte aligned, bytes a multiple of
// 16) in 16 KB pieces, one per lane of the calling warp
__device__ __forceinline__ void prefetch_l2(const void* p, unsigned bytes, int lane) {
  constexpr unsigned kPiece = 16384;
  for (unsigned o = (unsigned)lane * kPiece; o < bytes; o += 32 * kPiece) {
    const unsigned n = bytes - o < kPiece ? bytes - o : kPiece;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"((const char*)p + o), "r"(n)
                 : "memory");
  }
}

// row of group j of an x stage whose items are spread over N1 = 8 threads:
// the two rows of a half-warp are 8 apart (16 banks apart with stride L + 1).
// When L is 8 more than a multiple of 16, the last 8 rows pair rows 4 apart
// (a bijection on those rows; some of their accesses share banks).
template <int L> __device__ __forceinline__ int row_of_group(int j) {
  constexpr int full = L & ~15;
  if (L % 16 == 0 || j < full) return (j & ~15) | ((j & 1) << 3) | ((j >> 1) & 7);
  return full + ((j & 1) << 2) + ((j >> 1) & 3);
}

// ---- y transforms: lines are the columns (element stride RS)

// inverse stage B' from global memory (g: the plane in position order, row
// stride L): item (column, k2): positions k1 + N1 k2 -> inverse DFT_N1,
// conjugate twiddle, back to the same positions in shared memory.  Adjacent
// threads on adjacent columns; a thread's items (four when they divide
// evenly, else two at a time) are loaded before any is transformed.
template <int L, int NT>
__device__ __forceinline__ void col_inv_b_from(C* pl, const C* tw, const C* __restrict__ g) {
  using S = XyShape<L, NT>;
  constexpr int NI = L * S::n2;
  constexpr int IB = NI % (4 * S::nt) == 0 ? 4 : 2;  // items loaded per batch
  for (int i0 = threadIdx.x; i0 < NI; i0 += IB * S::nt) {
    C v[IB][S::n1];
#pragma unroll
    for (int t = 0; t < IB; ++t) {
      const int i = i0 + t * S::nt;
      if (NI % (IB * S::nt) == 0 || i < NI) {
        const int col = i % L, k2 = i / L;
        const C* q = g + (long long)(S::n1 * k2) * L + col;
#pragma unroll
        for (int k1 = 0; k1 < S::n1; ++k1) v[t][k1] = q[(long long)k1 * L];
      }
    }
#pragma unroll
    for (int t = 0; t < IB; ++t) {
      const int i = i0 + t * S::nt;
      if (NI % (IB * S::nt) == 0 || i < NI) {
        const int col = i % L, k2 = i / L;
        Dft<S::n1, +1, float>::run(v[t]);
#pragma unroll
        for (int n1 = 1; n1 < S::n1; ++n1) v[t][n1] = mulc<float>(v[t][n1], tw[(n1 * k2) % L]);
        C* p = pl + S::n1 * k2 * S::rs + col;
#pragma unroll
        for (int n1 = 0; n1 < S::n1; ++n1) p[n1 * S::rs] = v[t][n1];
      }
    }
  }
}

// inverse stage A': item (column, n1): positions n1 + N1 k2 -> inverse DFT_N2;
// element n1 + N1 n2 at its natural position
template <int L, int NT> __device__ __forceinline__ void col_inv_a(C* pl) {
  using S = XyShape<L, NT>;
  for (int i = threadIdx.x; i < L * S::n1; i += S::nt) {
    const int col = i % L, n1 = i / L;
    C* p = pl + n1 * S::rs + col;
    C u[S::n2];
#pragma unroll
    for (int k2 = 0; k2 < S::n2; ++k2) u[k2] = p[S::n1 * k2 * S::rs];
    Dft<S::n2, +1, float>::run(u);
#pragma unroll
    for (int n2 = 0; n2 < S::n2; ++n2) p[S::n1 * n2 * S::rs] = u[n2];
  }
}

// forward stage A: item (column, x1): positions x1 + N1 x2 -> DFT_N2, twiddle
template <int L, int NT> __device__ __forceinline__ void col_fwd_a(C* pl, const C* tw) {
  using S = XyShape<L, NT>;
  for (int i = threadIdx.x; i < L * S::n1; i += S::nt) {
    const int col = i % L, x1 = i / L;
    C* p = pl + x1 * S::rs + col;
    C v[S::n2];
#pragma unroll
    for (int x2 = 0; x2 < S::n2; ++x2) v[x2] = p[S::n1 * x2 * S::rs];
    Dft<S::n2, -1, float>::run(v);
#pragma unroll
    for (int k2 = 1; k2 < S::n2; ++k2) v[k2] = mul<float>(v[k2], tw[(x1 * k2) % L]);
#pragma unroll
    for (int k2 = 0; k2 < S::n2; ++k2) p[S::n1 * k2 * S::rs] = v[k2];
  }
}

// forward stage B to global memory: item (column, k2): positions x1 + N1 k2
// -> DFT_N1; element k2 + N2 k1 to position k1 + N1 k2 of g
template <int L, int NT> __device__ __forceinline__ void col_fwd_b_to(const C* pl, C* __restrict__ g) {
  using S = XyShape<L, NT>;
  for (int i = threadIdx.x; i < L * S::n2; i += S::nt) {
    const int col = i % L, k2 = i / L;
    const C* p = pl + S::n1 * k2 * S::rs + col;
    C w[S::n1];
#pragma unroll
    for (int x1 = 0; x1 < S::n1; ++x1) w[x1] = p[x1 * S::rs];
    Dft<S::n1, -1, float>::run(w);
    C* q = g + (long long)(S::n1 * k2) * L + col;
#pragma unroll
    for (int k1 = 0; k1 < S::n1; ++k1) q[(long long)k1 * L] = w[k1];
  }
}

// forward stage B of the current plane (to gcur) and inverse stage B' of the
// block's next plane (from gnext) in one pass: both stages have the items
// (column, k2) at the same shared-memory positions and the same thread
// mapping, so each thread first issues the loads of two next-plane items,
// then transforms and stores its current items, then transforms the loaded
// ones into the positions it has just read.  The next plane's load latency
// runs under the current plane's last stage, and one barrier goes.
template <int L, int NT>
__device__ __forceinline__ void col_fwd_b_inv_b_next(C* pl, const C* tw, C* __restrict__ gcur,
                                                     const C* __restrict__ gnext) {
  using S = XyShape<L, NT>;
  constexpr int NI = L * S::n2;
  constexpr int IB = 2;
  for (int i0 = threadIdx.x; i0 < NI; i0 += IB * S::nt) {
    C v[IB][S::n1];
#pragma unroll
    for (int t = 0; t < IB; ++t) {
      const int i = i0 + t * S::nt;
      if (NI % (IB * S::nt) == 0 || i < NI) {
        const int col = i % L, k2 = i / L;
        const C* q = gnext + (long long)(S::n1 * k2) * L + col;
#pragma unroll
        for (int k1 = 0; k1 < S::n1; ++k1) v[t][k1] = q[(long long)k1 * L];
      }
    }
#pragma unroll
    for (int t = 0; t < IB; ++t) {
      const int i = i0 + t * S::nt;
      if (NI % (IB * S::nt) == 0 || i < NI) {
        const int col = i % L, k2 = i / L;
        C* p = pl + S::n1 * k2 * S::rs + col;
        C w[S::n1];
#pragma unroll
        for (int x1 = 0; x1 < S::n1; ++x1) w[x1] = p[x1 * S::rs];
        Dft<S::n1, -1, float>::run(w);
        C* q = gcur + (long long)(S::n1 * k2) * L + col;
#pragma unroll
        for (int k1 = 0; k1 < S::n1; ++k1) q[(long long)k1 * L] = w[k1];
      }
    }
#pragma unroll
    for (int t = 0; t < IB; ++t) {
      const int i = i0 + t * S::nt;
      if (NI % (IB * S::nt) == 0 || i < NI) {
        const int col = i % L, k2 = i / L;
        Dft<S::n1, +1, float>::run(v[t]);
#pragma unroll
        for (int n1 = 1; n1 < S::n1; ++n1) v[t][n1] = mulc<float>(v[t][n1], tw[(n1 * k2) % L]);
        C* p = pl + S::n1 * k2 * S::rs + col;
#pragma unroll
        for (int n1 = 0; n1 < S::n1; ++n1) p[n1 * S::rs] = v[t][n1];
      }
    }
  }
}

// ---- x transforms: lines are the rows

// inverse stage B': item (row, k2): positions k1 + N1 k2 (elements k2 + N2 k1)
// -> inverse DFT_N1, conjugate twiddle
template <int L, int NT> __device__ __forceinline__ void row_inv_b(C* pl, const C* tw) {
  using S = XyShape<L, NT>;
  for (int i = threadIdx.x; i < L * S::n2; i += S::nt) {
    const int row = i % L, k2 = i / L;
    C* p = pl + row * S::rs + S::n1 * k2;
    C v[S::n1];
#pragma unroll
    for (int k1 = 0; k1 < S::n1; ++k1) v[k1] = p[k1];
    Dft<S::n1, +1, float>::run(v);
#pragma unroll
    for (int n1 = 1; n1 < S::n1; ++n1) v[n1] = mulc<float>(v[n1], tw[(n1 * k2) % L]);
#pragma unroll
    for (int n1 = 0; n1 < S::n1; ++n1) p[n1] = v[n1];
  }
}

// forward stage B: item (row, k2): positions x1 + N1 k2 -> DFT_N1; element
// k2 + N2 k1 stays at position k1 + N1 k2
template <int L, int NT> __device__ __forceinline__ void row_fwd_b(C* pl) {
  using S = XyShape<L, NT>;
  for (int i = threadIdx.x; i < L * S::n2; i += S::nt) {
    const int row = i % L, k2 = i / L;
    C* p = pl + row * S::rs + S::n1 * k2;
    C w[S::n1];
#pragma unroll
    for (int x1 = 0; x1 < S::n1; ++x1) w[x1] = p[x1];
    Dft<S::n1, -1, float>::run(w);
#pragma unroll
    for (int k1 = 0; k1 < S::n1; ++k1) p[k1] = w[k1];
  }
}

// x inverse stage A', the Newton epilogue and (FWD) x forward stage A in one
// step: item (row, n1) holds the natural elements n1 + N1 n2 of its row, which
// are also the inputs of forward item (row, x1 = n1).  psi_{j-1}, V and psi_j
// (plane offsets off in the batch, goff in one grid) are accessed at those
// elements: eight threads cover N1 = 8 adjacent elements (64 bytes) of a row.
template <int L, int NT, bool FWD>
__device__ __forceinline__ void row_inv_a_epi(C* pl, const C* tw, const PassArgs<float>& a,
                                              long long off, long long goff, float alpha,
                                              float beta) {
  using S = XyShape<L, NT>;
  const C* __restrict__ pin = a.psi_in ? a.psi_in + off : nullptr;
  const float* __restrict__ pv = a.pot + goff;
  C* __restrict__ pout = a.psi_out + off;
  for (int i = threadIdx.x; i < L * 8; i += S::nt) {
    const int n1 = i & 7, row = row_of_group<L>(i >> 3);
    const long long g0 = (long long)row * L + n1;
    // the item's psi_{j-1} and V are requested before its transform, so
    // their latency runs under the shared-memory reads and the DFT
    C q[S::n2];
    float v[S::n2];
#pragma unroll
    for (int n2 = 0; n2 < S::n2; ++n2) {
      const long long e = g0 + S::n1 * n2;
      q[n2] = pin ? pin[e] : mk<float>(0.f, 0.f);
      v[n2] = pv[e];
    }
    C* p = pl + row * S::rs + n1;
    C u[S::n2];
#pragma unroll
    for (int k2 = 0; k2 < S::n2; ++k2) u[k2] = p[S::n1 * k2];
    Dft<S::n2, +1, float>::run(u);
#pragma unroll
    for (int n2 = 0; n2 < S::n2; ++n2) {
      const C o = newton_epi<float>(u[n2], v[n2], q[n2], alpha, beta);
      pout[g0 + S::n1 * n2] = o;
      u[n2] = o;
    }
    if constexpr (FWD) {
      Dft<S::n2, -1, float>::run(u);
#pragma unroll
      for (int k2 = 1; k2 < S::n2; ++k2) u[k2] = mul<float>(u[k2], tw[(n1 * k2) % L]);
#pragma unroll
      for (int k2 = 0; k2 < S::n2; ++k2) p[S::n1 * k2] = u[k2];
    }
  }
}

// x forward stage A from global memory (natural order): item (row, x1)
template <int L, int NT>
__device__ __forceinline__ void row_fwd_a_from(C* pl, const C* tw, const C* __restrict__ g) {
  using S = XyShape<L, NT>;
  for (int i = threadIdx.x; i < L * 8; i += S::nt) {
    const int x1 = i & 7, row = row_of_group<L>(i >> 3);
    const C* q = g + (long long)row * L + x1;
    C v[S::n2];
#pragma unroll
    for (int x2 = 0; x2 < S::n2; ++x2) v[x2] = q[S::n1 * x2];
    Dft<S::n2, -1, float>::run(v);
#pragma unroll
    for (int k2 = 1; k2 < S::n2; ++k2) v[k2] = mul<float>(v[k2], tw[(x1 * k2) % L]);
    C* p = pl + row * S::rs + x1;
#pragma unroll
    for (int k2 = 0; k2 < S::n2; ++k2) p[S::n1 * k2] = v[k2];
  }
}

}  // namespace xy

// Block b of the grid walks the planes p = b + k gridDim.x of the batch (one
// block per SM, or one block per plane), plane p = (z, grid b) with z = p / B, b = p % B, so that the
// blocks running at one time share the plane of V.  After its epilogue a
// block prefetches the data of its next plane into L2, so that the plane's
// HBM reads overlap the forward transforms of this one; psi_{j-1} and V are
// prefetched when the plane starts.
// MODE: kFwd (x and y forward of src, or of data, natural order in),
// kInvEpi (y and x inverse + epilogue), kInvEpiFwd (and the forward
// transforms of the result).
template <int L, int MODE, int NT = XyTune<L>::nt, int MINB = XyTune<L>::min_blocks>
__global__ void __launch_bounds__(NT, MINB) xy_plane_pass(PassArgs<float> a, int B) {
  using C = cx<float>;
  using S = XyShape<L, NT>;
  extern __shared__ __align__(16) unsigned char xy_smem[];
  C* pl = reinterpret_cast<C*>(xy_smem);
  C* tw = pl + L * S::rs;
  const int tid = threadIdx.x;
  const long long N = (long long)L * L * a.nz;
  const long long planes = (long long)B * a.nz;
  const C* src = (MODE == kFwd && a.src) ? a.src : a.data;
  // the plane's data (prefetch distance: from the epilogue of the block's
  // previous plane), and its psi_{j-1} and V (from the start of the plane)
  auto prefetch_data = [&](long long p) {
    if (tid < 32 && p < planes)
      xy::prefetch_l2(src + (p % B) * N + (p / B) * L * L, (unsigned)(L * L * sizeof(C)), tid);
  };
  auto prefetch_epi = [&](long long p) {
    if (MODE != kFwd && tid < 32) {
      const long long goff = (p / B) * L * L, off = (p % B) * N + goff;
      if (a.psi_in) xy::prefetch_l2(a.psi_in + off, (unsigned)(L * L * sizeof(C)), tid);
      xy::prefetch_l2(a.pot + goff, (unsigned)(L * L * sizeof(float)), tid);
    }
  };
  prefetch_data(blockIdx.x);
  for (int m = tid; m < L; m += S::nt) tw[m] = a.tw[m];  // x and y tables are equal
  float alpha = a.alpha, beta = a.beta;
  if (a.coefs) {
    alpha = a.coefs[2 * a.step];
    beta = a.coefs[2 * a.step + 1];
  }
  bool loaded = false;  // kInvEpiFwd: this plane's first stage ran with the previous plane's last
  for (long long p = blockIdx.x; p < planes; p += gridDim.x) {
    prefetch_epi(p);
    const long long goff = (p / B) * L * L;  // offset in one grid
    const long long off = (p % B) * N + goff;
    __syncthreads();  // the previous plane's last stage has read the plane
    if constexpr (MODE == kFwd) {
      xy::row_fwd_a_from<L, NT>(pl, tw, src + off);  // x forward
    } else {
      if (!loaded) {
        xy::col_inv_b_from<L, NT>(pl, tw, a.data + off);  // y inverse
        __syncthreads();
      }
      xy::col_inv_a<L, NT>(pl);
      __syncthreads();
      xy::row_inv_b<L, NT>(pl, tw);  // x inverse, epilogue (and x forward stage A)
      __syncthreads();
      xy::row_inv_a_epi<L, NT, MODE == kInvEpiFwd>(pl, tw, a, off, goff, alpha, beta);
    }
    prefetch_data(p + gridDim.x);
    if constexpr (MODE != kInvEpi) {
      __syncthreads();
      xy::row_fwd_b<L, NT>(pl);
      __syncthreads();
      xy::col_fwd_a<L, NT>(pl, tw);  // y forward
      __syncthreads();
      const long long pn = p + gridDim.x;
      if (MODE == kInvEpiFwd && pn < planes) {
        // y forward stage B of this plane with y inverse stage B' of the next
        const long long offn = (pn % B) * N + (pn / B) * L * L;
        xy::col_fwd_b_inv_b_next<L, NT>(pl, tw, a.data + off, a.data + offn);
        loaded = true;
      } else {
        xy::col_fwd_b_to<L, NT>(pl, a.data + off);
      }
    }
  }
}

}  // namespace sep
