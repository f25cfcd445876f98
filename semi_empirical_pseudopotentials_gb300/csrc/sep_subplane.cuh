// sep_subplane.cuh -- the two-pass complex64 Newton step on sub-planes, for
// cubic grids L^3 with L in {96, 112, 128, 160, 192, 256}: xy planes that do
// not fit in one block's shared memory (a 192^2 plane is 295 KB), and planes
// of 96^2 to 128^2, of which one or two fit per SM.
//
// Each 1-D transform is a four-step split (sep_fftpass.cuh): for a length
// L = N1 N2, forward stage A (per residue x1: DFT_N2 over x1 + N1 x2,
// twiddle w_L^(x1 k2)) and stage B (per k2: DFT_N1 over x1 + N1 k2, element
// k2 + N2 k1 left at position k1 + N1 k2); inverse stage B' then A'.  Here y
// is split R x (L / R) (R = 4 for 96 and 128, 8 for the others) and z
// (LZ / 8) x 8.  Stage A of y only couples the L / R rows of one residue, and
// stage B only R adjacent rows, so:
//
//   zy pass (bricks of R adjacent position rows x TX columns x all z):
//     y stage B, z forward, k^2 (filter/init.c:141-142), z inverse,
//     y stage B'  -- the k^2 multiply sees the full (kx, ky, kz) spectrum
//   sub-plane pass (units (grid, z, residue y1): the L / R rows y1 + R j):
//     y stage A', x inverse, psi_j = alpha (T + V psi_{j-1}) + beta psi_{j-1}
//     (filter/hnorm.c:11-39), x forward, y stage A
//
// which is two passes over the grids per Newton step where the line passes
// take four.  A thread of the zy pass holds an R x 8 block (R rows, the 8 z
// of one residue x1 + (LZ / 8) x2): it does the y DFT_Rs and the z stage-A
// DFT_8s of the block in registers, so a brick crosses shared memory twice,
// as a z line pass does.  The sub-plane pass keeps x in the line passes'
// split (N1 x N2) and its sub-planes of 14 to 32 rows (13 to 66 KB) in
// shared memory, several blocks per SM.  Between passes x and y are kept in
// digit-reversed position order (element k2 + N2 k1 of an axis at position
// k1 + N1 k2), z in natural order; the k^2 tables follow the same order.
#pragma once

#include "sep_xypass.cuh"

namespace sep {

// sub-plane pass launch shape per length: threads per block, blocks per SM,
// whether the last stage of a unit runs with the first of the next (fastest
// measured, step pass on 0.5 GB of grids, fraction of the copy bandwidth:
// 96^2 0.83, 112^2 0.74, 128^2 0.84, 160^2 0.75, 192^2 0.84, 256^2 0.75)
template <int L> struct SpTune {
  static constexpr int nt = 128, min_blocks = 4;
  static constexpr bool fuse_next = true;
};
template <> struct SpTune<96> {
  static constexpr int nt = 96, min_blocks = 5;
  static constexpr bool fuse_next = true;
};
template <> struct SpTune<112> {
  static constexpr int nt = 64, min_blocks = 6;
  static constexpr bool fuse_next = true;
};
template <> struct SpTune<128> {  // 32-row sub-planes: the fused column stage spills
  static constexpr int nt = 128, min_blocks = 4;
  static constexpr bool fuse_next = false;
};
template <> struct SpTune<160> {
  static constexpr int nt = 64, min_blocks = 6;
  static constexpr bool fuse_next = true;
};
template <> struct SpTune<192> {
  static constexpr int nt = 96, min_blocks = 4;
  static constexpr bool fuse_next = true;
};
template <> struct SpTune<256> {
  static constexpr int nt = 128, min_blocks = 3;
  static constexpr bool fuse_next = true;
};

// R: the y transform's stage-B radix, done by the zy pass
template <int L> struct SpRows {
  static constexpr int r = 8;
};
template <> struct SpRows<96> {
  static constexpr int r = 4;
};
template <> struct SpRows<128> {
  static constexpr int r = 4;
};

template <int L, int NT> struct SpShape {
  static constexpr int n1 = Split<L>::n1, n2 = Split<L>::n2;  // x
  static constexpr int n1y = SpRows<L>::r, n2y = L / n1y;      // y
  static constexpr int rows = n2y;  // rows of a sub-plane
  static constexpr int rs = L + 1;  // row stride (elements): rows 2 banks apart
  static constexpr int nt = NT;
  static_assert(L % 16 == 0 && n2 <= 16 && n2y <= 32, "sub-plane shapes");
  static constexpr size_t smem_bytes = ((size_t)rows * rs + L) * sizeof(cx<float>);
};

// zy pass shape per length: TX adjacent columns per brick, threads per block,
// blocks per SM.  A thread holds an R x 8 block (about 90 registers for
// R = 4, 160 for R = 8); the brick is LZ x R TX elements (33 to 131 KB).
// Fastest measured (zy pass on 0.5 GB of grids, fraction of the copy
// bandwidth): 96^3 (R = 4) TX 8 0.75, 112^3 TX 8 0.64, 128^3 (R = 4) TX 8
// 0.74, 160^3 TX 4 0.48, 192^3 TX 4 0.51, 256^3 TX 8 0.40.  With R = 8 the
// pass is issue-bound (about 60 FP32 instructions per element for the two
// 8-point y stages and the z transform pair) with 12 warps per SM; R = 4
// needs no multiplies in its y stages and fits 20 warps per SM.
template <int L> struct ZyTune {
  static constexpr int tx = 8, nt = 128, min_blocks = 1;
};
template <> struct ZyTune<160> {
  static constexpr int tx = 4, nt = 128, min_blocks = 1;
};
template <> struct ZyTune<192> {
  static constexpr int tx = 4, nt = 128, min_blocks = 3;
};

template <int L, int LZ, int TX> struct ZyShape {
  static constexpr int r = SpRows<L>::r;  // position rows of a brick
  static constexpr int m = LZ / 8;        // z = x1 + m x2
  static constexpr int nl = r * TX;       // z lines of a brick
  static_assert(LZ % 8 == 0 && L % 8 == 0 && L % TX == 0, "brick shapes");
  static_assert(nl % 16 == 0 && (TX >= 16 || 16 % TX == 0), "brick swizzle");
  static constexpr size_t smem_bytes =
      ((size_t)LZ * nl + LZ + L) * sizeof(cx<float>) + LZ * sizeof(float);
  // element (z position p, line) of the brick.  The line index is XOR-ed with
  // a multiple of TX that changes with p, so that the 16 threads of a
  // half-warp on 16 / TX adjacent p and TX columns (same row) hit 16
  // different bank pairs; 16 adjacent lines of one p stay a permutation of
  // one 16-element group.
  static constexpr int zg = TX >= 16 ? 1 : 16 / TX;  // period of the swizzle in p
  static_assert(m % zg == 0, "positions x1 + m k2 share the swizzle of x1");
  static __device__ __forceinline__ int at(int p, int line) {
    return p * nl + (line ^ ((p % zg) * TX));
  }
};

struct ZyArgs {
  cx<float>* data;
  const cx<float>* tw_y;  // exp(-2 pi i m / L)
  const cx<float>* tw_z;  // exp(-2 pi i m / LZ)
  const float* kx;        // k^2 axis tables, x and y in position order
  const float* ky;
  const float* kz;
  float kcap;
};

namespace sp {

using C = cx<float>;

// y inverse stage A' from global memory: item = column; the N2 positions
// n1 + N1 k2 of a column (row stride N1 L in g) -> inverse DFT_N2 -> natural
// row n1 + N1 n2 = sub-plane row n2.  Two columns' loads go out before either
// is transformed when a thread has two.
template <int L, int NT>
__device__ __forceinline__ void col_inv_a_from(C* pl, const C* __restrict__ g) {
  using S = SpShape<L, NT>;
  constexpr int IB = (L % (2 * NT) == 0 && S::n2y <= 16) ? 2 : 1;
  for (int c0 = threadIdx.x; c0 < L; c0 += IB * NT) {
    C u[IB][S::n2y];
#pragma unroll
    for (int t = 0; t < IB; ++t) {
      const int col = c0 + t * NT;
      if (L % (IB * NT) == 0 || col < L) {
#pragma unroll
        for (int k2 = 0; k2 < S::n2y; ++k2) u[t][k2] = g[(long long)(S::n1y * k2) * L + col];
      }
    }
#pragma unroll
    for (int t = 0; t < IB; ++t) {
      const int col = c0 + t * NT;
      if (L % (IB * NT) == 0 || col < L) {
        Dft<S::n2y, +1, float>::run(u[t]);
#pragma unroll
        for (int n2 = 0; n2 < S::n2y; ++n2) pl[n2 * S::rs + col] = u[t][n2];
      }
    }
  }
}

// y forward stage A to global memory: item = column; sub-plane rows x2
// (natural rows x1 + N1 x2) -> DFT_N2, twiddle w_L^(x1 k2) -> positions
// x1 + N1 k2
template <int L, int NT>
__device__ __forceinline__ void col_fwd_a_to(const C* pl, const C* tw, int x1,
                                             C* __restrict__ g) {
  using S = SpShape<L, NT>;
  for (int col = threadIdx.x; col < L; col += NT) {
    C v[S::n2y];
#pragma unroll
    for (int x2 = 0; x2 < S::n2y; ++x2) v[x2] = pl[x2 * S::rs + col];
    Dft<S::n2y, -1, float>::run(v);
#pragma unroll
    for (int k2 = 1; k2 < S::n2y; ++k2) v[k2] = mul<float>(v[k2], tw[x1 * k2]);
#pragma unroll
    for (int k2 = 0; k2 < S::n2y; ++k2) g[(long long)(S::n1y * k2) * L + col] = v[k2];
  }
}

// y forward stage A of this unit (to gcur, residue x1) and y inverse stage A'
// of the block's next unit (from gnext) in one pass: both have the item
// "column" at the same shared-memory positions, so each thread issues its
// next-unit loads, writes out its current column, then transforms the loaded
// column into the positions it has just read.
template <int L, int NT>
__device__ __forceinline__ void col_fwd_a_inv_a_next(C* pl, const C* tw, int x1,
                                                     C* __restrict__ gcur,
                                                     const C* __restrict__ gnext) {
  using S = SpShape<L, NT>;
  for (int col = threadIdx.x; col < L; col += NT) {
    C u[S::n2y];
#pragma unroll
    for (int k2 = 0; k2 < S::n2y; ++k2) u[k2] = gnext[(long long)(S::n1y * k2) * L + col];
    C v[S::n2y];
#pragma unroll
    for (int x2 = 0; x2 < S::n2y; ++x2) v[x2] = pl[x2 * S::rs + col];
    Dft<S::n2y, -1, float>::run(v);
#pragma unroll
    for (int k2 = 1; k2 < S::n2y; ++k2) v[k2] = mul<float>(v[k2], tw[x1 * k2]);
#pragma unroll
    for (int k2 = 0; k2 < S::n2y; ++k2) gcur[(long long)(S::n1y * k2) * L + col] = v[k2];
    Dft<S::n2y, +1, float>::run(u);
#pragma unroll
    for (int n2 = 0; n2 < S::n2y; ++n2) pl[n2 * S::rs + col] = u[n2];
  }
}

// x inverse stage B' / forward stage B on the sub-plane's rows: item (row,
// k2), adjacent threads on adjacent rows (2 banks apart)
template <int L, int NT> __device__ __forceinline__ void row_inv_b(C* pl, const C* tw) {
  using S = SpShape<L, NT>;
  for (int i = threadIdx.x; i < S::rows * S::n2; i += NT) {
    const int row = i % S::rows, k2 = i / S::rows;
    C* p = pl + row * S::rs + S::n1 * k2;
    C v[S::n1];
#pragma unroll
    for (int k1 = 0; k1 < S::n1; ++k1) v[k1] = p[k1];
    Dft<S::n1, +1, float>::run(v);
#pragma unroll
    for (int n1 = 1; n1 < S::n1; ++n1) v[n1] = mulc<float>(v[n1], tw[n1 * k2]);
#pragma unroll
    for (int n1 = 0; n1 < S::n1; ++n1) p[n1] = v[n1];
  }
}
template <int L, int NT> __device__ __forceinline__ void row_fwd_b(C* pl) {
  using S = SpShape<L, NT>;
  for (int i = threadIdx.x; i < S::rows * S::n2; i += NT) {
    const int row = i % S::rows, k2 = i / S::rows;
    C* p = pl + row * S::rs + S::n1 * k2;
    C w[S::n1];
#pragma unroll
    for (int x1 = 0; x1 < S::n1; ++x1) w[x1] = p[x1];
    Dft<S::n1, -1, float>::run(w);
#pragma unroll
    for (int k1 = 0; k1 < S::n1; ++k1) p[k1] = w[k1];
  }
}

// item (row, n1) of an x stage A: N1 adjacent threads on the N1 adjacent
// elements n1 of a row; for N1 = 8 (16 rows) the two rows of a half-warp are
// 8 apart (16 banks apart)
template <int N1, int ROWS> __device__ __forceinline__ void item_row_n1(int i, int& row, int& n1) {
  n1 = i % N1;
  const int g = i / N1;
  row = (N1 == 8 && ROWS % 16 == 0) ? ((g & ~15) | ((g & 1) << 3) | ((g >> 1) & 7)) : g;
}

// x inverse stage A', the Newton epilogue and (FWD) x forward stage A on the
// sub-plane of residue y1: row j is natural row y1 + N1 j of plane goff
template <int L, int NT, bool FWD>
__device__ __forceinline__ void row_inv_a_epi(C* pl, const C* tw, const PassArgs<float>& a,
                                              long long off, long long goff, int y1,
                                              float alpha, float beta) {
  using S = SpShape<L, NT>;
  const C* __restrict__ pin = a.psi_in ? a.psi_in + off : nullptr;
  const float* __restrict__ pv = a.pot + goff;
  C* __restrict__ pout = a.psi_out + off;
  for (int i = threadIdx.x; i < S::rows * S::n1; i += NT) {
    int row, n1;
    item_row_n1<S::n1, S::rows>(i, row, n1);
    const long long g0 = (long long)(y1 + S::n1y * row) * L + n1;
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
      for (int k2 = 1; k2 < S::n2; ++k2) u[k2] = mul<float>(u[k2], tw[n1 * k2]);
#pragma unroll
      for (int k2 = 0; k2 < S::n2; ++k2) p[S::n1 * k2] = u[k2];
    }
  }
}

// x forward stage A from global memory (natural order), sub-plane residue y1
template <int L, int NT>
__device__ __forceinline__ void row_fwd_a_from(C* pl, const C* tw, int y1,
                                               const C* __restrict__ g) {
  using S = SpShape<L, NT>;
  for (int i = threadIdx.x; i < S::rows * S::n1; i += NT) {
    int row, x1;
    item_row_n1<S::n1, S::rows>(i, row, x1);
    const C* q = g + (long long)(y1 + S::n1y * row) * L + x1;
    C v[S::n2];
#pragma unroll
    for (int x2 = 0; x2 < S::n2; ++x2) v[x2] = q[S::n1 * x2];
    Dft<S::n2, -1, float>::run(v);
#pragma unroll
    for (int k2 = 1; k2 < S::n2; ++k2) v[k2] = mul<float>(v[k2], tw[x1 * k2]);
    C* p = pl + row * S::rs + x1;
#pragma unroll
    for (int k2 = 0; k2 < S::n2; ++k2) p[S::n1 * k2] = v[k2];
  }
}

// L2 prefetch of the N2 rows r0 + N1 j (L elements each) of a plane at g
// (N2 <= 32: one row per lane)
template <int L, int N1, int N2>
__device__ __forceinline__ void prefetch_rows(const void* g, int r0, unsigned esize, int lane) {
  if (lane < N2) {
    const char* p = (const char*)g + (size_t)(r0 + N1 * lane) * L * esize;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(L * esize)
                 : "memory");
  }
}

}  // namespace sp

// Block b walks the units u = b + k gridDim.x of the batch; unit u is
// (grid u % B, residue y1 = (u / B) % 8, plane z = u / 8 B), so the blocks
// running at one time share the planes of V.  MODE as xy_plane_pass.
template <int L, int MODE, int NT = SpTune<L>::nt, int MINB = SpTune<L>::min_blocks,
          bool FUSE = SpTune<L>::fuse_next>
__global__ void __launch_bounds__(NT, MINB) subplane_pass(PassArgs<float> a, int B) {
  using C = cx<float>;
  using S = SpShape<L, NT>;
  extern __shared__ __align__(16) unsigned char sp_smem[];
  C* pl = reinterpret_cast<C*>(sp_smem);
  C* tw = pl + S::rows * S::rs;
  const int tid = threadIdx.x;
  const long long N = (long long)L * L * a.nz;
  const long long units = (long long)B * S::n1y * a.nz;
  const C* src = (MODE == kFwd && a.src) ? a.src : a.data;
  auto geometry = [&](long long u, long long& off, long long& goff, int& y1) {
    const long long r = u / B;
    y1 = (int)(r % S::n1y);
    goff = (r / S::n1y) * L * L;
    off = (u % B) * N + goff;
  };
  for (int m = tid; m < L; m += NT) tw[m] = a.tw[m];  // x and y tables are equal
  float alpha = a.alpha, beta = a.beta;
  if (a.coefs) {
    alpha = a.coefs[2 * a.step];
    beta = a.coefs[2 * a.step + 1];
  }
  bool loaded = false;  // kInvEpiFwd: this unit's first stage ran with the previous unit's last
  for (long long u = blockIdx.x; u < units; u += gridDim.x) {
    long long off, goff;
    int y1;
    geometry(u, off, goff, y1);
    if (MODE != kFwd && tid < 32) {  // psi_{j-1} and V rows of the epilogue
      if (a.psi_in) sp::prefetch_rows<L, S::n1y, S::n2y>(a.psi_in + off, y1, sizeof(C), tid);
      sp::prefetch_rows<L, S::n1y, S::n2y>(a.pot + goff, y1, sizeof(float), tid);
    }
    __syncthreads();  // the previous unit's last stage has read the sub-plane
    if constexpr (MODE == kFwd) {
      sp::row_fwd_a_from<L, NT>(pl, tw, y1, src + off);  // x forward
    } else {
      if (!loaded) {
        sp::col_inv_a_from<L, NT>(pl, a.data + off + (long long)y1 * L);  // y inverse
        __syncthreads();
      }
      sp::row_inv_b<L, NT>(pl, tw);  // x inverse, epilogue (and x forward stage A)
      __syncthreads();
      sp::row_inv_a_epi<L, NT, MODE == kInvEpiFwd>(pl, tw, a, off, goff, y1, alpha, beta);
    }
    const long long un = u + gridDim.x;
    if (MODE != kFwd && tid < 32 && un < units) {
      long long offn, goffn;
      int y1n;
      geometry(un, offn, goffn, y1n);
      sp::prefetch_rows<L, S::n1y, S::n2y>(a.data + offn, y1n, sizeof(C), tid);
    }
    if constexpr (MODE != kInvEpi) {
      __syncthreads();
      sp::row_fwd_b<L, NT>(pl);
      __syncthreads();
      if (FUSE && MODE == kInvEpiFwd && un < units) {
        long long offn, goffn;
        int y1n;
        geometry(un, offn, goffn, y1n);
        sp::col_fwd_a_inv_a_next<L, NT>(pl, tw, y1, a.data + off + (long long)y1 * L,
                                        a.data + offn + (long long)y1n * L);
        loaded = true;
      } else {
        sp::col_fwd_a_to<L, NT>(pl, tw, y1, a.data + off + (long long)y1 * L);  // y forward
      }
    }
  }
}

// One block per brick (TX columns x0.., the R position rows R k2y.., all z,
// grid b) = (blockIdx.x, blockIdx.y, blockIdx.z).  z = x1 + M x2 (M = LZ / 8).
template <int L, int LZ, int TX = ZyTune<L>::tx, int NT = ZyTune<L>::nt,
          int MINB = ZyTune<L>::min_blocks>
__global__ void __launch_bounds__(NT, MINB) zy_pass(ZyArgs a) {
  using C = cx<float>;
  using S = ZyShape<L, LZ, TX>;
  constexpr int M = S::m, NL = S::nl, R = S::r;
  extern __shared__ __align__(16) unsigned char zy_smem[];
  C* br = reinterpret_cast<C*>(zy_smem);
  C* tz = br + LZ * NL;
  C* ty = tz + LZ;
  float* kz = reinterpret_cast<float*>(ty + L);
  const int tid = threadIdx.x;
  for (int m = tid; m < LZ; m += NT) {
    tz[m] = a.tw_z[m];
    kz[m] = a.kz[m];
  }
  for (int m = tid; m < L; m += NT) ty[m] = a.tw_y[m];
  const int x0 = blockIdx.x * TX, k2y = blockIdx.y, y0 = R * k2y;
  const long long zs = (long long)L * L;
  C* __restrict__ g = a.data + (long long)blockIdx.z * zs * LZ + (long long)y0 * L + x0;
  __syncthreads();  // tables

  // item (x, x1): the R rows x the 8 z = x1 + M x2 of column x.  y stage B
  // (DFT_R over the rows: element k2y + (L / R) k1 at row y0 + k1), then z
  // stage A (DFT_8 over x2, twiddle w_LZ^(x1 k2)) -> brick (x1 + M k2, k1 TX + x)
  for (int i = tid; i < TX * M; i += NT) {
    const int x = i % TX, x1 = i / TX;
    C v[R][8];
    const C* p = g + (long long)x1 * zs + x;
#pragma unroll
    for (int x2 = 0; x2 < 8; ++x2)
#pragma unroll
      for (int r = 0; r < R; ++r) v[r][x2] = p[(long long)(M * x2) * zs + (long long)r * L];
#pragma unroll
    for (int x2 = 0; x2 < 8; ++x2) {
      C c[R];
#pragma unroll
      for (int r = 0; r < R; ++r) c[r] = v[r][x2];
      Dft<R, -1, float>::run(c);
#pragma unroll
      for (int k1 = 0; k1 < R; ++k1) v[k1][x2] = c[k1];
    }
    // the item's twiddles (x1 k2 < LZ), read once: the brick stores could alias them
    C t[8];
#pragma unroll
    for (int k2 = 1; k2 < 8; ++k2) t[k2] = tz[x1 * k2];
    // brick (x1 + M k2, k1 TX + x) = q[M NL k2 + (k1 ^ sw) TX]: every position
    // of the item has the swizzle of x1
    C* q = br + x1 * NL + x;
    const int sw = x1 % S::zg;
#pragma unroll
    for (int k1 = 0; k1 < R; ++k1) {
      Dft<8, -1, float>::run(v[k1]);
#pragma unroll
      for (int k2 = 1; k2 < 8; ++k2) v[k1][k2] = mul<float>(v[k1][k2], t[k2]);
      C* qk = q + (k1 ^ sw) * TX;
#pragma unroll
      for (int k2 = 0; k2 < 8; ++k2) qk[k2 * (M * NL)] = v[k1][k2];
    }
  }
  __syncthreads();
  // z stage B (DFT_M over x1: element kz = k2 + 8 k1), k^2 (filter/init.c:
  // 141-142: (kx + ky) + kz, capped), z inverse stage B' (inverse DFT_M,
  // conjugate twiddle): item (line, k2)
  for (int i = tid; i < NL * 8; i += NT) {
    const int line = i % NL, k2 = i / NL;
    C* q = br + k2 * (M * NL);
    int ls[S::zg];  // the line's swizzled index for each residue of x1
#pragma unroll
    for (int j = 0; j < S::zg; ++j) ls[j] = line ^ (j * TX);
    C w[M];
#pragma unroll
    for (int x1 = 0; x1 < M; ++x1) w[x1] = q[x1 * NL + ls[x1 % S::zg]];
    Dft<M, -1, float>::run(w);
    const float kxy = a.kx[x0 + line % TX] + a.ky[y0 + line / TX];
#pragma unroll
    for (int k1 = 0; k1 < M; ++k1) {
      float k = kxy + kz[k2 + 8 * k1];
      k = (k > a.kcap) ? a.kcap : k;
      w[k1] = scale<float>(w[k1], k);
    }
    Dft<M, +1, float>::run(w);
#pragma unroll
    for (int n1 = 1; n1 < M; ++n1) w[n1] = mulc<float>(w[n1], tz[n1 * k2]);  // n1 k2 < LZ
#pragma unroll
    for (int n1 = 0; n1 < M; ++n1) q[n1 * NL + ls[n1 % S::zg]] = w[n1];
  }
  __syncthreads();
  // item (x, n1): z inverse stage A' (inverse DFT_8 over k2 per row: natural
  // z = n1 + M n2), then y inverse stage B' (inverse DFT_R over the rows,
  // conjugate twiddle w_L^(ny k2y)) -> rows y0 + ny
  C t[R];  // the brick's y twiddles (ny k2y < L)
#pragma unroll
  for (int ny = 1; ny < R; ++ny) t[ny] = ty[ny * k2y];
  for (int i = tid; i < TX * M; i += NT) {
    const int x = i % TX, n1 = i / TX;
    const C* q = br + n1 * NL + x;
    const int sw = n1 % S::zg;
    C u[R][8];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const C* qr = q + (r ^ sw) * TX;
#pragma unroll
      for (int k2 = 0; k2 < 8; ++k2) u[r][k2] = qr[k2 * (M * NL)];
      Dft<8, +1, float>::run(u[r]);
    }
    C* p = g + (long long)n1 * zs + x;
#pragma unroll
    for (int n2 = 0; n2 < 8; ++n2) {
      C c[R];
#pragma unroll
      for (int r = 0; r < R; ++r) c[r] = u[r][n2];
      Dft<R, +1, float>::run(c);
#pragma unroll
      for (int ny = 1; ny < R; ++ny) c[ny] = mulc<float>(c[ny], t[ny]);
#pragma unroll
      for (int ny = 0; ny < R; ++ny) p[(long long)(M * n2) * zs + (long long)ny * L] = c[ny];
    }
  }
}

}  // namespace sep
