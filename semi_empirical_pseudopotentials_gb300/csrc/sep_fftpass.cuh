// sep_fftpass.cuh -- one axis of the 3-D FFT Hamiltonian apply, fused with
// the pointwise work that the reference does in separate loops.
//
// Reference data path (filter/hamiltonian.c:27-44, filter/hnorm.c:11-39):
//   fftwpsi <- psi; FFT forward; fftwpsi *= ksqr; FFT backward;
//   phi <- fftwpsi + potl * psi;   (hnorm) psin = dE_1 phi - (2 + z + Vmin dE_1) psim1
// Here a batch of B complex grids [B][nz][ny][nx] (x fastest, as the
// reference's jxyz = nx (ny jz + jy) + jx) goes through line passes:
//   X forward  |  Y forward  |  Z forward * k^2 * Z inverse  |  Y inverse  |
//   X inverse + epilogue (V psi, affine) [+ X forward of the result]
// so that no pointwise loop touches HBM on its own.
//
// A line of length L = N1 * N2 is transformed by the four-step split
//   x = x1 + N1 x2, k = k2 + N2 k1:
//   stage A: per x1, DFT_N2 over x2, twiddle w_L^(S x1 k2)  -> shared memory
//   stage B: per k2, DFT_N1 over x1                       -> X[k2 + N2 k1]
// and the inverse by the mirrored split (input indexed k2 + N2 k1, output
// n1 + N1 n2), which consumes exactly the register layout that stage B
// produced; a forward/inverse pair therefore needs two shared-memory
// exchanges and no redistribution.
#pragma once

#include "sep_dft.cuh"

namespace sep {

enum PassMode : int {
  kFwd = 0,         // forward transform along the axis
  kInv = 1,         // backward (unnormalised) transform along the axis
  kFwdKInv = 2,     // forward, multiply by the k^2 table, backward (z axis)
  kInvEpi = 3,      // backward, then out = alpha (u + V psi_in) + beta psi_in (x axis)
  kInvEpiFwd = 4,   // kInvEpi, then forward transform of out back into data (x axis)
  kFwdPInv = 5,     // forward, multiply by 1 / (pc_a k^2 + pc_b), backward (z axis)
};

template <typename T> struct PassArgs {
  cx<T>* data;            // transformed in place
  const cx<T>* src;       // kFwd: read from here instead of data when not null
  const cx<T>* psi_in;    // epilogue: previous state (null: no V and no beta term)
  const cx<T>* extra;     // epilogue: added to T psi before the alpha scale (null: none)
  cx<T>* psi_out;         // epilogue: new state
  const T* pot;           // epilogue: V on the grid (shared by the batch)
  const cx<T>* tw;        // exp(-2 pi i m / L), m < L, for this axis
  const T* kx;            // k^2 axis tables, pre-scaled by 1/N (filter/init.c:125-135)
  const T* ky;
  const T* kz;
  T kcap;                 // Ekinmax / N (filter/init.c:137-143)
  T pc_a, pc_b;           // kFwdPInv: multiply by 1 / (pc_a k + pc_b) (kinetic preconditioner)
  T alpha, beta;          // epilogue scalars, unless coefs is set
  const T* coefs;         // epilogue: device (alpha, beta) pairs, entry `step`
  int step;
  long long nbatch_lines; // x axis: B * ny * nz
  int nx, ny, nz;
};

// line-length factorisations L = N1 * N2 (N1 >= 8 where possible so that x
// lines load in 128-byte segments)
template <int L> struct Split;
#define SEP_SPLIT(L_, A_, B_) \
  template <> struct Split<L_> { static constexpr int n1 = A_, n2 = B_; };
SEP_SPLIT(14, 2, 7)
SEP_SPLIT(16, 4, 4)
SEP_SPLIT(18, 6, 3)
SEP_SPLIT(20, 4, 5)
SEP_SPLIT(24, 4, 6)
SEP_SPLIT(32, 8, 4)
SEP_SPLIT(36, 6, 6)
SEP_SPLIT(40, 8, 5)
SEP_SPLIT(48, 8, 6)
SEP_SPLIT(56, 8, 7)
SEP_SPLIT(64, 8, 8)
SEP_SPLIT(72, 8, 9)
SEP_SPLIT(80, 8, 10)
SEP_SPLIT(96, 8, 12)
SEP_SPLIT(112, 8, 14)
SEP_SPLIT(128, 8, 16)
SEP_SPLIT(160, 10, 16)
SEP_SPLIT(192, 12, 16)
SEP_SPLIT(256, 16, 16)
#undef SEP_SPLIT

// lines handled by one block: x axis -> whole lines, y/z -> adjacent x.
// Two shapes per pass (V = 0, 1); the autotuner picks one per context.
template <typename T, int L, int AXIS, int V = 0> struct Tile {
  static constexpr int n1 = Split<L>::n1, n2 = Split<L>::n2;
  static constexpr int nmin = n1 < n2 ? n1 : n2;
  // V0 -- y/z: 16 adjacent x (256 B of complex128, 128 B of complex64 per
  // row); x: about 128 threads per block.
  // V1 -- y/z: 8 adjacent x for complex128, 32 for complex64; x: about 256
  // threads per block.
  static constexpr int yz_lines = (V == 0) ? 16 : (sizeof(T) == 8 ? 8 : 32);
  static constexpr int x_threads = (V == 0) ? 128 : 256;
  static constexpr int tl_raw =
      (AXIS == 0) ? ((x_threads / nmin) > 0 ? x_threads / nmin : 1) : yz_lines;
  // keep the exchange buffer under 40 KB of static shared memory
  static constexpr int bytes_per_line = L * (int)sizeof(cx<T>) + 32 * (int)sizeof(cx<T>);
  static constexpr int tl_cap = (40 * 1024) / bytes_per_line;
  static constexpr int pow2_floor(int v) { return v >= 2 ? 2 * pow2_floor(v / 2) : 1; }
  static constexpr int tl = pow2_floor(tl_raw < tl_cap ? tl_raw : (tl_cap > 0 ? tl_cap : 1));
  static constexpr int nt = tl * nmin;
};

template <typename T, int L, int AXIS, int MODE, int V = 0>
__global__ void __launch_bounds__(Tile<T, L, AXIS, V>::nt)
line_pass(PassArgs<T> a) {
  using C = cx<T>;
  constexpr int N1 = Split<L>::n1, N2 = Split<L>::n2;
  constexpr int TL = Tile<T, L, AXIS, V>::tl;
  constexpr int NT = Tile<T, L, AXIS, V>::nt;
  constexpr int NA = TL * N1, NB = TL * N2;
  constexpr int IA = (NA + NT - 1) / NT, IB = (NB + NT - 1) / NT;
  constexpr int PAD = (AXIS == 0) ? 1 : 0;
  constexpr int SROW = N1 + PAD;  // x axis: [line][b][a + pad]
  // x axis: lines start 8 elements off a multiple of 16 so that the lines a
  // warp touches at once fall on different banks
  constexpr int LSTR =
      (AXIS == 0) ? N2 * SROW + ((8 - (N2 * SROW) % 16) + 16) % 16 : N2 * SROW;

  __shared__ C sh[(AXIS == 0) ? TL * LSTR : TL * N2 * SROW];
  __shared__ C tws[L];

  const int tid = threadIdx.x;
  for (int m = tid; m < L; m += NT) tws[m] = a.tw[m];

  // shared index of element (line, a in [0,N1), b in [0,N2))
  auto sidx = [&](int line, int ia, int ib) -> int {
    if constexpr (AXIS == 0) return line * LSTR + ib * SROW + ia;
    else return (ia * N2 + ib) * TL + line;
  };

  // geometry of this block's lines
  const long long N = (long long)a.nx * a.ny * a.nz;
  long long base0;   // offset of line 0 of this block
  long long lstride; // offset between lines of this block
  long long es;      // element stride along the line
  int nvalid;        // lines of this block inside the grid
  int yk = 0, xk0 = 0;
  if constexpr (AXIS == 0) {
    const long long g0 = (long long)blockIdx.x * TL;
    base0 = g0 * a.nx;
    lstride = a.nx;
    es = 1;
    long long rem = a.nbatch_lines - g0;
    nvalid = rem < TL ? (int)rem : TL;
  } else {
    const int x0 = blockIdx.x * TL;
    const long long b = blockIdx.z;
    xk0 = x0;
    if constexpr (AXIS == 1) {
      base0 = b * N + (long long)blockIdx.y * a.nx * a.ny + x0;
      es = a.nx;
    } else {
      yk = blockIdx.y;
      base0 = b * N + (long long)blockIdx.y * a.nx + x0;
      es = (long long)a.nx * a.ny;
    }
    lstride = 1;
    nvalid = (a.nx - x0) < TL ? (a.nx - x0) : TL;
  }

  auto itemA = [&](int i, int& line, int& ia) {
    if constexpr (AXIS == 0) { line = i / N1; ia = i % N1; }
    else { line = i % TL; ia = i / TL; }
  };
  auto itemB = [&](int i, int& line, int& ib) {
    if constexpr (AXIS == 0) { line = i / N2; ib = i % N2; }
    else { line = i % TL; ib = i / TL; }
  };

  C va[IA][N2];  // A-items: element (x1 + N1 x2) or after inverse (n1 + N1 n2)
  C vb[IB][N1];  // B-items: element (k2 + N2 k1)

  // ---- forward from A layout (registers va) to B layout (registers vb)
  auto forward_from_va = [&]() {
#pragma unroll
    for (int r = 0; r < IA; ++r) {
      const int i = tid + r * NT;
      if (NA % NT == 0 || i < NA) {
        int line, x1;
        itemA(i, line, x1);
        Dft<N2, -1, T>::run(va[r]);
#pragma unroll
        for (int k2 = 1; k2 < N2; ++k2) va[r][k2] = mul<T>(va[r][k2], tws[(x1 * k2) % L]);
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) sh[sidx(line, x1, k2)] = va[r][k2];
      }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < IB; ++r) {
      const int i = tid + r * NT;
      if (NB % NT == 0 || i < NB) {
        int line, k2;
        itemB(i, line, k2);
#pragma unroll
        for (int x1 = 0; x1 < N1; ++x1) vb[r][x1] = sh[sidx(line, x1, k2)];
        Dft<N1, -1, T>::run(vb[r]);
      }
    }
  };

  // ---- inverse from B layout (vb) to A layout (va)
  auto inverse_from_vb = [&]() {
#pragma unroll
    for (int r = 0; r < IB; ++r) {
      const int i = tid + r * NT;
      if (NB % NT == 0 || i < NB) {
        int line, k2;
        itemB(i, line, k2);
        Dft<N1, +1, T>::run(vb[r]);
#pragma unroll
        for (int n1 = 1; n1 < N1; ++n1) vb[r][n1] = mulc<T>(vb[r][n1], tws[(n1 * k2) % L]);
#pragma unroll
        for (int n1 = 0; n1 < N1; ++n1) sh[sidx(line, n1, k2)] = vb[r][n1];
      }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < IA; ++r) {
      const int i = tid + r * NT;
      if (NA % NT == 0 || i < NA) {
        int line, n1;
        itemA(i, line, n1);
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) va[r][k2] = sh[sidx(line, n1, k2)];
        Dft<N2, +1, T>::run(va[r]);
      }
    }
  };

  auto loadA = [&](const C* src) {
#pragma unroll
    for (int r = 0; r < IA; ++r) {
      const int i = tid + r * NT;
      int line, x1;
      itemA(i, line, x1);
      const bool ok = (NA % NT == 0 || i < NA) && line < nvalid;
      const C* p = src + base0 + line * lstride;
#pragma unroll
      for (int x2 = 0; x2 < N2; ++x2)
        va[r][x2] = ok ? p[(long long)(x1 + N1 * x2) * es] : mk<T>(T(0), T(0));
    }
  };
  auto storeA = [&](C* dst) {
#pragma unroll
    for (int r = 0; r < IA; ++r) {
      const int i = tid + r * NT;
      int line, n1;
      itemA(i, line, n1);
      if ((NA % NT == 0 || i < NA) && line < nvalid) {
        C* p = dst + base0 + line * lstride;
#pragma unroll
        for (int n2 = 0; n2 < N2; ++n2) p[(long long)(n1 + N1 * n2) * es] = va[r][n2];
      }
    }
  };
  auto loadB = [&](const C* src) {
#pragma unroll
    for (int r = 0; r < IB; ++r) {
      const int i = tid + r * NT;
      int line, k2;
      itemB(i, line, k2);
      const bool ok = (NB % NT == 0 || i < NB) && line < nvalid;
      const C* p = src + base0 + line * lstride;
#pragma unroll
      for (int k1 = 0; k1 < N1; ++k1)
        vb[r][k1] = ok ? p[(long long)(k2 + N2 * k1) * es] : mk<T>(T(0), T(0));
    }
  };
  auto storeB = [&](C* dst) {
#pragma unroll
    for (int r = 0; r < IB; ++r) {
      const int i = tid + r * NT;
      int line, k2;
      itemB(i, line, k2);
      if ((NB % NT == 0 || i < NB) && line < nvalid) {
        C* p = dst + base0 + line * lstride;
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) p[(long long)(k2 + N2 * k1) * es] = vb[r][k1];
      }
    }
  };

  if constexpr (MODE == kFwd) {
    loadA(a.src ? a.src : a.data);
    __syncthreads();  // twiddle table
    forward_from_va();
    storeB(a.data);
  } else if constexpr (MODE == kInv) {
    loadB(a.data);
    __syncthreads();
    inverse_from_vb();
    storeA(a.data);
  } else if constexpr (MODE == kFwdKInv || MODE == kFwdPInv) {
    static_assert(AXIS == 2, "k^2 multiply is fused into the z pass");
    constexpr bool PRECOND = MODE == kFwdPInv;
    loadA(a.data);
    __syncthreads();
    forward_from_va();
    // k^2 (filter/init.c:141-142): (kx + ky) + kz, capped
#pragma unroll
    for (int r = 0; r < IB; ++r) {
      const int i = tid + r * NT;
      int line, k2;
      itemB(i, line, k2);
      const int jx = xk0 + (line < nvalid ? line : 0);
      const T kxy = a.kx[jx] + a.ky[yk];
#pragma unroll
      for (int k1 = 0; k1 < N1; ++k1) {
        T k = kxy + a.kz[k2 + N2 * k1];
        k = (k > a.kcap) ? a.kcap : k;
        if constexpr (PRECOND) k = T(1) / (a.pc_a * k + a.pc_b);
        vb[r][k1] = scale<T>(vb[r][k1], k);
      }
    }
    __syncthreads();  // the exchange buffer is reused
    inverse_from_vb();
    storeA(a.data);
  } else {
    static_assert(AXIS == 0, "the epilogue runs on the x pass");
    loadB(a.data);
    __syncthreads();
    inverse_from_vb();
    T alpha = a.alpha, beta = a.beta;
    if (a.coefs) {
      alpha = a.coefs[2 * a.step];
      beta = a.coefs[2 * a.step + 1];
    }
    // epilogue on A layout: element n1 + N1 n2 of each line
#pragma unroll
    for (int r = 0; r < IA; ++r) {
      const int i = tid + r * NT;
      int line, n1;
      itemA(i, line, n1);
      if ((NA % NT == 0 || i < NA) && line < nvalid) {
        const long long lb = base0 + line * lstride;          // offset in the batch array
        const long long gb = lb % N;                          // offset in one grid
        // psi_{j-1}, the extra term and V never alias psi_j: the loads of all
        // n2 can go out ahead of the stores
        const C* __restrict__ pin = a.psi_in ? a.psi_in + lb : nullptr;
        const C* __restrict__ pex = a.extra ? a.extra + lb : nullptr;
        C* __restrict__ pout = a.psi_out + lb;
        const T* __restrict__ pv = a.pot + gb;
#pragma unroll
        for (int n2 = 0; n2 < N2; ++n2) {
          const int x = n1 + N1 * n2;
          const C p = pin ? pin[x] : mk<T>(T(0), T(0));
          const T v = pv[x];
          C u = va[r][n2];
          if (pex) u = mk<T>(u.x + pex[x].x, u.y + pex[x].y);
          const C o = newton_epi<T>(u, v, p, alpha, beta);
          pout[x] = o;
          va[r][n2] = o;
        }
      }
    }
    if constexpr (MODE == kInvEpiFwd) {
      __syncthreads();  // the exchange buffer is reused
      forward_from_va();
      storeB(a.data);
    }
  }
}

}  // namespace sep
