// sep_engine.cuh -- device-side building blocks of the filter path.
//
// Layout in HBM (one context = one grid + one potential):
//   complex state batch  [B][nz][ny][nx]  (cx<T>, x fastest)
//   two real states travel in one complex grid: state 2b in the real part,
//   state 2b+1 in the imaginary part.  H of filter/hamiltonian.c is a real
//   operator (real V, even k^2), so H(a + i b) = H a + i H b and one complex
//   transform applies H to two states.
//   real state blocks    [M][N] (T), state-major like the reference's psitot
#pragma once

#include <cuda_runtime.h>

#include "sep_dd.cuh"
#include "sep_fftpass.cuh"

namespace sep {

// device tables of one grid in one precision (double, float, or ddf: the
// double-float form of the FP64 passes, sep_dd.cuh)
template <typename T> struct GridDev {
  int nx = 0, ny = 0, nz = 0;
  long long n = 0;
  cx<T>* tw[3] = {nullptr, nullptr, nullptr};  // x, y, z twiddles
  T* kx = nullptr;
  T* ky = nullptr;
  T* kz = nullptr;
  T kcap = 0;
  T* pot = nullptr;
  int variant[5] = {0, 0, 0, 0, 0};  // tile shape per pass kind (autotuned)
  // k^2 axis tables of x and y in the fused step's digit-reversed position
  // order (complex64 grids with a fused step; else null)
  T* kxr = nullptr;
  T* kyr = nullptr;
};

// pass kinds of a Newton step: x forward, y forward, z forward*k^2*inverse,
// y inverse, x inverse + epilogue (+ forward)
inline int pass_kind(int axis, int mode) {
  if (axis == 0) return mode == kFwd ? 0 : 4;
  if (axis == 1) return mode == kFwd ? 1 : 3;
  return 2;
}

// lengths with a compiled line pass
bool length_supported(int L);

// SMs of the current device (152 if the query fails), read once per process
inline int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0, v = 0;
    n = (cudaGetDevice(&dev) == cudaSuccess &&
         cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0)
            ? v
            : 152;
  }
  return n;
}

// buffers and scalars of one pass
template <typename T> struct PassIO {
  cx<T>* data = nullptr;
  const cx<T>* src = nullptr;
  const cx<T>* psi_in = nullptr;
  const cx<T>* extra = nullptr;  // x-pass epilogue: added to T psi (the spin-orbit term)
  cx<T>* psi_out = nullptr;
  T alpha = T(1), beta = T(0);
  const T* coefs = nullptr;  // device (alpha, beta) per step
  int step = 0;
  int variant = -1;          // -1: the grid's autotuned choice
  T pc_a = T(0), pc_b = T(0);  // z pass: 1 / (pc_a k + pc_b) instead of k when pc_a != 0
};

// One line pass over a batch of B grids (see sep_fftpass.cuh for modes).
template <typename T>
cudaError_t run_pass(int axis, int mode, const GridDev<T>& g, const PassIO<T>& io, int B,
                     cudaStream_t s);

// Fused two-pass Newton step of complex64 grids with nx = ny: the xy pass
// (modes kFwd, kInvEpi, kInvEpiFwd) and the z pass of that step.  Cubic grids
// with nx in {96, 112, 128, 160, 192, 256} take the sub-plane form: the xy pass works
// on sub-planes and the z pass also does the y transform's R-point stage
// (sep_subplane.cuh).  Other grids with nx in {40, ..., 128} take the plane
// form: the xy pass works on whole z-planes (sep_xypass.cuh) and the z pass is
// the z line pass.  Between the two passes x and y are kept in digit-reversed
// position order: element k = k2 + N2 k1 of an axis of length L = N1 N2 at
// position k1 + N1 k2, N1 = xy_split_n1(nx) for x and xy_split_y(nx, nz) for
// y (0: no fused step).
int xy_split_n1(int L);
int xy_split_y(int nx, int nz);
bool xy_supported(const GridDev<float>& g);
cudaError_t xy_prepare(const GridDev<float>& g);  // before any stream capture
cudaError_t run_xy_pass(int mode, const GridDev<float>& g, const PassIO<float>& io, int B,
                        cudaStream_t s);
cudaError_t run_xy_zpass(const GridDev<float>& g, const PassIO<float>& io, int B,
                         cudaStream_t s);
// the sub-plane form (sep_sp_f32.cu)
bool subplane_length(int L);
int subplane_rows(int L);  // R
cudaError_t subplane_prepare(int L);
cudaError_t subplane_launch(int mode, const PassArgs<float>& a, int B, cudaStream_t s);
cudaError_t zy_launch(const GridDev<float>& g, cx<float>* data, int B, cudaStream_t s);

// out = alpha (T x + V y) + beta y for B complex grids; y may be null (out = alpha T x).
// scratch: B * n complex; out may not alias x.
template <typename T>
cudaError_t apply_txvy(const GridDev<T>& g, const cx<T>* x, const cx<T>* y, cx<T>* out,
                       cx<T>* scratch, int B, T alpha, T beta, cudaStream_t s);

// Kinetic preconditioner on B complex grids: out = (T + shift)^-1 in, T the
// capped kinetic operator of the grid.  scratch: B * n complex.
template <typename T>
cudaError_t apply_precond(const GridDev<T>& g, const cx<T>* in, cx<T>* out, cx<T>* scratch,
                          int B, double shift, cudaStream_t s);

// H (or alpha H + beta) applied to B complex grids: out = alpha (T in + V in) + beta in.
// scratch: B * n complex.  out may not alias in.
template <typename T>
cudaError_t apply_h(const GridDev<T>& g, const cx<T>* in, cx<T>* out, cx<T>* scratch, int B,
                    T alpha, T beta, cudaStream_t s);

}  // namespace sep
