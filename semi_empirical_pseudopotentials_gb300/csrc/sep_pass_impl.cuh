// sep_pass_impl.cuh -- instantiation and launch of the line passes for one
// precision (included by sep_pass_f64.cu and sep_pass_f32.cu with SEP_T set).
#pragma once

#include <type_traits>

#include "sep_engine.cuh"

namespace sep {

template <typename T, int L, int AXIS, int MODE, int V>
cudaError_t launch_one(const PassArgs<T>& a, int B, cudaStream_t s) {
  constexpr int TL = Tile<T, L, AXIS, V>::tl;
  constexpr int NT = Tile<T, L, AXIS, V>::nt;
  dim3 grid;
  if (AXIS == 0) {
    long long blocks = (a.nbatch_lines + TL - 1) / TL;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
    grid = dim3((unsigned)blocks, 1, 1);
  } else {
    const int other = (AXIS == 1) ? a.nz : a.ny;
    if (other > 65535 || B > 65535) return cudaErrorInvalidValue;
    grid = dim3((unsigned)((a.nx + TL - 1) / TL), (unsigned)other, (unsigned)B);
  }
  line_pass<T, L, AXIS, MODE, V><<<grid, NT, 0, s>>>(a);
  return cudaGetLastError();
}

template <typename T, int L, int V>
cudaError_t launch_len(int axis, int mode, const PassArgs<T>& a, int B, cudaStream_t s) {
  if (axis == 0) {
    if (mode == kFwd) return launch_one<T, L, 0, kFwd, V>(a, B, s);
    if (mode == kInvEpi) return launch_one<T, L, 0, kInvEpi, V>(a, B, s);
    if (mode == kInvEpiFwd) return launch_one<T, L, 0, kInvEpiFwd, V>(a, B, s);
  } else if (axis == 1) {
    if (mode == kFwd) return launch_one<T, L, 1, kFwd, V>(a, B, s);
    if (mode == kInv) return launch_one<T, L, 1, kInv, V>(a, B, s);
  } else if (axis == 2) {
    if (mode == kFwdKInv) return launch_one<T, L, 2, kFwdKInv, V>(a, B, s);
    if constexpr (std::is_same<T, double>::value)  // the preconditioner of the FP64 refinement
      if (mode == kFwdPInv) return launch_one<T, L, 2, kFwdPInv, V>(a, B, s);
  }
  return cudaErrorInvalidValue;
}

// launch of one tile variant; each (precision, variant) lives in its own
// translation unit so they compile in parallel
template <typename T, int V>
cudaError_t launch_variant(int axis, int mode, int L, const PassArgs<T>& a, int B,
                           cudaStream_t s);

#ifdef SEP_V
template <>
cudaError_t launch_variant<SEP_T, SEP_V>(int axis, int mode, int L, const PassArgs<SEP_T>& a,
                                         int B, cudaStream_t s) {
  switch (L) {
#define SEP_CASE(LL) \
  case LL: return launch_len<SEP_T, LL, SEP_V>(axis, mode, a, B, s);
    SEP_CASE(14) SEP_CASE(16) SEP_CASE(18) SEP_CASE(20) SEP_CASE(24) SEP_CASE(32) SEP_CASE(36)
    SEP_CASE(40) SEP_CASE(48) SEP_CASE(56) SEP_CASE(64) SEP_CASE(72) SEP_CASE(80)
    SEP_CASE(96) SEP_CASE(112) SEP_CASE(128) SEP_CASE(160) SEP_CASE(192) SEP_CASE(256)
#undef SEP_CASE
    default: return cudaErrorInvalidValue;
  }
}
#endif

// The double-float passes (SEP_T = ddf, tile shape 0) compile in four
// translation units of a few lengths each: their kernels unroll the
// error-free operations into long straight-line code, and one unit with
// every length took minutes.
#define SEP_DD_GROUP0(X) X(14) X(16) X(18) X(20) X(24) X(32) X(36)
#define SEP_DD_GROUP1(X) X(40) X(48) X(56) X(64) X(72) X(80)
#define SEP_DD_GROUP2(X) X(96) X(112) X(128)
#define SEP_DD_GROUP3(X) X(160) X(192) X(256)
template <int G>
cudaError_t launch_dd_group(int axis, int mode, int L, const PassArgs<ddf>& a, int B,
                            cudaStream_t s);

#ifdef SEP_DD_G
template <>
cudaError_t launch_dd_group<SEP_DD_G>(int axis, int mode, int L, const PassArgs<ddf>& a, int B,
                                      cudaStream_t s) {
  switch (L) {
#define SEP_CASE(LL) \
  case LL: return launch_len<ddf, LL, 0>(axis, mode, a, B, s);
    SEP_DD_LIST(SEP_CASE)
#undef SEP_CASE
    default: return cudaErrorInvalidValue;
  }
}
#endif

#ifdef SEP_DISPATCH
template <>
cudaError_t run_pass<SEP_T>(int axis, int mode, const GridDev<SEP_T>& g,
                            const PassIO<SEP_T>& io, int B, cudaStream_t s) {
  PassArgs<SEP_T> a;
  a.data = io.data;
  a.src = io.src;
  a.psi_in = io.psi_in;
  a.extra = io.extra;
  a.psi_out = io.psi_out;
  a.coefs = io.coefs;
  a.step = io.step;
  a.pot = g.pot;
  a.tw = g.tw[axis];
  a.kx = g.kx;
  a.ky = g.ky;
  a.kz = g.kz;
  a.kcap = g.kcap;
  a.alpha = io.alpha;
  a.beta = io.beta;
  a.pc_a = io.pc_a;
  a.pc_b = io.pc_b;
  a.nbatch_lines = (long long)B * g.ny * g.nz;
  a.nx = g.nx;
  a.ny = g.ny;
  a.nz = g.nz;
  const int L = axis == 0 ? g.nx : (axis == 1 ? g.ny : g.nz);
#ifdef SEP_IS_DD  // double-float: tile shape 0 only, the lengths in four units
#define SEP_DD_IN(LL) || L == LL
  if (false SEP_DD_GROUP0(SEP_DD_IN)) return launch_dd_group<0>(axis, mode, L, a, B, s);
  if (false SEP_DD_GROUP1(SEP_DD_IN)) return launch_dd_group<1>(axis, mode, L, a, B, s);
  if (false SEP_DD_GROUP2(SEP_DD_IN)) return launch_dd_group<2>(axis, mode, L, a, B, s);
  if (false SEP_DD_GROUP3(SEP_DD_IN)) return launch_dd_group<3>(axis, mode, L, a, B, s);
#undef SEP_DD_IN
  return cudaErrorInvalidValue;
#else
  const int v = io.variant >= 0 ? io.variant : g.variant[pass_kind(axis, mode)];
  if (v == 1) return launch_variant<SEP_T, 1>(axis, mode, L, a, B, s);
  return launch_variant<SEP_T, 0>(axis, mode, L, a, B, s);
#endif
}

template <>
cudaError_t apply_txvy<SEP_T>(const GridDev<SEP_T>& g, const cx<SEP_T>* x, const cx<SEP_T>* y,
                              cx<SEP_T>* out, cx<SEP_T>* scratch, int B, SEP_T alpha,
                              SEP_T beta, cudaStream_t s) {
  cudaError_t e;
  PassIO<SEP_T> io;
  io.data = scratch;
  io.src = x;
  if ((e = run_pass<SEP_T>(0, kFwd, g, io, B, s))) return e;
  io.src = nullptr;
  if ((e = run_pass<SEP_T>(1, kFwd, g, io, B, s))) return e;
  if ((e = run_pass<SEP_T>(2, kFwdKInv, g, io, B, s))) return e;
  if ((e = run_pass<SEP_T>(1, kInv, g, io, B, s))) return e;
  io.psi_in = y;
  io.psi_out = out;
  io.alpha = alpha;
  io.beta = beta;
  return run_pass<SEP_T>(0, kInvEpi, g, io, B, s);
}

template <>
cudaError_t apply_h<SEP_T>(const GridDev<SEP_T>& g, const cx<SEP_T>* in, cx<SEP_T>* out,
                           cx<SEP_T>* scratch, int B, SEP_T alpha, SEP_T beta,
                           cudaStream_t s) {
  cudaError_t e;
  PassIO<SEP_T> io;
  io.data = scratch;
  io.src = in;
  if ((e = run_pass<SEP_T>(0, kFwd, g, io, B, s))) return e;
  io.src = nullptr;
  if ((e = run_pass<SEP_T>(1, kFwd, g, io, B, s))) return e;
  if ((e = run_pass<SEP_T>(2, kFwdKInv, g, io, B, s))) return e;
  if ((e = run_pass<SEP_T>(1, kInv, g, io, B, s))) return e;
  io.psi_in = in;
  io.psi_out = out;
  io.alpha = alpha;
  io.beta = beta;
  return run_pass<SEP_T>(0, kInvEpi, g, io, B, s);
}

template <>
cudaError_t apply_precond<SEP_T>(const GridDev<SEP_T>& g, const cx<SEP_T>* in, cx<SEP_T>* out,
                                 cx<SEP_T>* scratch, int B, double shift, cudaStream_t s) {
  // the k tables carry 1/N and the transform pair a factor N: multiplying by
  // 1 / (N^2 k + N shift) leaves (T + shift)^-1
  cudaError_t e;
  const double nn = (double)g.n;
  PassIO<SEP_T> io;
  io.data = scratch;
  io.src = in;
  if ((e = run_pass<SEP_T>(0, kFwd, g, io, B, s))) return e;
  io.src = nullptr;
  if ((e = run_pass<SEP_T>(1, kFwd, g, io, B, s))) return e;
  io.pc_a = (SEP_T)(nn * nn);
  io.pc_b = (SEP_T)(nn * shift);
  if ((e = run_pass<SEP_T>(2, kFwdPInv, g, io, B, s))) return e;
  io.pc_a = io.pc_b = (SEP_T)0;
  if ((e = run_pass<SEP_T>(1, kInv, g, io, B, s))) return e;
  io.psi_in = nullptr;  // epilogue with no V term: out = the transformed grid
  io.psi_out = out;
  io.alpha = (SEP_T)1;
  io.beta = (SEP_T)0;
  return run_pass<SEP_T>(0, kInvEpi, g, io, B, s);
}

#endif  // SEP_DISPATCH

}  // namespace sep
