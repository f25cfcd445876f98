// sep_xy_f32.cu -- launch of the fused xy plane pass (complex64).
#include "sep_engine.cuh"
#include "sep_xypass.cuh"

namespace sep {

namespace {

template <int L> constexpr size_t xy_smem() {
  return (size_t)L * (L + 1) * sizeof(cx<float>) + 2 * (size_t)L * sizeof(cx<float>);
}

template <int L, int MODE>
cudaError_t launch_xy(const PassArgs<float>& a, int B, cudaStream_t s) {
  if (a.nz > 65535 || B < 1) return cudaErrorInvalidValue;
  xy_plane_pass<L, L, MODE><<<dim3((unsigned)B, (unsigned)a.nz), kXyThreads, xy_smem<L>(), s>>>(a);
  return cudaGetLastError();
}

template <int L> cudaError_t prepare_len() {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(xy_plane_pass<L, L, kFwd>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xy_smem<L>())))
    return e;
  if ((e = cudaFuncSetAttribute(xy_plane_pass<L, L, kInvEpi>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xy_smem<L>())))
    return e;
  return cudaFuncSetAttribute(xy_plane_pass<L, L, kInvEpiFwd>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xy_smem<L>());
}

template <int L>
cudaError_t launch_mode(int mode, const PassArgs<float>& a, int B, cudaStream_t s) {
  if (mode == kFwd) return launch_xy<L, kFwd>(a, B, s);
  if (mode == kInvEpi) return launch_xy<L, kInvEpi>(a, B, s);
  if (mode == kInvEpiFwd) return launch_xy<L, kInvEpiFwd>(a, B, s);
  return cudaErrorInvalidValue;
}

}  // namespace

bool xy_supported(const GridDev<float>& g) {
  return g.nx == g.ny && (g.nx == 64 || g.nx == 96 || g.nx == 128);
}

cudaError_t xy_prepare(const GridDev<float>& g) {
  if (g.nx == 64) return prepare_len<64>();
  if (g.nx == 96) return prepare_len<96>();
  if (g.nx == 128) return prepare_len<128>();
  return cudaErrorInvalidValue;
}

cudaError_t run_xy_pass(int mode, const GridDev<float>& g, const PassIO<float>& io, int B,
                        cudaStream_t s) {
  PassArgs<float> a{};
  a.data = io.data;
  a.src = io.src;
  a.psi_in = io.psi_in;
  a.psi_out = io.psi_out;
  a.coefs = io.coefs;
  a.step = io.step;
  a.pot = g.pot;
  a.tw = g.tw[0];
  a.tw2 = g.tw[1];
  a.alpha = io.alpha;
  a.beta = io.beta;
  a.nx = g.nx;
  a.ny = g.ny;
  a.nz = g.nz;
  if (g.nx == 64) return launch_mode<64>(mode, a, B, s);
  if (g.nx == 96) return launch_mode<96>(mode, a, B, s);
  if (g.nx == 128) return launch_mode<128>(mode, a, B, s);
  return cudaErrorInvalidValue;
}

}  // namespace sep
