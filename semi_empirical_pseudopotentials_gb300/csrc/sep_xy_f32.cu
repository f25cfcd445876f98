// sep_xy_f32.cu -- launch of the fused xy plane pass (complex64).
#include "sep_engine.cuh"
#include "sep_xypass.cuh"

namespace sep {

namespace {

int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1)
      n = 152;
  }
  return n;
}

template <int L, int MODE>
cudaError_t launch_xy(const PassArgs<float>& a, int B, cudaStream_t s) {
  if (a.nz > 65535 || B < 1) return cudaErrorInvalidValue;
  // 96^2 and 128^2 planes: one block per SM walks its planes; 64^2 planes
  // (three blocks per SM) take one block each
  const long long planes = (long long)B * a.nz;
  if (planes > 0x7fffffffLL) return cudaErrorInvalidValue;
  const int grid = (L <= 64 || planes < sm_count()) ? (int)planes : sm_count();
  xy_plane_pass<L, MODE><<<grid, XyShape<L>::nt, XyShape<L>::smem_bytes, s>>>(a, B);
  return cudaGetLastError();
}

template <int L> cudaError_t prepare_len() {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(xy_plane_pass<L, kFwd>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)XyShape<L>::smem_bytes)))
    return e;
  if ((e = cudaFuncSetAttribute(xy_plane_pass<L, kInvEpi>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)XyShape<L>::smem_bytes)))
    return e;
  return cudaFuncSetAttribute(xy_plane_pass<L, kInvEpiFwd>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)XyShape<L>::smem_bytes);
}

template <int L>
cudaError_t launch_mode(int mode, const PassArgs<float>& a, int B, cudaStream_t s) {
  if (mode == kFwd) return launch_xy<L, kFwd>(a, B, s);
  if (mode == kInvEpi) return launch_xy<L, kInvEpi>(a, B, s);
  if (mode == kInvEpiFwd) return launch_xy<L, kInvEpiFwd>(a, B, s);
  return cudaErrorInvalidValue;
}

}  // namespace

int xy_split_n1(int L) {
  if (L == 64) return Split<64>::n1;
  if (L == 96) return Split<96>::n1;
  if (L == 128) return Split<128>::n1;
  return 0;
}

bool xy_supported(const GridDev<float>& g) {
  return g.nx == g.ny && xy_split_n1(g.nx) > 0 && g.kxr && g.kyr;
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
