// sep_xy_f32.cu -- launch of the fused xy plane pass (complex64) and dispatch
// of the fused Newton step's two passes (plane form here, sub-plane form in
// sep_sp_f32.cu).
#include "sep_engine.cuh"
#include "sep_xypass.cuh"

namespace sep {

namespace {

template <int L, int MODE>
cudaError_t launch_xy(const PassArgs<float>& a, int B, cudaStream_t s) {
  using T = XyTune<L>;
  using S = XyShape<L, T::nt>;
  if (a.nz > 65535 || B < 1) return cudaErrorInvalidValue;
  // planes up to 64^2 take one block each (several per SM); larger planes:
  // min_blocks blocks per SM walk the planes
  const long long planes = (long long)B * a.nz;
  if (planes > 0x7fffffffLL) return cudaErrorInvalidValue;
  const long long walkers = (long long)sm_count() * T::min_blocks;
  const int grid = (L <= 64 || planes < walkers) ? (int)planes : (int)walkers;
  xy_plane_pass<L, MODE><<<grid, T::nt, S::smem_bytes, s>>>(a, B);
  return cudaGetLastError();
}

template <int L> cudaError_t prepare_len() {
  constexpr int smem = (int)XyShape<L, XyTune<L>::nt>::smem_bytes;
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(xy_plane_pass<L, kFwd>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, smem)))
    return e;
  if ((e = cudaFuncSetAttribute(xy_plane_pass<L, kInvEpi>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, smem)))
    return e;
  return cudaFuncSetAttribute(xy_plane_pass<L, kInvEpiFwd>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
}

template <int L>
cudaError_t launch_mode(int mode, const PassArgs<float>& a, int B, cudaStream_t s) {
  if (mode == kFwd) return launch_xy<L, kFwd>(a, B, s);
  if (mode == kInvEpi) return launch_xy<L, kInvEpi>(a, B, s);
  if (mode == kInvEpiFwd) return launch_xy<L, kInvEpiFwd>(a, B, s);
  return cudaErrorInvalidValue;
}

}  // namespace

// the plane lengths with a plane pass: N1 = 8, a multiple of 8 rows, the
// plane in one block's shared memory
#define SEP_XY_LENGTHS(X) X(40) X(48) X(56) X(64) X(72) X(80) X(96) X(112) X(128)

int xy_split_n1(int L) {
#define SEP_XY_N1(LL) \
  if (L == LL) return Split<LL>::n1;
  SEP_XY_LENGTHS(SEP_XY_N1)
#undef SEP_XY_N1
  if (L == 160) return Split<160>::n1;
  if (L == 192) return Split<192>::n1;
  if (L == 256) return Split<256>::n1;
  return 0;
}

namespace {
bool plane_length(int L) {
#define SEP_XY_IS(LL) \
  if (L == LL) return true;
  SEP_XY_LENGTHS(SEP_XY_IS)
#undef SEP_XY_IS
  return false;
}

// 2: sub-plane form, 1: plane form, 0: none
int xy_form(int nx, int ny, int nz) {
  if (nx != ny) return 0;
  if (nz == nx && subplane_length(nx)) return 2;
  return plane_length(nx) ? 1 : 0;
}
}  // namespace

// y: R x (L / R) in the sub-plane form, the plane pass's N1 = 8 otherwise
int xy_split_y(int nx, int nz) {
  const int f = xy_form(nx, nx, nz);
  return f == 2 ? subplane_rows(nx) : (f == 1 ? xy_split_n1(nx) : 0);
}

bool xy_supported(const GridDev<float>& g) {
  return g.kxr && g.kyr && xy_form(g.nx, g.ny, g.nz) > 0;
}

cudaError_t xy_prepare(const GridDev<float>& g) {
  if (xy_form(g.nx, g.ny, g.nz) == 2) return subplane_prepare(g.nx);
#define SEP_XY_PREP(LL) \
  if (g.nx == LL) return prepare_len<LL>();
  SEP_XY_LENGTHS(SEP_XY_PREP)
#undef SEP_XY_PREP
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
  const int form = xy_form(g.nx, g.ny, g.nz);
  if (form == 2) return subplane_launch(mode, a, B, s);
  if (form != 1) return cudaErrorInvalidValue;
#define SEP_XY_RUN(LL) \
  if (g.nx == LL) return launch_mode<LL>(mode, a, B, s);
  SEP_XY_LENGTHS(SEP_XY_RUN)
#undef SEP_XY_RUN
  return cudaErrorInvalidValue;
}

// the z pass of the fused step: the z line pass with x and y looked up in
// position order, or (sub-plane form) the zy pass
cudaError_t run_xy_zpass(const GridDev<float>& g, const PassIO<float>& io, int B,
                         cudaStream_t s) {
  const int form = xy_form(g.nx, g.ny, g.nz);
  if (form == 2) return zy_launch(g, io.data, B, s);
  if (form != 1) return cudaErrorInvalidValue;
  GridDev<float> gz = g;
  gz.kx = g.kxr;
  gz.ky = g.kyr;
  return run_pass<float>(2, kFwdKInv, gz, io, B, s);
}

}  // namespace sep
