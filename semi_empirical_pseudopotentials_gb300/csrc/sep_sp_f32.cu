// sep_sp_f32.cu -- launch of the sub-plane pass and the zy pass (complex64),
// the fused Newton step for nx = ny = nz in {96, 112, 128, 160, 192, 256}.
#include "sep_engine.cuh"
#include "sep_subplane.cuh"

namespace sep {

namespace {

template <int L, int MODE>
cudaError_t launch_sp(const PassArgs<float>& a, int B, cudaStream_t s) {
  using T = SpTune<L>;
  using S = SpShape<L, T::nt>;
  if (B < 1) return cudaErrorInvalidValue;
  // min_blocks blocks per SM walk the units (grid, z, residue)
  const long long units = (long long)B * S::n1y * a.nz;
  const long long walkers = (long long)sm_count() * T::min_blocks;
  const long long grid = units < walkers ? units : walkers;
  if (grid > 0x7fffffffLL) return cudaErrorInvalidValue;
  subplane_pass<L, MODE><<<(int)grid, T::nt, S::smem_bytes, s>>>(a, B);
  return cudaGetLastError();
}

template <int L> cudaError_t launch_zy(const ZyArgs& z, int B, cudaStream_t s) {
  using T = ZyTune<L>;
  using S = ZyShape<L, L, T::tx>;
  if (B < 1 || B > 65535) return cudaErrorInvalidValue;
  const dim3 grid(L / T::tx, L / S::r, (unsigned)B);
  zy_pass<L, L><<<grid, T::nt, S::smem_bytes, s>>>(z);
  return cudaGetLastError();
}

template <int L> cudaError_t prepare_sp() {
  constexpr int smem = (int)SpShape<L, SpTune<L>::nt>::smem_bytes;
  constexpr int zsmem = (int)ZyShape<L, L, ZyTune<L>::tx>::smem_bytes;
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(subplane_pass<L, kFwd>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, smem)))
    return e;
  if ((e = cudaFuncSetAttribute(subplane_pass<L, kInvEpi>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, smem)))
    return e;
  if ((e = cudaFuncSetAttribute(subplane_pass<L, kInvEpiFwd>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize, smem)))
    return e;
  return cudaFuncSetAttribute(zy_pass<L, L>, cudaFuncAttributeMaxDynamicSharedMemorySize, zsmem);
}

template <int L>
cudaError_t launch_sp_mode(int mode, const PassArgs<float>& a, int B, cudaStream_t s) {
  if (mode == kFwd) return launch_sp<L, kFwd>(a, B, s);
  if (mode == kInvEpi) return launch_sp<L, kInvEpi>(a, B, s);
  if (mode == kInvEpiFwd) return launch_sp<L, kInvEpiFwd>(a, B, s);
  return cudaErrorInvalidValue;
}

}  // namespace

#define SEP_SP_LENGTHS(X) X(96) X(112) X(128) X(160) X(192) X(256)

bool subplane_length(int L) {
#define SEP_SP_IS(LL) \
  if (L == LL) return true;
  SEP_SP_LENGTHS(SEP_SP_IS)
#undef SEP_SP_IS
  return false;
}

int subplane_rows(int L) {
#define SEP_SP_R(LL) \
  if (L == LL) return SpRows<LL>::r;
  SEP_SP_LENGTHS(SEP_SP_R)
#undef SEP_SP_R
  return 0;
}

cudaError_t subplane_prepare(int L) {
#define SEP_SP_PREP(LL) \
  if (L == LL) return prepare_sp<LL>();
  SEP_SP_LENGTHS(SEP_SP_PREP)
#undef SEP_SP_PREP
  return cudaErrorInvalidValue;
}

cudaError_t subplane_launch(int mode, const PassArgs<float>& a, int B, cudaStream_t s) {
#define SEP_SP_RUN(LL) \
  if (a.nx == LL) return launch_sp_mode<LL>(mode, a, B, s);
  SEP_SP_LENGTHS(SEP_SP_RUN)
#undef SEP_SP_RUN
  return cudaErrorInvalidValue;
}

cudaError_t zy_launch(const GridDev<float>& g, cx<float>* data, int B, cudaStream_t s) {
  if (g.nz != g.nx || g.ny != g.nx) return cudaErrorInvalidValue;
  ZyArgs z;
  z.data = data;
  z.tw_y = g.tw[1];
  z.tw_z = g.tw[2];
  z.kx = g.kxr;
  z.ky = g.kyr;
  z.kz = g.kz;
  z.kcap = g.kcap;
#define SEP_ZY_RUN(LL) \
  if (g.nx == LL) return launch_zy<LL>(z, B, s);
  SEP_SP_LENGTHS(SEP_ZY_RUN)
#undef SEP_ZY_RUN
  return cudaErrorInvalidValue;
}

}  // namespace sep
