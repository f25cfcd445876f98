// sep_vbuild.cu -- local potential on the grid and its backward.
//
// Forward (filter/init.c:157-182, filter/interpolate.c:11-23, with the
// per-atom factor of filterStrainCube/interpolate.c:11-25):
//   potl[g] = sum_a v_{t(a)}(|r_g - R_a|),  v = a r + b on the table segment
//   i = (long)(r / dr), zero when i > n - 2.
// The reference loops over every atom for every point.  Here each block owns
// a brick of grid points, keeps (in atom order) only the atoms whose table
// range reaches the brick, and sums those; the dropped atoms contribute
// exactly zero, so the per-point sum is the reference's, term for term.
// Products and sums are issued with explicit round-to-nearest intrinsics so
// the compiler cannot contract them into FMAs: the result is bit-identical to
// the reference's C loop.
//
// Backward: dL/dtab_v[t][i] (and dL/dscale[a]) from dL/dpotl, through the
// linear interpolation weights v = s ((1 - w) p_i + w p_{i+1}),
// w = (r - r_i) / (r_{i+1} - r_i).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <vector>

#include "../../include/sep_gb300.h"
#include "sep_ctx.cuh"

namespace sep {
int cuda_fail(cudaError_t e, const char* what, int line);
int arg_fail(const char* msg);
}  // namespace sep

using namespace sep;

#define CK(...)                                                  \
  do {                                                            \
    cudaError_t _e = (__VA_ARGS__);                                      \
    if (_e != cudaSuccess) return cuda_fail(_e, #__VA_ARGS__, __LINE__); \
  } while (0)

namespace {

constexpr int BX = 8, BY = 8, BZ = 4;  // 256 points per block
constexpr int kListCap = 2048;         // atoms kept per round

struct VArgs {
  const double* xyz;     // natom x 3
  const int* types;
  const double* scale;   // or null
  const double* tab_r;   // ntype x stride
  const double* tab_v;
  const long* tab_n;
  const double* rcut;    // ntype: (n - 1) * dr, beyond which the table gives 0
  long long natom;
  long long stride;
  const double* vx;      // axis coordinates (running sums, filter/init.c:157-159)
  const double* vy;
  const double* vz;
  int nx, ny, nz;
  double rcut_max;
};

__device__ __forceinline__ double seg_value(double r, const double* tr, const double* tv,
                                            long n, double s, bool scaled) {
  const double dr = __dadd_rn(tr[1], -tr[0]);
  const long i = (long)(r / dr);
  if (i > n - 2) return 0.0;
  double a, b;
  if (scaled) {
    a = __dmul_rn(s, __dadd_rn(tv[i + 1], -tv[i])) / __dadd_rn(tr[i + 1], -tr[i]);
    b = __dadd_rn(__dmul_rn(s, tv[i]), -__dmul_rn(tr[i], a));
  } else {
    a = __dadd_rn(tv[i + 1], -tv[i]) / __dadd_rn(tr[i + 1], -tr[i]);
    b = __dadd_rn(tv[i], -__dmul_rn(tr[i], a));
  }
  return __dadd_rn(__dmul_rn(a, r), b);
}

// distance from point p to the interval [lo, hi] along one axis
__device__ __forceinline__ double gap(double p, double lo, double hi) {
  return p < lo ? lo - p : (p > hi ? p - hi : 0.0);
}

// in-order compaction of the atoms of one 256-atom chunk that can reach the brick
__device__ int collect(const VArgs& a, long long a0, double bx0, double bx1, double by0,
                       double by1, double bz0, double bz1, int* list, int base) {
  __shared__ int warp_tot[8];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const long long ai = a0 + tid;
  bool keep = false;
  if (ai < a.natom) {
    const double px = a.xyz[3 * ai], py = a.xyz[3 * ai + 1], pz = a.xyz[3 * ai + 2];
    const double gx = gap(px, bx0, bx1), gy = gap(py, by0, by1), gz = gap(pz, bz0, bz1);
    const double rc = a.rcut[a.types[ai]] * (1.0 + 1e-12) + 1e-12;
    keep = gx * gx + gy * gy + gz * gz <= rc * rc;
  }
  const unsigned m = __ballot_sync(0xffffffffu, keep);
  const int before = __popc(m & ((1u << lane) - 1u));
  if (lane == 0) warp_tot[w] = __popc(m);
  __syncthreads();
  int off = 0, tot = 0;
  for (int k = 0; k < 8; ++k) {
    if (k < w) off += warp_tot[k];
    tot += warp_tot[k];
  }
  if (keep) list[base + off + before] = (int)ai;
  __syncthreads();
  return tot;
}

__global__ void __launch_bounds__(256) k_vbuild(VArgs a, double* __restrict__ potl) {
  __shared__ int list[kListCap + 256];
  const int tx = threadIdx.x % BX, ty = (threadIdx.x / BX) % BY, tz = threadIdx.x / (BX * BY);
  const int jx0 = blockIdx.x * BX, jy0 = blockIdx.y * BY, jz0 = blockIdx.z * BZ;
  const int jx = jx0 + tx, jy = jy0 + ty, jz = jz0 + tz;
  const bool inside = jx < a.nx && jy < a.ny && jz < a.nz;
  const int ex = min(jx0 + BX, a.nx) - 1, ey = min(jy0 + BY, a.ny) - 1,
            ez = min(jz0 + BZ, a.nz) - 1;
  const double bx0 = a.vx[jx0], bx1 = a.vx[ex], by0 = a.vy[jy0], by1 = a.vy[ey],
               bz0 = a.vz[jz0], bz1 = a.vz[ez];
  const double px = inside ? a.vx[jx] : 0.0, py = inside ? a.vy[jy] : 0.0,
               pz = inside ? a.vz[jz] : 0.0;
  double sum = 0.0;
  long long a0 = 0;
  while (a0 < a.natom) {
    int cnt = 0;
    // fill the list with up to kListCap kept atoms, in atom order
    while (a0 < a.natom && cnt <= kListCap - 256) {
      cnt += collect(a, a0, bx0, bx1, by0, by1, bz0, bz1, list, cnt);
      a0 += 256;
    }
    if (inside) {
      for (int k = 0; k < cnt; ++k) {
        const int ia = list[k];
        const double dx = __dadd_rn(px, -a.xyz[3 * ia]);
        const double dy = __dadd_rn(py, -a.xyz[3 * ia + 1]);
        const double dz = __dadd_rn(pz, -a.xyz[3 * ia + 2]);
        const double d = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)),
                                        __dmul_rn(dz, dz)));
        const int t = a.types[ia];
        sum = __dadd_rn(sum, seg_value(d, a.tab_r + t * a.stride, a.tab_v + t * a.stride,
                                       a.tab_n[t], a.scale ? a.scale[ia] : 1.0,
                                       a.scale != nullptr));
      }
    }
    __syncthreads();
  }
  if (inside) potl[(long long)a.nx * ((long long)a.ny * jz + jy) + jx] = sum;
}

constexpr int kMaxTypesSmem = 4;

__global__ void __launch_bounds__(256)
k_vbuild_bwd(VArgs a, const double* __restrict__ dpotl, int ntype, int nbins_smem,
             double* __restrict__ dtab, double* __restrict__ dscale) {
  extern __shared__ double hist[];  // ntype * stride when it fits
  __shared__ int list[kListCap + 256];
  const bool use_smem = nbins_smem > 0;
  for (int i = threadIdx.x; i < nbins_smem; i += blockDim.x) hist[i] = 0.0;
  __syncthreads();
  const int tx = threadIdx.x % BX, ty = (threadIdx.x / BX) % BY, tz = threadIdx.x / (BX * BY);
  const int jx0 = blockIdx.x * BX, jy0 = blockIdx.y * BY, jz0 = blockIdx.z * BZ;
  const int jx = jx0 + tx, jy = jy0 + ty, jz = jz0 + tz;
  const bool inside = jx < a.nx && jy < a.ny && jz < a.nz;
  const int ex = min(jx0 + BX, a.nx) - 1, ey = min(jy0 + BY, a.ny) - 1,
            ez = min(jz0 + BZ, a.nz) - 1;
  const double bx0 = a.vx[jx0], bx1 = a.vx[ex], by0 = a.vy[jy0], by1 = a.vy[ey],
               bz0 = a.vz[jz0], bz1 = a.vz[ez];
  const double px = inside ? a.vx[jx] : 0.0, py = inside ? a.vy[jy] : 0.0,
               pz = inside ? a.vz[jz] : 0.0;
  const double gval =
      inside ? dpotl[(long long)a.nx * ((long long)a.ny * jz + jy) + jx] : 0.0;
  long long a0 = 0;
  while (a0 < a.natom) {
    int cnt = 0;
    while (a0 < a.natom && cnt <= kListCap - 256) {
      cnt += collect(a, a0, bx0, bx1, by0, by1, bz0, bz1, list, cnt);
      a0 += 256;
    }
    if (inside && gval != 0.0) {
      for (int k = 0; k < cnt; ++k) {
        const int ia = list[k];
        const double dx = px - a.xyz[3 * ia], dy = py - a.xyz[3 * ia + 1],
                     dz = pz - a.xyz[3 * ia + 2];
        const double d = sqrt(dx * dx + dy * dy + dz * dz);
        const int t = a.types[ia];
        const double* tr = a.tab_r + t * a.stride;
        const double* tv = a.tab_v + t * a.stride;
        const long n = a.tab_n[t];
        const long i = (long)(d / (tr[1] - tr[0]));
        if (i > n - 2) continue;
        const double w = (d - tr[i]) / (tr[i + 1] - tr[i]);
        const double s = a.scale ? a.scale[ia] : 1.0;
        const double g0 = gval * s * (1.0 - w), g1 = gval * s * w;
        const long long b = (long long)t * a.stride + i;
        if (use_smem) {
          atomicAdd(&hist[b], g0);
          atomicAdd(&hist[b + 1], g1);
        } else {
          atomicAdd(&dtab[b], g0);
          atomicAdd(&dtab[b + 1], g1);
        }
        if (dscale) atomicAdd(&dscale[ia], gval * ((1.0 - w) * tv[i] + w * tv[i + 1]));
      }
    }
    __syncthreads();
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nbins_smem; i += blockDim.x)
    if (hist[i] != 0.0) atomicAdd(&dtab[i], hist[i]);
}

struct VHost {
  std::vector<double> vx, vy, vz, rcut;
  double rmax = 0.0;
};

int prepare(sep_ctx* c, long natom, const double* xyz, const int* types, const double* scale,
            long ntype, const double* tab_r, const double* tab_v, const long* tab_n,
            long stride, const double mins[3], VHost& h, VArgs& a, DevBuf& buf) {
  if (natom < 1 || ntype < 1 || stride < 2 || !xyz || !types || !tab_r || !tab_v || !tab_n ||
      !mins)
    return arg_fail("sep_vbuild: bad argument");
  for (long a_ = 0; a_ < natom; ++a_)
    if (types[a_] < 0 || types[a_] >= ntype) return arg_fail("sep_vbuild: atom type out of range");
  for (long t = 0; t < ntype; ++t)
    if (tab_n[t] < 0 || tab_n[t] > stride) return arg_fail("sep_vbuild: table length > stride");
  h.vx = host::axis_coords(c->nx, mins[0], c->dx);
  h.vy = host::axis_coords(c->ny, mins[1], c->dy);
  h.vz = host::axis_coords(c->nz, mins[2], c->dz);
  h.rcut.assign(ntype, 0.0);
  for (long t = 0; t < ntype; ++t) {
    const long n = tab_n[t];
    if (n >= 2) {
      // i = (long)(r/dr) <= n - 2 needs r < (n - 1) dr
      const double dr = tab_r[t * stride + 1] - tab_r[t * stride];
      h.rcut[t] = (double)(n - 1) * dr;
      h.rmax = std::max(h.rmax, h.rcut[t]);
    }
  }
  const size_t sz_xyz = 3 * (size_t)natom, sz_tab = (size_t)ntype * stride;
  const size_t doubles = sz_xyz + (scale ? natom : 0) + 2 * sz_tab + ntype + c->nx + c->ny +
                         c->nz + 16;
  const size_t bytes = doubles * sizeof(double) + (size_t)natom * sizeof(int) +
                       (size_t)ntype * sizeof(long) + 256;
  CK(buf.ensure(bytes));
  char* p = static_cast<char*>(buf.p);
  auto put = [&](const void* src, size_t nb) {
    void* dst = p;
    cudaMemcpyAsync(dst, src, nb, cudaMemcpyHostToDevice, c->stream);
    p += (nb + 15) / 16 * 16;
    return dst;
  };
  a.xyz = (const double*)put(xyz, sizeof(double) * sz_xyz);
  a.scale = scale ? (const double*)put(scale, sizeof(double) * natom) : nullptr;
  a.tab_r = (const double*)put(tab_r, sizeof(double) * sz_tab);
  a.tab_v = (const double*)put(tab_v, sizeof(double) * sz_tab);
  a.rcut = (const double*)put(h.rcut.data(), sizeof(double) * ntype);
  a.vx = (const double*)put(h.vx.data(), sizeof(double) * c->nx);
  a.vy = (const double*)put(h.vy.data(), sizeof(double) * c->ny);
  a.vz = (const double*)put(h.vz.data(), sizeof(double) * c->nz);
  a.types = (const int*)put(types, sizeof(int) * natom);
  a.tab_n = (const long*)put(tab_n, sizeof(long) * ntype);
  a.natom = natom;
  a.stride = stride;
  a.nx = (int)c->nx;
  a.ny = (int)c->ny;
  a.nz = (int)c->nz;
  a.rcut_max = h.rmax;
  CK(cudaGetLastError());
  return kOk;
}

}  // namespace

extern "C" {

int sep_vbuild(sep_ctx* c, long natom, const double* xyz, const int* types, const double* scale,
               long ntype, const double* tab_r, const double* tab_v, const long* tab_n,
               long tab_stride, const double mins[3], double* potl, int install) {
  if (!c) return arg_fail("sep_vbuild: null context");
  CK(cudaSetDevice(c->device));
  DevBuf in;
  VHost h;
  VArgs a;
  int r = prepare(c, natom, xyz, types, scale, ntype, tab_r, tab_v, tab_n, tab_stride, mins, h,
                  a, in);
  if (r != kOk) {
    in.release();
    return r;
  }
  double* d_pot = nullptr;
  cudaError_t e = cudaMalloc(&d_pot, sizeof(double) * c->n);
  if (e != cudaSuccess) {
    in.release();
    return cuda_fail(e, "cudaMalloc potl", __LINE__);
  }
  dim3 g((unsigned)((c->nx + BX - 1) / BX), (unsigned)((c->ny + BY - 1) / BY),
         (unsigned)((c->nz + BZ - 1) / BZ));
  k_vbuild<<<g, 256, 0, c->stream>>>(a, d_pot);
  e = cudaGetLastError();
  if (e == cudaSuccess && potl)
    e = cudaMemcpyAsync(potl, d_pot, sizeof(double) * c->n, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  int rr = (e == cudaSuccess) ? kOk : cuda_fail(e, "vbuild", __LINE__);
  if (rr == kOk && install) rr = sep_ctx_set_potential_dev(c, d_pot);
  cudaStreamSynchronize(c->stream);
  cudaFree(d_pot);
  in.release();
  return rr;
}

int sep_vbuild_backward(sep_ctx* c, long natom, const double* xyz, const int* types,
                        const double* scale, long ntype, const double* tab_r,
                        const double* tab_v, const long* tab_n, long tab_stride,
                        const double mins[3], const double* dpotl, double* dtab_v,
                        double* dscale) {
  if (!c || !dpotl || !dtab_v) return arg_fail("sep_vbuild_backward: null argument");
  CK(cudaSetDevice(c->device));
  DevBuf in;
  VHost h;
  VArgs a;
  int r = prepare(c, natom, xyz, types, scale, ntype, tab_r, tab_v, tab_n, tab_stride, mins, h,
                  a, in);
  if (r != kOk) {
    in.release();
    return r;
  }
  const size_t nb = (size_t)ntype * tab_stride;
  double *d_g = nullptr, *d_tab = nullptr, *d_sc = nullptr;
  cudaError_t e = cudaMalloc(&d_g, sizeof(double) * c->n);
  if (e == cudaSuccess) e = cudaMalloc(&d_tab, sizeof(double) * nb);
  if (e == cudaSuccess && dscale) e = cudaMalloc(&d_sc, sizeof(double) * natom);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_g, dpotl, sizeof(double) * c->n, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_tab, 0, sizeof(double) * nb, c->stream);
  if (e == cudaSuccess && d_sc) e = cudaMemsetAsync(d_sc, 0, sizeof(double) * natom, c->stream);
  if (e == cudaSuccess) {
    const int smem_bins = (nb * sizeof(double) <= 36 * 1024) ? (int)nb : 0;
    dim3 g((unsigned)((c->nx + BX - 1) / BX), (unsigned)((c->ny + BY - 1) / BY),
           (unsigned)((c->nz + BZ - 1) / BZ));
    k_vbuild_bwd<<<g, 256, smem_bins * sizeof(double), c->stream>>>(a, d_g, (int)ntype,
                                                                    smem_bins, d_tab, d_sc);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dtab_v, d_tab, sizeof(double) * nb, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess && dscale)
    e = cudaMemcpyAsync(dscale, d_sc, sizeof(double) * natom, cudaMemcpyDeviceToHost,
                        c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(d_g);
  cudaFree(d_tab);
  if (d_sc) cudaFree(d_sc);
  in.release();
  return (e == cudaSuccess) ? kOk : cuda_fail(e, "vbuild backward", __LINE__);
}

}  // extern "C"
