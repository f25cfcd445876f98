// sep_api.cu -- extern "C" entry points of include/sep_gb300.h.
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/sep_gb300.h"
#include "sep_ctx.cuh"
#include "sep_eigh.cuh"

namespace sep {
const char* last_error();
int cuda_fail(cudaError_t e, const char* what, int line);
int arg_fail(const char* msg);
}  // namespace sep

using namespace sep;

#define CK(...)                                                  \
  do {                                                            \
    cudaError_t _e = (__VA_ARGS__);                                      \
    if (_e != cudaSuccess) return cuda_fail(_e, #__VA_ARGS__, __LINE__); \
  } while (0)
#define RET(...)                \
  do {                        \
    int _r = (__VA_ARGS__);             \
    if (_r != kOk) return _r; \
  } while (0)

namespace {

template <typename T> void free_grid(GridDev<T>& g) {
  for (int a = 0; a < 3; ++a)
    if (g.tw[a]) cudaFree(g.tw[a]);
  if (g.kx) cudaFree(g.kx);
  if (g.ky) cudaFree(g.ky);
  if (g.kz) cudaFree(g.kz);
  if (g.kxr) cudaFree(g.kxr);
  if (g.kyr) cudaFree(g.kyr);
  if (g.pot) cudaFree(g.pot);
  g = GridDev<T>();
}

template <typename T> int upload_grid(sep_ctx* c, GridDev<T>& g) {
  g.nx = (int)c->nx;
  g.ny = (int)c->ny;
  g.nz = (int)c->nz;
  g.n = c->n;
  const long lens[3] = {c->nx, c->ny, c->nz};
  for (int a = 0; a < 3; ++a) {
    std::vector<double> w = host::twiddles((int)lens[a]);
    std::vector<T> wt(w.begin(), w.end());
    CK(cudaMalloc(&g.tw[a], sizeof(T) * wt.size()));
    CK(cudaMemcpy(g.tw[a], wt.data(), sizeof(T) * wt.size(), cudaMemcpyHostToDevice));
  }
  const std::vector<double>* k[3] = {&c->ktab.kx, &c->ktab.ky, &c->ktab.kz};
  T** dst[3] = {&g.kx, &g.ky, &g.kz};
  for (int a = 0; a < 3; ++a) {
    std::vector<T> kt(k[a]->begin(), k[a]->end());
    CK(cudaMalloc(dst[a], sizeof(T) * kt.size()));
    CK(cudaMemcpy(*dst[a], kt.data(), sizeof(T) * kt.size(), cudaMemcpyHostToDevice));
  }
  g.kcap = (T)c->ktab.cap;
  const int n1x = (c->nx == c->ny && sizeof(T) == sizeof(float)) ? xy_split_n1((int)c->nx) : 0;
  if (n1x > 0) {  // x and y tables in the fused step's position order
    const int L = (int)c->nx;
    const int n1s[2] = {n1x, xy_split_y(L, (int)c->nz)};
    const std::vector<double>* kxy[2] = {&c->ktab.kx, &c->ktab.ky};
    T** dr[2] = {&g.kxr, &g.kyr};
    for (int a = 0; a < 2; ++a) {
      const int n1 = n1s[a], n2 = L / n1;
      std::vector<T> kt(L);
      for (int p = 0; p < L; ++p) kt[p] = (T)(*kxy[a])[(p / n1) + n2 * (p % n1)];
      CK(cudaMalloc(dr[a], sizeof(T) * L));
      CK(cudaMemcpy(*dr[a], kt.data(), sizeof(T) * L, cudaMemcpyHostToDevice));
    }
  }
  CK(cudaMalloc(&g.pot, sizeof(T) * c->n));
  CK(cudaMemset(g.pot, 0, sizeof(T) * c->n));
  return kOk;
}

}  // namespace

namespace sep {
// the grid's tables and V in double-float, uploaded on first use
int ensure_dd_grid(sep_ctx* c) {
  if (c->dd_ready) return kOk;
  free_grid(c->gdd);  // what a failed earlier upload left
  RET(upload_grid<ddf>(c, c->gdd));
  if (c->have_pot) CK(convert_f64_to_dd(c->g64.pot, c->gdd.pot, c->n, c->stream));
  c->dd_ready = true;
  return kOk;
}
}  // namespace sep

namespace {

int check_ctx(sep_ctx* c, bool need_pot = true) {
  if (!c) return arg_fail("null context");
  if (need_pot && !c->have_pot) return arg_fail("the context has no potential yet");
  CK(cudaSetDevice(c->device));
  return kOk;
}

// install a potential given on the device (FP64); min/max as filter/init.c:196-199
int install_potential(sep_ctx* c, const double* d_pot) {
  CK(cudaMemcpyAsync(c->g64.pot, d_pot, sizeof(double) * c->n, cudaMemcpyDeviceToDevice,
                     c->stream));
  if (c->precision == 1) CK(convert_f64_to_f32(c->g64.pot, c->g32.pot, c->n, c->stream));
  if (c->dd_ready) CK(convert_f64_to_dd(c->g64.pot, c->gdd.pot, c->n, c->stream));
  std::vector<double> h(c->n);
  CK(cudaMemcpyAsync(h.data(), c->g64.pot, sizeof(double) * c->n, cudaMemcpyDeviceToHost,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  double lo = 1.0e10, hi = -1.0e10;
  for (double v : h) {
    if (hi < v) hi = v;
    if (lo > v) lo = v;
  }
  c->vmin = lo;
  c->vmax = hi;
  c->have_pot = true;
  return kOk;
}

// a device copy of a host array in a workspace buffer
int to_device(sep_ctx* c, DevBuf& b, const double* h, size_t count) {
  if (count * sizeof(double) > b.bytes) {
    CK(cudaStreamSynchronize(c->stream));
    for (auto& g : c->graphs)
      if (g.exec) cudaGraphExecDestroy(g.exec);
    c->graphs.clear();
    CK(b.ensure(count * sizeof(double)));
  }
  CK(cudaMemcpyAsync(b.p, h, count * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  return kOk;
}
int ensure_buf(sep_ctx* c, DevBuf& b, size_t bytes) {
  if (bytes > b.bytes) {
    CK(cudaStreamSynchronize(c->stream));
    for (auto& g : c->graphs)
      if (g.exec) cudaGraphExecDestroy(g.exec);
    c->graphs.clear();
    CK(b.ensure(bytes));
  }
  return kOk;
}

}  // namespace

sep_ctx::~sep_ctx() {
  if (stream) cudaStreamSynchronize(stream);
  for (auto& g : graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  free_grid(g64);
  free_grid(g32);
  free_grid(gdd);
  w_refine.release();
  for (DevBuf* b : {&w_hist, &w_fft, &w_acc, &w_coef, &w_steps, &w_start, &w_out, &w_red,
                    &w_small, &w_states, &w_states2, &w_tmp, &w_solver, &w_gemm, &w_hpsi,
                    &w_ozA, &w_ozB, &w_ozP, &w_ozE, &w_nlc, &w_nl, &w_elkb, &w_so, &w_so2,
                    &w_so3, &w_eigh})
    b->release();
  if (solver) cusolverDnDestroy(solver);
  if (h2d) cudaStreamDestroy(h2d);
  if (d2h) cudaStreamDestroy(d2h);
  if (stream) cudaStreamDestroy(stream);
}

extern "C" {

const char* sep_last_error(void) { return sep::last_error(); }

int sep_version(void) { return 100; }

int sep_device_count(int* count) {
  if (!count) return arg_fail("null count");
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) n = 0;
  *count = n;
  return kOk;
}

int sep_ctx_create(const long dims[3], const double steps[3], double ekinmax,
                   const double* potl, int precision, sep_ctx** out) {
  if (!dims || !steps || !out) return arg_fail("sep_ctx_create: null argument");
  *out = nullptr;
  for (int a = 0; a < 3; ++a) {
    if (!length_supported((int)dims[a])) {
      char b[160];
      snprintf(b, sizeof b,
               "sep_ctx_create: axis length %ld has no compiled line pass "
               "(14 16 18 20 24 32 36 40 48 56 64 72 80 96 112 128 160 192 256)",
               dims[a]);
      return arg_fail(b);
    }
    if (!(steps[a] > 0.0)) return arg_fail("sep_ctx_create: grid steps must be positive");
  }
  if (precision != 0 && precision != 1) return arg_fail("sep_ctx_create: unknown precision");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    sep::set_error("sep_ctx_create: no CUDA device");
    return kErrNoDevice;
  }
  sep_ctx* c = new sep_ctx();
  cudaGetDevice(&c->device);
  c->precision = precision;
  c->dd_arith = precision == 1 ? 1 : 0;
  c->nx = dims[0];
  c->ny = dims[1];
  c->nz = dims[2];
  c->n = (long long)dims[0] * dims[1] * dims[2];
  c->dx = steps[0];
  c->dy = steps[1];
  c->dz = steps[2];
  c->dv = steps[0] * steps[1] * steps[2];
  c->ekinmax = ekinmax;
  c->ktab = host::k_tables(c->nx, c->ny, c->nz, c->dx, c->dy, c->dz, ekinmax);
  int r = kOk;
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) r = cuda_fail(e, "cudaStreamCreate", __LINE__);
  if (r == kOk && cusolverDnCreate(&c->solver) != CUSOLVER_STATUS_SUCCESS) {
    sep::set_error("sep_ctx_create: cusolverDnCreate failed");
    r = kErrSolver;
  }
  if (r == kOk) cusolverDnSetStream(c->solver, c->stream);
  if (r == kOk) r = upload_grid<double>(c, c->g64);
  if (r == kOk && precision == 1) r = upload_grid<float>(c, c->g32);
  if (r == kOk && potl) {
    r = to_device(c, c->w_tmp, potl, (size_t)c->n);
    if (r == kOk) r = install_potential(c, c->w_tmp.as<double>());
  }
  if (r != kOk) {
    delete c;
    return r;
  }
  *out = c;
  return kOk;
}

int sep_ctx_destroy(sep_ctx* ctx) {
  if (!ctx) return kOk;
  cudaSetDevice(ctx->device);
  delete ctx;
  return kOk;
}

int sep_ctx_set_potential(sep_ctx* c, const double* potl) {
  if (!c || !potl) return arg_fail("sep_ctx_set_potential: null argument");
  CK(cudaSetDevice(c->device));
  RET(to_device(c, c->w_tmp, potl, (size_t)c->n));
  return install_potential(c, c->w_tmp.as<double>());
}

int sep_ctx_set_potential_dev(sep_ctx* c, const double* potl) {
  if (!c || !potl) return arg_fail("sep_ctx_set_potential_dev: null argument");
  CK(cudaSetDevice(c->device));
  return install_potential(c, potl);
}

int sep_ctx_info(sep_ctx* c, double* vmin, double* vmax, double* dv, long* ngrid) {
  if (!c) return arg_fail("null context");
  if (vmin) *vmin = c->vmin;
  if (vmax) *vmax = c->vmax;
  if (dv) *dv = c->dv;
  if (ngrid) *ngrid = (long)c->n;
  return kOk;
}

int sep_ctx_stream(sep_ctx* c, void** s) {
  if (!c || !s) return arg_fail("null argument");
  *s = (void*)c->stream;
  return kOk;
}

int sep_ctx_set_graphs(sep_ctx* c, int enable) {
  if (!c) return arg_fail("null context");
  c->use_graphs = enable != 0;
  return kOk;
}

int sep_ctx_set_block_steps(sep_ctx* c, int k) {
  if (!c || k < 1 || k > 128) return arg_fail("sep_ctx_set_block_steps: 1 <= k <= 128");
  c->block_steps = k;
  return kOk;
}

// ---- Hamiltonian ---------------------------------------------------------
int sep_hamiltonian_dev(sep_ctx* c, const double* psi, double* hpsi, long nstates) {
  RET(check_ctx(c));
  if (!psi || !hpsi) return arg_fail("sep_hamiltonian: null argument");
  if (psi == hpsi) return arg_fail("sep_hamiltonian: psi and hpsi must differ");
  return hamiltonian_device(c, psi, hpsi, nstates);
}

int sep_hamiltonian(sep_ctx* c, const double* psi, double* hpsi, long nstates) {
  RET(check_ctx(c));
  if (!psi || !hpsi || nstates < 1) return arg_fail("sep_hamiltonian: bad argument");
  const size_t cnt = 2 * (size_t)c->n * nstates;
  RET(to_device(c, c->w_start, psi, cnt));
  RET(ensure_buf(c, c->w_out, cnt * sizeof(double)));
  RET(hamiltonian_device(c, c->w_start.as<double>(), c->w_out.as<double>(), nstates));
  CK(cudaMemcpyAsync(hpsi, c->w_out.p, cnt * sizeof(double), cudaMemcpyDeviceToHost,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return kOk;
}

int sep_apply(sep_ctx* c, const double* x, const double* y, double* out, long nstates,
              double alpha, double beta) {
  RET(check_ctx(c));
  if (!x || !out || nstates < 1) return arg_fail("sep_apply: bad argument");
  const size_t cnt = 2 * (size_t)c->n * nstates;
  RET(to_device(c, c->w_start, x, cnt));
  if (y) RET(to_device(c, c->w_states, y, cnt));
  RET(ensure_buf(c, c->w_out, cnt * sizeof(double)));
  RET(ensure_buf(c, c->w_fft, sizeof(cx<double>) * (size_t)c->n * nstates));
  CK(apply_txvy<double>(c->g64, c->w_start.as<cx<double>>(),
                        y ? c->w_states.as<cx<double>>() : nullptr, c->w_out.as<cx<double>>(),
                        c->w_fft.as<cx<double>>(), (int)nstates, alpha, beta, c->stream));
  CK(cudaMemcpyAsync(out, c->w_out.p, cnt * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return kOk;
}

int sep_ctx_set_kcap(sep_ctx* c, double kcap) {
  if (!c || !(kcap > 0.0)) return arg_fail("sep_ctx_set_kcap: bad argument");
  c->ktab.cap = kcap;
  c->g64.kcap = kcap;
  c->g32.kcap = (float)kcap;
  for (auto& g : c->graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  c->graphs.clear();
  return kOk;
}

int sep_normalize_states(double* psi, long m, long ngrid, double dv) {
  if (!psi || m < 1 || ngrid < 1 || !(dv > 0.0)) return arg_fail("sep_normalize_states: bad argument");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    sep::set_error("sep_normalize_states: no CUDA device");
    return kErrNoDevice;
  }
  const size_t cnt = (size_t)m * ngrid;
  double *d = nullptr, *red = nullptr;
  CK(cudaMalloc(&d, sizeof(double) * cnt));
  cudaError_t e = cudaMalloc(&red, sizeof(double) * (reduce_partial_doubles(m) + m + 64));
  if (e == cudaSuccess) e = cudaMemcpy(d, psi, sizeof(double) * cnt, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = normalize_rows<double>(d, m, ngrid, dv, red, red + reduce_partial_doubles(m), 0);
  if (e == cudaSuccess) e = cudaMemcpy(psi, d, sizeof(double) * cnt, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (red) cudaFree(red);
  if (e != cudaSuccess) return cuda_fail(e, "sep_normalize_states", __LINE__);
  return kOk;
}

int sep_row_sumsq(const double* x, long m, long len, double* out) {
  if (!x || !out || m < 1 || len < 1) return arg_fail("sep_row_sumsq: bad argument");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    sep::set_error("sep_row_sumsq: no CUDA device");
    return kErrNoDevice;
  }
  const size_t cnt = (size_t)m * len;
  double *d = nullptr, *red = nullptr;
  CK(cudaMalloc(&d, sizeof(double) * cnt));
  cudaError_t e = cudaMalloc(&red, sizeof(double) * (reduce_partial_doubles(m) + m + 64));
  if (e == cudaSuccess) e = cudaMemcpy(d, x, sizeof(double) * cnt, cudaMemcpyHostToDevice);
  double* res = red ? red + reduce_partial_doubles(m) : nullptr;
  if (e == cudaSuccess) e = row_dots<double>(d, d, m, len, 1.0, res, red, 0);
  if (e == cudaSuccess) e = cudaMemcpy(out, res, sizeof(double) * m, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (red) cudaFree(red);
  if (e != cudaSuccess) return cuda_fail(e, "sep_row_sumsq", __LINE__);
  return kOk;
}

int sep_hf_density(sep_ctx* c, const double* psi, long m, const double* w, double* rho) {
  RET(check_ctx(c, false));
  if (!psi || !w || !rho || m < 1) return arg_fail("sep_hf_density: bad argument");
  RET(to_device(c, c->w_start, psi, (size_t)c->n * m));
  RET(to_device(c, c->w_coef, w, (size_t)m));
  RET(ensure_buf(c, c->w_out, sizeof(double) * (size_t)c->n));
  CK(weighted_density(c->w_start.as<double>(), c->w_coef.as<double>(), m, c->n, c->dv,
                      c->w_out.as<double>(), c->stream));
  CK(cudaMemcpyAsync(rho, c->w_out.p, sizeof(double) * c->n, cudaMemcpyDeviceToHost,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return kOk;
}

int sep_ctx_ksqr(sep_ctx* c, double* out) {
  if (!c || !out) return arg_fail("sep_ctx_ksqr: null argument");
  host::ksqr_grid(c->ktab, c->nx, c->ny, c->nz, out);
  return kOk;
}

double sep_ran_nrc(long* idum) { return host::global_ran_nrc(idum); }

int sep_init_psi(long* idum, long ngrid, double dv, double* psi_re) {
  if (!idum || !psi_re || ngrid < 1) return arg_fail("sep_init_psi: bad argument");
  host::global_init_psi(idum, ngrid, dv, psi_re);
  return kOk;
}

int sep_hnorm(sep_ctx* c, const double* psim1, double* psin, long nstates, double dE_1,
              double vmin, double zm1) {
  RET(check_ctx(c));
  if (!psim1 || !psin || nstates < 1) return arg_fail("sep_hnorm: bad argument");
  const size_t cnt = 2 * (size_t)c->n * nstates;
  RET(to_device(c, c->w_start, psim1, cnt));
  RET(ensure_buf(c, c->w_out, cnt * sizeof(double)));
  RET(ensure_buf(c, c->w_fft, sizeof(cx<double>) * (size_t)c->n * nstates));
  const double shift = 2.0 + zm1 + vmin * dE_1;
  CK(apply_h<double>(c->g64, c->w_start.as<cx<double>>(), c->w_out.as<cx<double>>(),
                     c->w_fft.as<cx<double>>(), (int)nstates, dE_1, -shift, c->stream));
  CK(cudaMemcpyAsync(psin, c->w_out.p, cnt * sizeof(double), cudaMemcpyDeviceToHost,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return kOk;
}

// ---- filter --------------------------------------------------------------
int sep_filter_dev(sep_ctx* c, const double* start, long ns, const double* an_re,
                   const double* zn, long ms, long nc, double dE_1, double vmin, double* out) {
  RET(check_ctx(c));
  if (!start || !an_re || !zn || !out) return arg_fail("sep_filter: null argument");
  return filter_device(c, start, ns, an_re, zn, ms, nc, dE_1, vmin, out);
}

int sep_filter(sep_ctx* c, const double* start, long ns, const double* an_re, const double* zn,
               long ms, long nc, double dE_1, double vmin, double* out) {
  RET(check_ctx(c));
  if (!start || !an_re || !zn || !out || ns < 1 || ms < 1)
    return arg_fail("sep_filter: bad argument");
  RET(ensure_buf(c, c->w_start, sizeof(double) * (size_t)c->n * ns));
  RET(ensure_buf(c, c->w_out, sizeof(double) * (size_t)c->n * ns * ms));
  const HostIO host{start, out};
  return filter_device(c, c->w_start.as<double>(), ns, an_re, zn, ms, nc, dE_1, vmin,
                       c->w_out.as<double>(), &host);
}

// ---- norms and energies --------------------------------------------------
int sep_normalize_all(sep_ctx* c, double* psi, long m) {
  RET(check_ctx(c, false));
  if (!psi || m < 1) return arg_fail("sep_normalize_all: bad argument");
  RET(to_device(c, c->w_start, psi, (size_t)c->n * m));
  RET(normalize_device(c, c->w_start.as<double>(), m));
  CK(cudaMemcpyAsync(psi, c->w_start.p, sizeof(double) * (size_t)c->n * m,
                     cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return kOk;
}

int sep_energy_all(sep_ctx* c, const double* psi, long m, double* ene) {
  RET(check_ctx(c));
  if (!psi || !ene || m < 1) return arg_fail("sep_energy_all: bad argument");
  RET(to_device(c, c->w_start, psi, (size_t)c->n * m));
  return energy_all_device(c, c->w_start.as<double>(), m, ene);
}

int sep_energy_range(sep_ctx* c, double vmin, double* emax, double* dE, long* iters) {
  RET(check_ctx(c));
  if (!emax || !dE) return arg_fail("sep_energy_range: null argument");
  return energy_range_device(c, vmin, emax, dE, iters);
}

// ---- subspace ------------------------------------------------------------
int sep_ortho(sep_ctx* c, double* psi, long m, long* mkept) {
  RET(check_ctx(c, false));
  if (!psi || !mkept || m < 1) return arg_fail("sep_ortho: bad argument");
  RET(to_device(c, c->w_start, psi, (size_t)c->n * m));
  RET(ortho_device(c, c->w_start.as<double>(), m, mkept));
  RET(normalize_device(c, c->w_start.as<double>(), *mkept));
  CK(cudaMemcpyAsync(psi, c->w_start.p, sizeof(double) * (size_t)c->n * (*mkept),
                     cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return kOk;
}

int sep_rayleigh_ritz(sep_ctx* c, double* psi, long m, double* eval) {
  RET(check_ctx(c));
  if (!psi || !eval || m < 1) return arg_fail("sep_rayleigh_ritz: bad argument");
  RET(to_device(c, c->w_start, psi, (size_t)c->n * m));
  RET(rayleigh_ritz_device(c, c->w_start.as<double>(), m, eval));
  CK(cudaMemcpyAsync(psi, c->w_start.p, sizeof(double) * (size_t)c->n * m,
                     cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return kOk;
}

int sep_sigma(sep_ctx* c, const double* psi, long m, double* sige) {
  RET(check_ctx(c));
  if (!psi || !sige || m < 1) return arg_fail("sep_sigma: bad argument");
  RET(to_device(c, c->w_start, psi, (size_t)c->n * m));
  return sigma_device(c, c->w_start.as<double>(), m, sige);
}

// ---- whole path ----------------------------------------------------------
int sep_pipeline(sep_ctx* c, const double* start, long ns, const double* el, long ms, long nc,
                 double vmin, double dE, double* psi_out, double* eval, double* sige,
                 long* mkept, sep_timing* timing) {
  RET(check_ctx(c));
  if (!start || !el || !eval || !sige || !mkept || ns < 1 || ms < 1 || nc < 1)
    return arg_fail("sep_pipeline: bad argument");
  sep_timing t;
  std::memset(&t, 0, sizeof t);
  cudaEvent_t ev[7];
  for (auto& e : ev) CK(cudaEventCreate(&e));
  const long long n = c->n;
  const long m = ns * ms;
  RET(to_device(c, c->w_start, start, (size_t)n * ns));
  RET(ensure_buf(c, c->w_out, sizeof(double) * (size_t)n * m));
  CK(cudaEventRecord(ev[0], c->stream));
  if (!(dE > 0.0)) RET(energy_range_device(c, vmin, &t.emax, &dE, &t.power_iterations));
  CK(cudaEventRecord(ev[1], c->stream));
  const double dt = ((double)nc / (2.5 * dE)) * ((double)nc / (2.5 * dE));  // main.c:70
  std::vector<double> an_re((size_t)ms * nc), an_im((size_t)ms * nc), zn(nc);
  host::coefficients(ms, nc, dE, vmin, dt, el, an_re.data(), an_im.data(), zn.data());
  double* d_psi = c->w_out.as<double>();
  RET(filter_device(c, c->w_start.as<double>(), ns, an_re.data(), zn.data(), ms, nc, 4.0 / dE,
                    vmin, d_psi));
  RET(normalize_device(c, d_psi, m));  // filter.c:33 per cycle
  // ortho holds a second m x n block (its orthonormal rows) beside psi, plus
  // about 6 GB of contraction workspace: make room on large grids
  RET(release_filter_workspace_if_short(c, sizeof(double) * (size_t)n * m + ((size_t)6 << 30)));
  CK(cudaEventRecord(ev[2], c->stream));
  long k = 0;
  RET(ortho_device(c, d_psi, m, &k));
  RET(normalize_device(c, d_psi, k));  // main.c:112
  CK(cudaEventRecord(ev[3], c->stream));
  double* hpsi = nullptr;  // H psi of the Ritz vectors, when it fits beside them
  RET(rayleigh_ritz_device(c, d_psi, k, eval, &hpsi));
  RET(normalize_device(c, d_psi, k, hpsi));  // main.c:122
  for (int it = 0; it < c->refine_steps; ++it) {  // optional FP64 refinement
    long k2 = k;
    RET(refine_device(c, d_psi, k, m, eval, &hpsi, &k2));
    k = k2;
  }
  CK(cudaEventRecord(ev[4], c->stream));
  RET(sigma_device(c, d_psi, k, sige, hpsi));
  CK(cudaEventRecord(ev[5], c->stream));
  long polish_applies = 0;
  if (c->polish_nc > 0) {
    double lo = el[0], hi = el[0];
    for (long e = 1; e < ms; ++e) {
      lo = std::min(lo, el[e]);
      hi = std::max(hi, el[e]);
    }
    RET(polish_device(c, d_psi, &k, lo, hi, dE, vmin, eval, sige, &polish_applies));
  }
  CK(cudaEventRecord(ev[6], c->stream));
  if (psi_out)
    CK(cudaMemcpyAsync(psi_out, d_psi, sizeof(double) * (size_t)n * k, cudaMemcpyDeviceToHost,
                       c->stream));
  CK(cudaStreamSynchronize(c->stream));
  float ms_[6];
  for (int i = 0; i < 6; ++i) CK(cudaEventElapsedTime(&ms_[i], ev[i], ev[i + 1]));
  for (auto& e : ev) cudaEventDestroy(e);
  t.energy_range_s = ms_[0] * 1e-3;
  t.filter_s = ms_[1] * 1e-3;
  t.ortho_s = ms_[2] * 1e-3;
  t.rayleigh_ritz_s = ms_[3] * 1e-3;
  t.sigma_s = ms_[4] * 1e-3;
  t.polish_s = ms_[5] * 1e-3;
  t.total_s = t.energy_range_s + t.filter_s + t.ortho_s + t.rayleigh_ritz_s + t.sigma_s +
              t.polish_s;
  t.mkept = k;
  t.dE = dE;
  t.dt = dt;
  t.h_applies = (long)(t.power_iterations + 1) + (long)ns * (nc - 1) + (hpsi ? 1 : 2) * k +
                polish_applies;
  *mkept = k;
  if (timing) *timing = t;
  return kOk;
}

int sep_ctx_autotune(sep_ctx* c, long npairs, int reps, int* choices) {
  RET(check_ctx(c));
  return autotune_device(c, npairs, reps, choices);
}

int sep_batch_create(int njobs, sep_ctx* const* ctxs, const long* ns, long ms, long nc,
                     sep_batch** out) {
  if (!ctxs || !out) return arg_fail("sep_batch_create: null argument");
  for (int j = 0; j < njobs; ++j) RET(check_ctx(ctxs[j]));
  return batch_create(njobs, ctxs, ns, ms, nc, out);
}

int sep_batch_io(sep_batch* b, int job, double** start_dev, double** out_dev) {
  if (!b || job < 0 || job >= (int)b->ctx.size()) return arg_fail("sep_batch_io: bad job");
  if (start_dev) *start_dev = b->start[job];
  if (out_dev) *out_dev = b->out[job];
  return kOk;
}

int sep_batch_set_coefficients(sep_batch* b, int job, const double* an_re, const double* zn,
                               double dE_1, double vmin) {
  return batch_set_coefficients(b, job, an_re, zn, dE_1, vmin);
}

int sep_batch_run(sep_batch* b) { return batch_run(b); }

int sep_batch_load_start(sep_batch* b, int job, const double* host) {
  if (!b || job < 0 || job >= (int)b->ctx.size() || !host)
    return arg_fail("sep_batch_load_start: bad argument");
  CK(cudaMemcpy(b->start[job], host, sizeof(double) * (size_t)b->ns[job] * b->ctx[job]->n,
                cudaMemcpyHostToDevice));
  return kOk;
}

int sep_batch_read_out(sep_batch* b, int job, double* host) {
  if (!b || job < 0 || job >= (int)b->ctx.size() || !host)
    return arg_fail("sep_batch_read_out: bad argument");
  CK(cudaMemcpy(host, b->out[job],
                sizeof(double) * (size_t)b->ns[job] * b->ms * b->ctx[job]->n,
                cudaMemcpyDeviceToHost));
  return kOk;
}

int sep_ctx_set_tiles(sep_ctx* c, const int* choices) {
  if (!c || !choices) return arg_fail("sep_ctx_set_tiles: null argument");
  for (int k = 0; k < 5; ++k) {
    if (choices[k] != 0 && choices[k] != 1) return arg_fail("sep_ctx_set_tiles: shapes are 0 or 1");
    c->g64.variant[k] = choices[k];
    c->g32.variant[k] = choices[k];
  }
  for (auto& g : c->graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  c->graphs.clear();
  return kOk;
}

int sep_batch_destroy(sep_batch* b) {
  batch_release(b);
  delete b;
  return kOk;
}

int sep_time_passes(sep_ctx* c, long npairs, int reps, double* ms_out) {
  RET(check_ctx(c));
  if (!ms_out) return arg_fail("sep_time_passes: null argument");
  return time_passes_device(c, npairs, reps, ms_out);
}

int sep_time_fused_step(sep_ctx* c, long npairs, int reps, double* ms_out) {
  RET(check_ctx(c));
  if (!ms_out) return arg_fail("sep_time_fused_step: null argument");
  return time_fused_step_device(c, npairs, reps, ms_out);
}

int sep_ctx_set_refine(sep_ctx* c, int steps) {
  if (!c || steps < 0 || steps > 8) return arg_fail("sep_ctx_set_refine: steps in [0, 8]");
  c->refine_steps = steps;
  return kOk;
}

int sep_ctx_set_polish(sep_ctx* c, long nc, double guard) {
  if (!c || !(nc == 0 || (nc >= 2 && nc <= 8192)) || !(guard >= 0.0) || !std::isfinite(guard))
    return arg_fail("sep_ctx_set_polish: nc in {0} or [2, 8192] and a finite guard >= 0");
  c->polish_nc = nc;
  c->polish_guard = guard;
  return kOk;
}

int sep_ctx_set_arith(sep_ctx* c, int mode) {
  if (!c || (mode != 0 && mode != 1)) return arg_fail("sep_ctx_set_arith: mode is 0 or 1");
  c->dd_arith = mode;
  return kOk;
}

int sep_ctx_set_eigensolver(sep_ctx* c, int mode) {
  if (!c || mode < 0 || mode > 1) return arg_fail("sep_ctx_set_eigensolver: mode 0 or 1");
  c->eigensolver = mode;
  return kOk;
}

int sep_eigh(const double* a, long n, double* w, double* v) {
  if (!a || !w || !v || n < 1 || n > 16384) return arg_fail("sep_eigh: bad argument");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    set_error("sep_eigh: no CUDA device");
    return kErrNoDevice;
  }
  const size_t nn = (size_t)n * n;
  double *dA = nullptr, *dw = nullptr, *work = nullptr;
  cudaStream_t s = nullptr;
  auto done = [&](int r) {
    if (s) cudaStreamSynchronize(s);
    cudaFree(dA);
    cudaFree(dw);
    cudaFree(work);
    if (s) cudaStreamDestroy(s);
    return r;
  };
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&dA, sizeof(double) * nn) != cudaSuccess ||
      cudaMalloc(&dw, sizeof(double) * n) != cudaSuccess ||
      cudaMalloc(&work, sizeof(double) * eigh::work_doubles(n)) != cudaSuccess)
    return done(cuda_fail(cudaGetLastError(), "sep_eigh: allocation", __LINE__));
  cudaError_t e = cudaMemcpyAsync(dA, a, sizeof(double) * nn, cudaMemcpyHostToDevice, s);
  int bad = 0;
  if (e == cudaSuccess) e = eigh::solve(dA, (int)n, dw, work, s, &bad);
  if (e == cudaSuccess) e = cudaMemcpyAsync(w, dw, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(v, dA, sizeof(double) * nn, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return done(cuda_fail(e, "sep_eigh", __LINE__));
  if (bad) {
    set_error("sep_eigh: the QL iteration of a leaf did not converge");
    return done(kErrSolver);
  }
  return done(kOk);
}

size_t sep_eigh_work_bytes(long n) {
  return n < 1 ? 0 : sizeof(double) * eigh::work_doubles(n);
}

int sep_eigh_dev(double* a_dev, long n, double* w_dev, double* work_dev, void* cuda_stream,
                 double* stage_ms) {
  if (!a_dev || !w_dev || !work_dev || n < 1 || n > 16384)
    return arg_fail("sep_eigh_dev: bad argument");
  int bad = 0;
  cudaError_t e = eigh::solve(a_dev, (int)n, w_dev, work_dev,
                              static_cast<cudaStream_t>(cuda_stream), &bad, stage_ms);
  if (e != cudaSuccess) return cuda_fail(e, "sep_eigh_dev", __LINE__);
  if (bad) {
    set_error("sep_eigh_dev: the QL iteration of a leaf did not converge");
    return kErrSolver;
  }
  return kOk;
}

int sep_ctx_set_fusion(sep_ctx* c, int enable) {
  if (!c) return arg_fail("null context");
  c->fuse_xy = enable ? 1 : 0;
  return kOk;
}

int sep_ctx_set_subspace(sep_ctx* c, int mode) {
  if (!c || (mode != 0 && mode != 1)) return arg_fail("sep_ctx_set_subspace: mode is 0 or 1");
  c->subspace_tc = mode;
  return kOk;
}

namespace {
// device copies of host operands for the two subspace entry points below
struct Tmp {
  std::vector<double*> p;
  ~Tmp() {
    for (double* q : p) cudaFree(q);
  }
  cudaError_t get(size_t count, double** out) {
    double* q = nullptr;
    cudaError_t e = cudaMalloc(&q, sizeof(double) * (count ? count : 1));
    if (e == cudaSuccess) p.push_back(q);
    *out = q;
    return e;
  }
};
}  // namespace

int sep_subspace_gemm(sep_ctx* c, const double* A, const double* B, long m, long n, long k,
                      double alpha, int sym, double* C) {
  RET(check_ctx(c, false));
  if (!A || !C || (!sym && !B) || m < 1 || n < 1 || k < 1 || (sym && m != n))
    return arg_fail("sep_subspace_gemm: bad argument");
  Tmp t;
  double *dA, *dB = nullptr, *dC;
  CK(t.get((size_t)m * k, &dA));
  if (!sym) CK(t.get((size_t)n * k, &dB));
  CK(t.get((size_t)m * n, &dC));
  CK(cudaMemcpyAsync(dA, A, sizeof(double) * m * k, cudaMemcpyHostToDevice, c->stream));
  if (!sym) CK(cudaMemcpyAsync(dB, B, sizeof(double) * n * k, cudaMemcpyHostToDevice, c->stream));
  RET(subspace_gemm_device(c, dA, sym ? dA : dB, m, n, k, alpha, sym != 0, dC));
  CK(cudaMemcpyAsync(C, dC, sizeof(double) * m * n, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return kOk;
}

int sep_subspace_gemm_dev(sep_ctx* c, const double* A, const double* B, long m, long n, long k,
                          double alpha, int sym, double* C) {
  RET(check_ctx(c, false));
  if (!A || !C || (!sym && !B) || m < 1 || n < 1 || k < 1 || (sym && m != n))
    return arg_fail("sep_subspace_gemm_dev: bad argument");
  return subspace_gemm_device(c, A, sym ? A : B, m, n, k, alpha, sym != 0, C);
}

int sep_subspace_rotate(sep_ctx* c, const double* W, const double* X, long m, long k, long w,
                        double* out) {
  RET(check_ctx(c, false));
  if (!W || !X || !out || m < 1 || k < 1 || w < 1)
    return arg_fail("sep_subspace_rotate: bad argument");
  Tmp t;
  double *dW, *dX, *dO;
  CK(t.get((size_t)m * k, &dW));
  CK(t.get((size_t)k * w, &dX));
  CK(t.get((size_t)m * w, &dO));
  CK(cudaMemcpyAsync(dW, W, sizeof(double) * m * k, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(dX, X, sizeof(double) * k * w, cudaMemcpyHostToDevice, c->stream));
  RET(subspace_rotate_device(c, dW, dX, m, k, w, dO));
  CK(cudaMemcpyAsync(out, dO, sizeof(double) * m * w, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return kOk;
}

// ---- host helpers --------------------------------------------------------
int sep_filter_chunk_plan(long pairs, long max_pairs, int host_buffers, double copy_ratio,
                          long* counts, long cap, long* nchunks) {
  if (pairs < 1 || max_pairs < 1 || !counts || !nchunks || cap < 1 || std::isnan(copy_ratio))
    return arg_fail("sep_filter_chunk_plan: bad argument");
  const auto plan = host::filter_chunks(pairs, max_pairs, host_buffers != 0, copy_ratio);
  *nchunks = (long)plan.size();
  if ((long)plan.size() > cap) return arg_fail("sep_filter_chunk_plan: cap too small");
  for (size_t k = 0; k < plan.size(); ++k) counts[k] = (long)plan[k].second;
  return kOk;
}

int sep_coefficients(long ms, long nc, double dE, double vmin, double dt, const double* el,
                     double* an_re, double* an_im, double* zn) {
  if (ms < 1 || nc < 1 || !el || !an_re || !an_im || !zn || !(dE > 0.0))
    return arg_fail("sep_coefficients: bad argument");
  host::coefficients(ms, nc, dE, vmin, dt, el, an_re, an_im, zn);
  return kOk;
}

int sep_start_states(long idum, long ns, long ngrid, double dv, double* out) {
  if (ns < 1 || ngrid < 1 || !out) return arg_fail("sep_start_states: bad argument");
  host::Rand r(idum);
  for (long s = 0; s < ns; ++s) host::init_psi(r, ngrid, dv, out + (size_t)s * ngrid);
  return kOk;
}

int sep_ksqr(const long dims[3], const double steps[3], double ekinmax, double* ksqr) {
  if (!dims || !steps || !ksqr) return arg_fail("sep_ksqr: null argument");
  host::KTables t = host::k_tables(dims[0], dims[1], dims[2], steps[0], steps[1], steps[2],
                                   ekinmax);
  host::ksqr_grid(t, dims[0], dims[1], dims[2], ksqr);
  return kOk;
}

int sep_form_factor_table(const double params[4], double vol_per_atom, double* r, double* v) {
  if (!params || !r || !v) return arg_fail("sep_form_factor_table: null argument");
  host::form_factor_table(params, vol_per_atom, r, v);
  return kOk;
}

}  // extern "C"
