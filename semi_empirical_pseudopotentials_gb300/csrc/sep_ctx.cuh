// sep_ctx.cuh -- the context behind the C ABI: device tables, workspace,
// stream, solver handle, cached Newton-loop graphs.
#pragma once

#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <map>
#include <string>
#include <vector>

#include "sep_engine.cuh"
#include "sep_host.h"
#include "sep_kernels.cuh"

namespace sep {

// status codes of include/sep_gb300.h
enum : int { kOk = 0, kErrArg = -1, kErrCuda = -2, kErrNomem = -3, kErrSolver = -4,
             kErrNoDevice = -5, kErrNumeric = -6 };

void set_error(const std::string& msg);

// a growable device buffer
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t want);
  void release();
  template <typename T> T* as() const { return static_cast<T*>(p); }
};

struct FilterGraph {
  cudaGraphExec_t exec = nullptr;
  long long key[8] = {};
};

}  // namespace sep

struct sep_ctx;

// a set of jobs (one context each) whose Newton loops form one CUDA graph
struct sep_batch {
  std::vector<sep_ctx*> ctx;
  std::vector<long> ns;
  long ms = 0, nc = 0;
  std::vector<double*> start, out;
  cudaStream_t master = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  cudaGraphExec_t exec = nullptr;
  ~sep_batch() {
    if (master) cudaStreamSynchronize(master);
    if (exec) cudaGraphExecDestroy(exec);
    for (double* p : start) cudaFree(p);
    for (double* p : out) cudaFree(p);
    for (cudaEvent_t e : join) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
    if (master) cudaStreamDestroy(master);
  }
};

struct sep_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t h2d = nullptr, d2h = nullptr;  // host copies beside the filter (sep_filter)
  // output copy time over filter time per pair, measured on the previous
  // host-buffer filter call (< 0: not yet measured); sets the chunk plan
  double host_copy_ratio = -1.0;
  cusolverDnHandle_t solver = nullptr;
  int precision = 0;
  long nx = 0, ny = 0, nz = 0;
  long long n = 0;
  double dx = 0, dy = 0, dz = 0, dv = 0, ekinmax = 10.0;
  double vmin = 0, vmax = 0;
  bool have_pot = false;
  bool use_graphs = true;
  int block_steps = 32;
  int refine_steps = 0;  // FP64 residual-subspace steps after Rayleigh-Ritz in sep_pipeline
  long polish_nc = 0;     // FP64 polish of the window's Ritz pairs in sep_pipeline (0 = off)
  double polish_guard = 0.01;  // hartree beyond the target window included in the polish
  int subspace_tc = 1;  // subspace contractions on the tensor cores (1) or the FP64 pipe (0)
  int eigensolver = 1;  // dense symmetric eigensolves: the library's own (1, default) or cuSOLVER (0)
  int fuse_xy = 1;      // complex64 Newton steps with the fused xy plane pass when it applies
  bool xy_ready = false;
  int batch_holds = 0;  // batches whose graph points at the filter workspace
  sep::host::KTables ktab;
  sep::GridDev<double> g64;
  sep::GridDev<float> g32;
  // FP64-class arithmetic of the pipeline's Rayleigh-Ritz, sigma, refinement
  // and polish H applies: IEEE FP64 (0) or double-float (1, sep_dd.cuh; the
  // default for complex64 contexts); gdd holds the grid's tables and V in
  // double-float once it is first needed
  int dd_arith = 0;
  bool dd_ready = false;
  sep::GridDev<sep::ddf> gdd;
  // workspace
  sep::DevBuf w_refine;  // psi and its residual directions (refine_device)
  // spin-orbit operator of the spinor path (sep_spinor_set_operator): the
  // neighbour lists (nlc_st layout), their counts and the Kleinman-Bylander
  // energies on the device; w_so / w_so2 / w_so3: Vso psi and spinor blocks
  long so_natom = 0, so_nnlc = 0;
  double so_sigma = 0.0;
  int so_flagkb = 0;
  bool so_ready = false;
  sep::DevBuf w_nlc, w_nl, w_elkb, w_so, w_so2, w_so3;
  sep::DevBuf w_eigh;  // workspace of the symmetric eigensolver
  sep::DevBuf w_hist, w_fft, w_acc, w_coef, w_steps, w_start, w_out, w_red, w_small,
      w_states, w_states2, w_tmp, w_solver, w_gemm, w_hpsi, w_ozA, w_ozB, w_ozP, w_ozE;
  std::vector<sep::FilterGraph> graphs;
  ~sep_ctx();
};

namespace sep {

// Host buffers of a filter call.  With them the filter runs in chunks of
// pairs: the start states of a chunk go up on ctx->h2d, and its output comes
// down on ctx->d2h while the next chunk is filtered.
struct HostIO {
  const double* start;  // ns x n
  double* out;          // ns x ms x n
};

// device-side operations used by the ABI (all on ctx->stream)
int filter_device(sep_ctx* c, const double* d_start, long ns, const double* an_re,
                  const double* zn, long ms, long nc, double dE_1, double vmin, double* d_out,
                  const HostIO* host = nullptr);
int hamiltonian_device(sep_ctx* c, const double* d_psi, double* d_hpsi, long nstates);
int energy_all_device(sep_ctx* c, const double* d_psi, long m, double* ene_host);
int energy_range_device(sep_ctx* c, double vmin, double* emax, double* dE, long* iters);
int ortho_device(sep_ctx* c, double* d_psi, long m, long* mkept);
// Frees the Newton filter's workspaces (history ring, transform and
// accumulator grids) and the start states when fewer than `need` bytes of
// device memory are free; the next filter call allocates them again.
int release_filter_workspace_if_short(sep_ctx* c, size_t need);
// keep_hpsi: also return H psi of the rotated states (rotated with them) in
// *hpsi when the device has room for it, else *hpsi = nullptr
int rayleigh_ritz_device(sep_ctx* c, double* d_psi, long m, double* eval_host,
                         double** hpsi = nullptr);
// One FP64 refinement step of k Ritz pairs (psi rows): the subspace grows by
// the residuals H psi - E psi, made orthogonal to psi and orthonormal, and
// the k lowest Ritz pairs of Rayleigh-Ritz on it replace psi (*k_out = k).
// *hpsi: H psi of the rows when known (as rayleigh_ritz_device returns it).
int refine_device(sep_ctx* c, double* d_psi, long k, long m_cap, double* eval_host,
                  double** hpsi, long* k_out);
// FP64 polish of the Ritz pairs whose values lie within c->polish_guard of
// [elmin, elmax]: a wide FP64 Gaussian filter at the window's centre
// (c->polish_nc Newton steps), then ortho, Rayleigh-Ritz and sigma of that
// block, which replaces its rows (eval, sige on the host).  *k: row count in
// and out; *applies: FP64 H applies made.
int polish_device(sep_ctx* c, double* d_psi, long* k, double elmin, double elmax, double dE,
                  double vmin, double* eval, double* sige, long* applies);
// d_hpsi: H psi of these states when already known (no H applies then)
int sigma_device(sep_ctx* c, const double* d_psi, long m, double* sige_host,
                 const double* d_hpsi = nullptr);
// also: rows scaled by the same factors as psi's (H psi follows psi)
int normalize_device(sep_ctx* c, double* d_psi, long m, double* also = nullptr);
int time_passes_device(sep_ctx* c, long npairs, int reps, double* ms_out);
int time_fused_step_device(sep_ctx* c, long npairs, int reps, double* ms_out);
int ensure_dd_grid(sep_ctx* c);  // uploads c->gdd (sep_api.cu)
int subspace_gemm_device(sep_ctx* c, const double* A, const double* B, long long m, long long n,
                         long long k, double alpha, bool sym, double* C);
int subspace_rotate_device(sep_ctx* c, const double* W, const double* X, long long m,
                           long long k, long long w, double* out);
int autotune_device(sep_ctx* c, long npairs, int reps, int* choice);
int batch_create(int njobs, sep_ctx* const* ctxs, const long* ns, long ms, long nc,
                 sep_batch** out);
int batch_set_coefficients(sep_batch* b, int job, const double* an_re, const double* zn,
                           double dE_1, double vmin);
int batch_run(sep_batch* b);
void batch_release(sep_batch* b);

}  // namespace sep
