// sep_ctx.cu -- orchestration of the filter path on one GPU.
//
// Stage order and semantics follow filter/main.c:64-142; every stage runs on
// the context's stream with device-resident data:
//   energy range (power iteration)  -> Newton filter (graph-captured loop)
//   -> normalise -> ortho (Gram + eigensolver, two passes) -> Rayleigh-Ritz
//   -> sigma.
#include <cuda_runtime.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <utility>
#include <vector>

#include "sep_ctx.cuh"
#include "sep_eigh.cuh"
#include "sep_ozaki.cuh"

namespace sep {

namespace {
thread_local std::string g_err;
}

void set_error(const std::string& msg) { g_err = msg; }
const char* last_error() { return g_err.c_str(); }

int cuda_fail(cudaError_t e, const char* what, int line) {
  char buf[512];
  snprintf(buf, sizeof buf, "CUDA error %d (%s) at sep_ctx.cu:%d in %s", (int)e,
           cudaGetErrorString(e), line, what);
  set_error(buf);
  return (e == cudaErrorMemoryAllocation) ? kErrNomem : kErrCuda;
}
int arg_fail(const char* msg) {
  set_error(msg);
  return kErrArg;
}

#define CK(...)                                              \
  do {                                                        \
    cudaError_t _e = (__VA_ARGS__);                                  \
    if (_e != cudaSuccess) return cuda_fail(_e, #__VA_ARGS__, __LINE__); \
  } while (0)
#define CKS(...)                                                          \
  do {                                                                     \
    cusolverStatus_t _s = (__VA_ARGS__);                                          \
    if (_s != CUSOLVER_STATUS_SUCCESS) {                                   \
      char _b[256];                                                        \
      snprintf(_b, sizeof _b, "cusolver status %d at sep_ctx.cu:%d in %s", \
               (int)_s, __LINE__, #__VA_ARGS__);                                  \
      set_error(_b);                                                       \
      return kErrSolver;                                                   \
    }                                                                      \
  } while (0)
#define RET(...)               \
  do {                       \
    int _r = (__VA_ARGS__);            \
    if (_r != kOk) return _r; \
  } while (0)

cudaError_t DevBuf::ensure(size_t want) {
  if (want <= bytes) return cudaSuccess;
  release();
  cudaError_t e = cudaMalloc(&p, want);
  if (e != cudaSuccess) {
    p = nullptr;
    bytes = 0;
    return e;
  }
  bytes = want;
  return cudaSuccess;
}
void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

bool length_supported(int L) {
  static const int ok[] = {14, 16, 18, 20, 24, 32, 36, 40, 48, 56, 64, 72, 80, 96, 112, 128, 160,
                           192, 256};
  for (int v : ok)
    if (v == L) return true;
  return false;
}

// helpers shared with sep_spinor_path.cu (declared in sep_ctx_detail.cuh)
namespace detail {

void drop_graphs(sep_ctx* c) {
  for (auto& g : c->graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  c->graphs.clear();
}

// grow a workspace buffer; a reallocation invalidates captured graphs.  The
// filter buffers cannot move while a batch graph refers to them.
int grow(sep_ctx* c, DevBuf& b, size_t bytes) {
  if (bytes <= b.bytes) return kOk;
  if (c->batch_holds > 0 && (&b == &c->w_hist || &b == &c->w_fft || &b == &c->w_acc ||
                             &b == &c->w_coef || &b == &c->w_steps))
    return arg_fail("the context's filter workspace is held by a batch; destroy the batch or "
                    "use sizes that fit it");
  cudaStreamSynchronize(c->stream);
  drop_graphs(c);
  cudaError_t e = b.ensure(bytes);
  if (e != cudaSuccess) return cuda_fail(e, "workspace allocation", __LINE__);
  return kOk;
}

size_t free_device_bytes() {
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return 0;
  return fr;
}

// ------------------------------------------------------------------------
// Newton filter, filter/filter.c:59-83, for the pairs of one chunk.
template <typename T> struct Prec;
template <> struct Prec<double> {
  static GridDev<double>& grid(sep_ctx* c) { return c->g64; }
};
template <> struct Prec<float> {
  static GridDev<float>& grid(sep_ctx* c) { return c->g32; }
};
template <> struct Prec<ddf> {
  static GridDev<ddf>& grid(sep_ctx* c) { return c->gdd; }
};
// tag of the precision in the filter graph cache (ddf and double are both 8 bytes)
template <typename T> constexpr long long prec_tag() {
  return std::is_same<T, ddf>::value ? 9 : (long long)sizeof(T);
}

// the fused xy plane pass runs complex64 Newton steps on square xy planes
template <typename T> bool use_xy(sep_ctx*) { return false; }
template <> bool use_xy<float>(sep_ctx* c) { return c->fuse_xy && xy_supported(c->g32); }

template <typename T>
int newton_loop_xy(sep_ctx* c, int Bc, long long nstates, long ms, long nc, int K);

template <typename T>
int newton_loop(sep_ctx* c, int Bc, long long nstates, long ms, long nc, int K) {
  if (use_xy<T>(c)) return newton_loop_xy<T>(c, Bc, nstates, ms, nc, K);
  GridDev<T>& g = Prec<T>::grid(c);
  const long long n = c->n;
  cx<T>* hist = c->w_hist.as<cx<T>>();
  cx<T>* fft = c->w_fft.as<cx<T>>();
  T* acc = c->w_acc.as<T>();
  const T* an = c->w_coef.as<T>();
  const T* steps = c->w_steps.as<T>();
  cudaStream_t s = c->stream;
  PassIO<T> io;
  io.data = fft;
  io.src = hist;  // slot 0 = the start states
  CK(run_pass<T>(0, kFwd, g, io, Bc, s));
  io.src = nullptr;
  io.coefs = steps;
  for (long j = 1; j < nc; ++j) {
    CK(run_pass<T>(1, kFwd, g, io, Bc, s));
    CK(run_pass<T>(2, kFwdKInv, g, io, Bc, s));
    CK(run_pass<T>(1, kInv, g, io, Bc, s));
    io.psi_in = hist + (long long)((j - 1) % K) * Bc * n;
    io.psi_out = hist + (long long)(j % K) * Bc * n;
    io.step = (int)j;
    CK(run_pass<T>(0, (j + 1 < nc) ? kInvEpiFwd : kInvEpi, g, io, Bc, s));
    if ((j + 1) % K == 0 || j == nc - 1) {
      const long count = j % K + 1;
      const long j0 = j - count + 1;
      CK(newton_accumulate<T, T>(hist, K, Bc, n, j0, (int)count, an, nc, (int)ms, acc, nstates,
                                 j0 == 0, s));
    }
  }
  if (nc == 1)
    CK(newton_accumulate<T, T>(hist, K, Bc, n, 0, 1, an, nc, (int)ms, acc, nstates, true, s));
  return kOk;
}

// Newton loop with two passes per step: z (forward, k^2, inverse; with the
// y transform's 8-point stage for the sub-plane form), then the xy pass (y and
// x inverse, epilogue, x and y forward) on planes or sub-planes.  The plane
// form does the same arithmetic per line as the four line passes.
template <typename T>
int newton_loop_xy(sep_ctx* c, int Bc, long long nstates, long ms, long nc, int K) {
  if constexpr (!std::is_same<T, float>::value) {
    return arg_fail("the fused xy step is complex64 only");
  } else {
    const GridDev<float>& g = c->g32;
    const long long n = c->n;
    cx<float>* hist = c->w_hist.as<cx<float>>();
    const float* an = c->w_coef.as<float>();
    cudaStream_t s = c->stream;
    PassIO<float> io;
    io.data = c->w_fft.as<cx<float>>();
    io.src = hist;  // slot 0 = the start states
    CK(run_xy_pass(kFwd, g, io, Bc, s));
    io.src = nullptr;
    io.coefs = c->w_steps.as<float>();
    for (long j = 1; j < nc; ++j) {
      CK(run_xy_zpass(g, io, Bc, s));
      io.psi_in = hist + (long long)((j - 1) % K) * Bc * n;
      io.psi_out = hist + (long long)(j % K) * Bc * n;
      io.step = (int)j;
      CK(run_xy_pass((j + 1 < nc) ? kInvEpiFwd : kInvEpi, g, io, Bc, s));
      if ((j + 1) % K == 0 || j == nc - 1) {
        const long count = j % K + 1;
        const long j0 = j - count + 1;
        CK(newton_accumulate<float, float>(hist, K, Bc, n, j0, (int)count, an, nc, (int)ms,
                                           c->w_acc.as<float>(), nstates, j0 == 0, s));
      }
    }
    if (nc == 1)
      CK(newton_accumulate<float, float>(hist, K, Bc, n, 0, 1, an, nc, (int)ms,
                                         c->w_acc.as<float>(), nstates, true, s));
    return kOk;
  }
}

template <typename T>
int filter_impl(sep_ctx* c, const double* d_start, long ns, const double* an_re,
                const double* zn, long ms, long nc, double dE_1, double vmin, double* d_out,
                const HostIO* host) {
  const long long n = c->n;
  int K = c->block_steps;
  if (K > nc) K = (int)nc;
  if (K < 1) K = 1;
  const long long B = (ns + 1) / 2;
  const size_t per_pair = sizeof(cx<T>) * (size_t)n * (size_t)(K + 1) +
                          sizeof(T) * 2 * (size_t)ms * (size_t)n;
  const size_t have = c->w_hist.bytes + c->w_fft.bytes + c->w_acc.bytes;
  size_t budget = (size_t)(0.6 * (double)free_device_bytes()) + have;
  long long Bc = (long long)(budget / per_pair);
  if (Bc < 1) return arg_fail("filter: not enough device memory for one pair of states");
  if (Bc > B) Bc = B;
  if (Bc > 65535) Bc = 65535;
  RET(grow(c, c->w_hist, sizeof(cx<T>) * (size_t)n * K * Bc));
  RET(grow(c, c->w_fft, sizeof(cx<T>) * (size_t)n * Bc));
  RET(grow(c, c->w_acc, sizeof(T) * 2 * (size_t)ms * n * Bc));
  RET(grow(c, c->w_coef, sizeof(T) * (size_t)ms * nc));
  RET(grow(c, c->w_steps, sizeof(T) * 2 * (size_t)nc));
  // coefficients and per-step epilogue scalars (hnorm.c:17-23)
  {
    std::vector<T> a((size_t)ms * nc), st(2 * (size_t)nc, T(0));
    for (size_t i = 0; i < a.size(); ++i) a[i] = (T)an_re[i];
    for (long j = 1; j < nc; ++j) {
      const double shift = 2.0 + zn[j - 1] + vmin * dE_1;
      st[2 * j] = (T)dE_1;
      st[2 * j + 1] = (T)(-shift);
    }
    CK(cudaMemcpyAsync(c->w_coef.p, a.data(), sizeof(T) * a.size(), cudaMemcpyHostToDevice,
                       c->stream));
    CK(cudaMemcpyAsync(c->w_steps.p, st.data(), sizeof(T) * st.size(), cudaMemcpyHostToDevice,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));  // host vectors go out of scope
  }
  const bool fused = use_xy<T>(c);
  if (fused && !c->xy_ready) {  // kernel attributes, outside any stream capture
    CK(xy_prepare(c->g32));
    c->xy_ready = true;
  }
  // chunks of pairs [first, first + count): at most Bc each.  With host
  // buffers each chunk's output copy runs under the next chunk's filter, and
  // only the last chunk's copy is not overlapped; small chunks filter fewer
  // pairs per second (on a 128^3 grid 4 pairs cost 17% more per pair than
  // 32).  So the last chunk splits off a tail:
  //  - copy/filter ratio r measured by an earlier call: the smallest tail t
  //    (at least 4 pairs) whose filter time covers the copy of the rest,
  //    r (c - t) <= t (32 pairs at r = 0.06: 28 + 4);
  //  - not measured yet: halved while it has 8 pairs or more (32 pairs:
  //    16, 8, 4, 4), which overlaps the copies even when they are slow.
  const std::vector<std::pair<long long, long long>> chunks =
      host::filter_chunks(B, Bc, host != nullptr, c->host_copy_ratio);
  const long long nchunks = (long long)chunks.size();
  std::vector<cudaEvent_t> ev;  // per chunk: start states up, output computed
  // timing of chunk 0: filter (on the stream) and output copy (on d2h)
  cudaEvent_t tm[4] = {nullptr, nullptr, nullptr, nullptr};
  if (host) {
    for (cudaStream_t* st : {&c->h2d, &c->d2h})
      if (!*st) CK(cudaStreamCreateWithFlags(st, cudaStreamNonBlocking));
    ev.assign(2 * nchunks, nullptr);
    for (auto& e : ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (auto& e : tm) CK(cudaEventCreate(&e));
  }
  auto chunk_states = [&](long long k, long long& s0, long long& nst) {
    s0 = 2 * chunks[k].first;
    nst = std::min<long long>(2 * chunks[k].second, ns - s0);
  };
  auto upload = [&](long long k, cudaStream_t st) -> int {
    long long s0, nst;
    chunk_states(k, s0, nst);
    CK(cudaMemcpyAsync(const_cast<double*>(d_start) + s0 * n, host->start + s0 * n,
                       sizeof(double) * (size_t)(nst * n), cudaMemcpyHostToDevice, st));
    CK(cudaEventRecord(ev[2 * k], st));
    return kOk;
  };
  int rc = kOk;
  if (host) rc = upload(0, c->stream);
  for (long long k = 0; k < nchunks && rc == kOk; ++k) {
    const int bc = (int)chunks[k].second;
    long long s0, nst;
    chunk_states(k, s0, nst);
    if (host) {
      if (k + 1 < nchunks && (rc = upload(k + 1, c->h2d)) != kOk) break;
      if (cudaStreamWaitEvent(c->stream, ev[2 * k], 0) != cudaSuccess) {
        rc = cuda_fail(cudaGetLastError(), "cudaStreamWaitEvent", __LINE__);
        break;
      }
    }
    if (host && k == 0) CK(cudaEventRecord(tm[0], c->stream));
    CK(pack_pairs<T, double>(d_start + s0 * n, nst, n, c->w_hist.as<cx<T>>(), c->stream));
    if (c->use_graphs) {
      const long long key[8] = {bc, nst, ms, nc, K, (long long)(size_t)c->w_hist.p,
                                (long long)(size_t)c->w_acc.p,
                                prec_tag<T>() + (fused ? 256 : 0)};
      FilterGraph* hit = nullptr;
      for (auto& fg : c->graphs)
        if (std::memcmp(fg.key, key, sizeof key) == 0) hit = &fg;
      if (!hit) {
        cudaGraph_t graph;
        CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        int r = newton_loop<T>(c, bc, nst, ms, nc, K);
        cudaError_t e2 = cudaStreamEndCapture(c->stream, &graph);
        if (r != kOk) return r;
        CK(e2);
        FilterGraph fg;
        std::memcpy(fg.key, key, sizeof key);
        cudaError_t e3 = cudaGraphInstantiate(&fg.exec, graph, 0);
        cudaGraphDestroy(graph);
        CK(e3);
        if (c->graphs.size() >= 4) {
          cudaGraphExecDestroy(c->graphs.front().exec);
          c->graphs.erase(c->graphs.begin());
        }
        c->graphs.push_back(fg);
        hit = &c->graphs.back();
      }
      CK(cudaGraphLaunch(hit->exec, c->stream));
    } else {
      RET(newton_loop<T>(c, bc, nst, ms, nc, K));
    }
    double* dst = d_out + s0 * ms * n;
    CK(unpack_accumulators<T>(c->w_acc.as<T>(), bc, n, (int)ms, nst, dst, c->stream));
    if (host) {  // the chunk's output goes down while the next chunk is filtered
      CK(cudaEventRecord(ev[2 * k + 1], c->stream));
      if (k == 0) CK(cudaEventRecord(tm[1], c->stream));
      CK(cudaStreamWaitEvent(c->d2h, ev[2 * k + 1], 0));
      if (k == 0) CK(cudaEventRecord(tm[2], c->d2h));
      CK(cudaMemcpyAsync(host->out + s0 * ms * n, dst, sizeof(double) * (size_t)(nst * ms * n),
                         cudaMemcpyDeviceToHost, c->d2h));
      if (k == 0) CK(cudaEventRecord(tm[3], c->d2h));
    }
  }
  if (host) {
    cudaError_t e1 = cudaStreamSynchronize(c->h2d);
    cudaError_t e2 = cudaStreamSynchronize(c->d2h);
    cudaError_t e3 = cudaStreamSynchronize(c->stream);
    float t_filter = 0.f, t_copy = 0.f;
    if (rc == kOk && e1 == cudaSuccess && e2 == cudaSuccess && e3 == cudaSuccess &&
        cudaEventElapsedTime(&t_filter, tm[0], tm[1]) == cudaSuccess &&
        cudaEventElapsedTime(&t_copy, tm[2], tm[3]) == cudaSuccess && t_filter > 0.f)
      c->host_copy_ratio = (double)t_copy / (double)t_filter;
    for (auto e : ev) cudaEventDestroy(e);
    for (auto e : tm) cudaEventDestroy(e);
    if (rc == kOk) {
      CK(e1);
      CK(e2);
      CK(e3);
    }
  }
  return rc;
}

// complex states through H in chunks that fit the scratch (FP64 or its
// double-float form: both 16 bytes per complex value)
template <typename T>
int apply_h_chunked_t(sep_ctx* c, const cx<T>* in, cx<T>* out, long long nst) {
  const long long n = c->n;
  long long chunk = (long long)((0.25 * (double)free_device_bytes() + c->w_fft.bytes) /
                                (sizeof(cx<T>) * (double)n));
  if (chunk < 1) return arg_fail("hamiltonian: not enough device memory");
  chunk = std::min<long long>(chunk, std::min<long long>(nst, 4096));
  RET(grow(c, c->w_fft, sizeof(cx<T>) * (size_t)n * chunk));
  for (long long b0 = 0; b0 < nst; b0 += chunk) {
    const int bc = (int)std::min<long long>(chunk, nst - b0);
    CK(apply_h<T>(Prec<T>::grid(c), in + b0 * n, out + b0 * n, c->w_fft.as<cx<T>>(), bc, T(1.0),
                  T(0.0), c->stream));
  }
  return kOk;
}
int apply_h_chunked(sep_ctx* c, const cx<double>* in, cx<double>* out, long long nst) {
  return apply_h_chunked_t<double>(c, in, out, nst);
}

// H applied to m real states (rows of psi) -> hpsi rows, via pair packing;
// in double-float when the context says so (FP64 in and out either way)
template <typename T>
int apply_h_real_t(sep_ctx* c, const double* d_psi, double* d_hpsi, long long m) {
  const long long n = c->n;
  const long long B = (m + 1) / 2;
  RET(grow(c, c->w_states, sizeof(cx<T>) * (size_t)n * B));
  RET(grow(c, c->w_states2, sizeof(cx<T>) * (size_t)n * B));
  CK(pack_pairs<T, double>(d_psi, m, n, c->w_states.as<cx<T>>(), c->stream));
  RET(apply_h_chunked_t<T>(c, c->w_states.as<cx<T>>(), c->w_states2.as<cx<T>>(), B));
  CK(unpack_pairs<T, double>(c->w_states2.as<cx<T>>(), m, n, d_hpsi, c->stream));
  return kOk;
}
int apply_h_real(sep_ctx* c, const double* d_psi, double* d_hpsi, long long m) {
  if (c->dd_arith) {
    RET(ensure_dd_grid(c));
    return apply_h_real_t<ddf>(c, d_psi, d_hpsi, m);
  }
  return apply_h_real_t<double>(c, d_psi, d_hpsi, m);
}

// (T + shift)^-1 applied to m real states (rows of x), in place, via pair
// packing, in chunks through w_fft
int precond_real(sep_ctx* c, double* d_x, long long m, double shift) {
  const long long n = c->n;
  const long long B = (m + 1) / 2;
  RET(grow(c, c->w_states, sizeof(cx<double>) * (size_t)n * B));
  RET(grow(c, c->w_states2, sizeof(cx<double>) * (size_t)n * B));
  CK(pack_pairs<double, double>(d_x, m, n, c->w_states.as<cx<double>>(), c->stream));
  long long chunk = (long long)((0.25 * (double)free_device_bytes() + c->w_fft.bytes) /
                                (sizeof(cx<double>) * (double)n));
  if (chunk < 1) return arg_fail("preconditioner: not enough device memory");
  chunk = std::min<long long>(chunk, std::min<long long>(B, 4096));
  RET(grow(c, c->w_fft, sizeof(cx<double>) * (size_t)n * chunk));
  for (long long b0 = 0; b0 < B; b0 += chunk) {
    const int bc = (int)std::min<long long>(chunk, B - b0);
    CK(apply_precond<double>(c->g64, c->w_states.as<cx<double>>() + b0 * n,
                             c->w_states2.as<cx<double>>() + b0 * n,
                             c->w_fft.as<cx<double>>(), bc, shift, c->stream));
  }
  CK(unpack_pairs<double, double>(c->w_states2.as<cx<double>>(), m, n, d_x, c->stream));
  return kOk;
}

// symmetric eigen-decomposition in place (column-major == row-major); w ascending.
// c->eigensolver 1: the library's own solver (sep_eigh.cu); 0: cuSOLVER syevd.
int syevd(sep_ctx* c, double* d_a, long long m, double* d_w) {
  if (c->eigensolver == 1) {
    RET(grow(c, c->w_eigh, sizeof(double) * eigh::work_doubles(m)));
    int bad = 0;
    CK(eigh::solve(d_a, (int)m, d_w, c->w_eigh.as<double>(), c->stream, &bad));
    if (bad) {
      set_error("eigensolver: the QL iteration of a leaf did not converge");
      return kErrSolver;
    }
    return kOk;
  }
  int lwork = 0;
  CKS(cusolverDnDsyevd_bufferSize(c->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER,
                                  (int)m, d_a, (int)m, d_w, &lwork));
  RET(grow(c, c->w_solver, sizeof(double) * ((size_t)lwork + 8)));
  int* info = reinterpret_cast<int*>(c->w_solver.as<double>() + lwork);
  CKS(cusolverDnDsyevd(c->solver, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_UPPER, (int)m, d_a,
                       (int)m, d_w, c->w_solver.as<double>(), lwork, info));
  int hinfo = 0;
  CK(cudaMemcpyAsync(&hinfo, info, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (hinfo != 0) {
    char b[128];
    snprintf(b, sizeof b, "eigensolver failed, info = %d", hinfo);
    set_error(b);
    return kErrSolver;
  }
  return kOk;
}

// ---- subspace contractions --------------------------------------------------
// On the tensor cores by exact splitting (sep_ozaki.cuh) when c->subspace_tc,
// else on the FP64 pipe.  Both give FP64-accurate products.
constexpr double kSliceBudgetBytes = 4.0e9;  // slice planes held per contraction pass

struct OzSpace {
  oz::Planes A, B;
  long long* part = nullptr;
  int* err = nullptr;
};

// workspace for operands of up to rowsA / rowsB rows and kk values of K
int oz_space(sep_ctx* c, long long rowsA, long long rowsB, long long kk, bool same, int nsplit,
             OzSpace& w) {
  const size_t ea = oz::plane_elems(rowsA, kk);
  const size_t eb = same ? 0 : oz::plane_elems(rowsB, kk);
  RET(grow(c, c->w_ozA, 2 * ea));
  if (!same) RET(grow(c, c->w_ozB, 2 * eb));
  RET(grow(c, c->w_ozP, 8 * (oz::part_elems(rowsA, rowsB, nsplit) + 8)));
  const size_t ne = 64 + (size_t)(rowsA + rowsB) + 512;
  RET(grow(c, c->w_ozE, sizeof(int) * ne));
  int* e = c->w_ozE.as<int>();
  CK(cudaMemsetAsync(e, 0, sizeof(int), c->stream));
  w.err = e;
  w.A.d = c->w_ozA.as<uint16_t>();
  w.A.expo = e + 64;
  w.B.d = same ? w.A.d : c->w_ozB.as<uint16_t>();
  w.B.expo = same ? w.A.expo : e + 64 + (rowsA + 256);
  w.part = c->w_ozP.as<long long>();
  return kOk;
}

int oz_check(sep_ctx* c) {
  if (!c->subspace_tc || !c->w_ozE.p) return kOk;
  int h = 0;
  CK(oz::check_status(c->w_ozE.as<int>(), c->stream, &h));
  if (h != 0) {
    char b[160];
    snprintf(b, sizeof b, "tensor-core contraction: a bounded wait in the kernel ran out (%d)", h);
    set_error(b);
    CK(cudaMemsetAsync(c->w_ozE.p, 0, sizeof(int), c->stream));
    return kErrCuda;
  }
  return kOk;
}

// C (M x Nn, dense) = alpha A B^T, A (M x K) and B (Nn x K) with rows K apart;
// sym: A == B, the symmetric result is mirrored
int sub_gemm_nt(sep_ctx* c, const double* A, const double* B, long long M, long long Nn,
                long long K, double alpha, double* C, bool sym) {
  if (!c->subspace_tc) {
    const size_t wd = gemm_nt_work_doubles(M, Nn, K);
    RET(grow(c, c->w_gemm, sizeof(double) * wd));
    CK(gemm_nt_f64(A, B, M, Nn, K, alpha, C, sym, c->w_gemm.as<double>(), wd, c->stream));
    return kOk;
  }
  const bool same = sym || A == B;
  const long long rows = (M + 127) / 128 * 128 + (same ? 0 : (Nn + 127) / 128 * 128);
  long long kc = (long long)(kSliceBudgetBytes / (double)(rows * oz::kSlices * 2));
  kc = std::max<long long>(oz::kDrainK, kc / oz::kDrainK * oz::kDrainK);
  kc = std::min<long long>(kc, (K + oz::kChunkK - 1) / oz::kChunkK * oz::kChunkK);
  const int nsplit = oz::choose_splits(M, Nn, kc, sym);
  OzSpace w;
  RET(oz_space(c, M, Nn, kc, same, nsplit, w));
  for (long long k0 = 0; k0 < K; k0 += kc) {
    const long long kw = std::min<long long>(kc, K - k0);
    CK(oz::slice_rows(A + k0, M, kw, K, w.A, c->stream));
    if (!same) CK(oz::slice_rows(B + k0, Nn, kw, K, w.B, c->stream));
    else w.B = w.A;
    CK(oz::gemm_nt(w.A, w.B, alpha, sym, k0 > 0, C, Nn, w.part, nsplit, w.err, c->stream));
  }
  return oz_check(c);
}

// C (M x w, dense) = W (M x K, dense) * X[0:K, 0:w] (rows of X ldx apart)
int sub_gemm_nn_ld(sep_ctx* c, const double* W, const double* X, long long M, long long w,
                   long long K, long long ldx, double* C) {
  if (!c->subspace_tc) {
    CK(gemm_nn_f64_ld(W, X, M, w, K, ldx, C, c->stream));
    return kOk;
  }
  OzSpace s;
  RET(oz_space(c, M, w, K, false, 1, s));
  CK(oz::slice_rows(W, M, K, K, s.A, c->stream));
  CK(oz::slice_cols(X, K, w, ldx, s.B, c->stream));
  CK(oz::gemm_nt(s.A, s.B, 1.0, false, false, C, w, nullptr, 1, s.err, c->stream));
  return kOk;
}

// rows of psi (m x n) <- W (k x m) psi, in place over column chunks
int rotate_rows(sep_ctx* c, double* d_psi, long long m, long long k, const double* d_w) {
  const long long n = c->n;
  long long cols = (long long)((size_t)1 << 27) / (sizeof(double) * std::max<long long>(k, 1));
  cols = std::max<long long>(64, std::min<long long>(cols, n));
  RET(grow(c, c->w_tmp, sizeof(double) * (size_t)k * cols));
  // psi is row-major m x n; a column chunk is a strided sub-matrix: use a
  // gather through the temporary (rows of the chunk are contiguous pieces)
  for (long long g0 = 0; g0 < n; g0 += cols) {
    const long long w = std::min<long long>(cols, n - g0);
    // out_chunk (k x w) = W (k x m) * psi[:, g0:g0+w] (m x w, leading dim n)
    RET(sub_gemm_nn_ld(c, d_w, d_psi + g0, k, w, m, n, c->w_tmp.as<double>()));
    CK(cudaMemcpy2DAsync(d_psi + g0, sizeof(double) * n, c->w_tmp.p, sizeof(double) * w,
                         sizeof(double) * w, k, cudaMemcpyDeviceToDevice, c->stream));
  }
  return oz_check(c);
}

}  // namespace detail
using namespace detail;

int release_filter_workspace_if_short(sep_ctx* c, size_t need) {
  if (free_device_bytes() >= need || c->batch_holds > 0) return kOk;
  CK(cudaStreamSynchronize(c->stream));
  drop_graphs(c);
  for (DevBuf* b : {&c->w_hist, &c->w_fft, &c->w_acc, &c->w_start}) b->release();
  return kOk;
}

// =========================================================================
int filter_device(sep_ctx* c, const double* d_start, long ns, const double* an_re,
                  const double* zn, long ms, long nc, double dE_1, double vmin,
                  double* d_out, const HostIO* host) {
  if (ns < 1 || ms < 1 || nc < 1 || ms > 32) return arg_fail("filter: need ns, nc >= 1 and 1 <= ms <= 32");
  if (c->precision == 1)
    return filter_impl<float>(c, d_start, ns, an_re, zn, ms, nc, dE_1, vmin, d_out, host);
  if (c->dd_arith) {  // an FP64 context that asked for double-float arithmetic
    RET(ensure_dd_grid(c));
    return filter_impl<ddf>(c, d_start, ns, an_re, zn, ms, nc, dE_1, vmin, d_out, host);
  }
  return filter_impl<double>(c, d_start, ns, an_re, zn, ms, nc, dE_1, vmin, d_out, host);
}

int hamiltonian_device(sep_ctx* c, const double* d_psi, double* d_hpsi, long nstates) {
  if (nstates < 1) return arg_fail("hamiltonian: nstates < 1");
  return apply_h_chunked(c, reinterpret_cast<const cx<double>*>(d_psi),
                         reinterpret_cast<cx<double>*>(d_hpsi), nstates);
}

int normalize_device(sep_ctx* c, double* d_psi, long m, double* also) {
  RET(grow(c, c->w_red, sizeof(double) * (reduce_partial_doubles(m) + (size_t)m + 64)));
  double* part = c->w_red.as<double>();
  double* norms = part + reduce_partial_doubles(m);
  CK(normalize_rows<double>(d_psi, m, c->n, c->dv, part, norms, c->stream));
  if (also) CK(scale_rows<double>(also, m, c->n, norms, c->dv, c->stream));
  return kOk;
}

int energy_all_device(sep_ctx* c, const double* d_psi, long m, double* ene_host) {
  const long long n = c->n;
  const long long B = (m + 1) / 2;
  RET(grow(c, c->w_states, sizeof(cx<double>) * (size_t)n * B));
  RET(grow(c, c->w_states2, sizeof(cx<double>) * (size_t)n * B));
  RET(grow(c, c->w_red, sizeof(double) * (reduce_partial_doubles(B) + 2 * (size_t)B + 64)));
  CK(pack_pairs<double, double>(d_psi, m, n, c->w_states.as<cx<double>>(), c->stream));
  RET(apply_h_chunked(c, c->w_states.as<cx<double>>(), c->w_states2.as<cx<double>>(), B));
  double* part = c->w_red.as<double>();
  double2* out = reinterpret_cast<double2*>(part + reduce_partial_doubles(B));
  CK(pair_dots<double>(c->w_states.as<cx<double>>(), c->w_states2.as<cx<double>>(), (int)B, n,
                       c->dv, out, part, c->stream));
  std::vector<double2> h(B);
  CK(cudaMemcpyAsync(h.data(), out, sizeof(double2) * B, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (long long b = 0; b < B; ++b) {
    ene_host[2 * b] = h[b].x;
    if (2 * b + 1 < m) ene_host[2 * b + 1] = h[b].y;
  }
  return kOk;
}

// filter/energy.c:53-83.  The reference applies H twice per iteration; the
// second product (H psi_{k+1}, used for the energy) is the first product of
// the next iteration, so it is reused.
int energy_range_device(sep_ctx* c, double vmin, double* emax, double* dE, long* iters) {
  const long long n = c->n;
  std::vector<double> re(n);
  host::Rand r(-874917403);
  host::init_psi(r, n, c->dv, re.data());
  RET(grow(c, c->w_states, sizeof(cx<double>) * (size_t)n));
  RET(grow(c, c->w_states2, sizeof(cx<double>) * (size_t)n));
  RET(grow(c, c->w_red, sizeof(double) * (reduce_partial_doubles(1) + 64)));
  RET(grow(c, c->w_tmp, sizeof(double) * (size_t)n));
  CK(cudaMemcpyAsync(c->w_tmp.p, re.data(), sizeof(double) * n, cudaMemcpyHostToDevice,
                     c->stream));
  cx<double>* psi = c->w_states.as<cx<double>>();
  cx<double>* hp = c->w_states2.as<cx<double>>();
  CK(pack_pairs<double, double>(c->w_tmp.as<double>(), 1, n, psi, c->stream));
  double* part = c->w_red.as<double>();
  double2* d2 = reinterpret_cast<double2*>(part + reduce_partial_doubles(1));
  double ene = 0.0 + 0.1, old = 0.0;
  long it = 0;
  RET(apply_h_chunked(c, psi, hp, 1));  // H psi_0
  for (it = 0; std::fabs((ene - old) / ene) > 1.0e-4 && it < 500; ++it) {
    // psi <- H psi / |H psi| (normalize of norm.c:9-36 over re and im)
    CK(pair_dots<double>(hp, hp, 1, n, 1.0, d2, part, c->stream));
    double2 nn;
    CK(cudaMemcpyAsync(&nn, d2, sizeof nn, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    const double nrm = std::sqrt((nn.x + nn.y) * c->dv);
    CK(scale_copy<double>(hp, psi, n, 1.0 / nrm, c->stream));
    old = ene;
    RET(apply_h_chunked(c, psi, hp, 1));
    CK(pair_dots<double>(psi, hp, 1, n, c->dv, d2, part, c->stream));
    CK(cudaMemcpyAsync(&nn, d2, sizeof nn, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    ene = nn.x + nn.y;
  }
  *emax = ene;
  *dE = 1.1 * (ene - vmin);
  if (iters) *iters = it;
  if (!std::isfinite(ene)) {
    set_error("energy range: power iteration produced a non-finite energy");
    return kErrNumeric;
  }
  return kOk;
}

// filter/ortho.c:11-52: orthonormalise the filtered states (dgesvd "O", in
// place) and keep the directions with singular-value ratio S_i/S_0 >= 1e-10.
//
// Level 1: the dv-weighted Gram matrix G = Psi Psi^T dv has eigenpairs
// (S_i^2, v_i); Q1 = Lambda^-1/2 V^T Psi are the left singular vectors of the
// directions G resolves (S_i/S_0 above ~sqrt(m eps), here 2e-7), cleaned by a
// symmetric (Loewdin) second pass.
// Level 2: the part of Psi outside span(Q1), R = Psi - Q1^T (Q1 Psi^T dv)
// (projected twice), has the small singular values as the large ones of its
// own Gram matrix; its directions down to S/S_0 = 1e-10 are appended the same
// way.  Rows of psi on return: Q1 then Q2, largest singular values first.
namespace {

// out (k x n, dense) = W (k x m) * psi (m x n), over column chunks through w_tmp
int rotate_into(sep_ctx* c, const double* d_psi, long long m, long long k, const double* d_w,
                double* d_out) {
  const long long n = c->n;
  long long cols = (long long)((size_t)1 << 27) / (sizeof(double) * std::max<long long>(k, 1));
  cols = std::max<long long>(64, std::min<long long>(cols, n));
  RET(grow(c, c->w_tmp, sizeof(double) * (size_t)k * cols));
  for (long long g0 = 0; g0 < n; g0 += cols) {
    const long long w = std::min<long long>(cols, n - g0);
    RET(sub_gemm_nn_ld(c, d_w, d_psi + g0, k, w, m, n, c->w_tmp.as<double>()));
    CK(cudaMemcpy2DAsync(d_out + g0, sizeof(double) * n, c->w_tmp.p, sizeof(double) * w,
                         sizeof(double) * w, k, cudaMemcpyDeviceToDevice, c->stream));
  }
  return oz_check(c);
}

// x (m x n) -= P^T Q with P = Q x^T dv (k x m): removes span(Q) from the rows of x
int project_out(sep_ctx* c, double* d_x, long long m, const double* d_q, long long k,
                double* P, double* Pt) {
  const long long n = c->n;
  const size_t wd = gemm_nt_work_doubles(k, m, n);
  RET(grow(c, c->w_gemm, sizeof(double) * wd));
  (void)wd;
  RET(sub_gemm_nt(c, d_q, d_x, k, m, n, c->dv, P, false));
  CK(transpose_f64(P, k, m, Pt, c->stream));  // Pt: m x k
  long long cols = (long long)((size_t)1 << 27) / (sizeof(double) * std::max<long long>(m, 1));
  cols = std::max<long long>(64, std::min<long long>(cols, n));
  RET(grow(c, c->w_tmp, sizeof(double) * (size_t)m * cols));
  for (long long g0 = 0; g0 < n; g0 += cols) {
    const long long w = std::min<long long>(cols, n - g0);
    RET(sub_gemm_nn_ld(c, Pt, d_q + g0, m, w, k, n, c->w_tmp.as<double>()));
    CK(sub_2d_f64(d_x + g0, n, c->w_tmp.as<double>(), m, w, c->stream));
  }
  return oz_check(c);
}

// Loewdin: rows of x (k x n) <- (x x^T dv)^-1/2 x, in place
int loewdin(sep_ctx* c, double* d_x, long long k, double* G, double* lam, double* W,
            double* W2) {
  const long long n = c->n;
  const size_t wd = gemm_nt_work_doubles(k, k, n);
  RET(grow(c, c->w_gemm, sizeof(double) * wd));
  (void)wd;
  RET(sub_gemm_nt(c, d_x, d_x, k, k, n, c->dv, G, true));
  RET(syevd(c, G, k, lam));
  // (x x^T dv)^-1/2 = V diag(lam^-1/2) V^T; the column-major eigenvector
  // buffer read row-major is R = V^T, so the factor is R^T (diag(lam^-1/2) R)
  CK(scale_rows_isqrt(G, lam, k, W, c->stream));
  CK(transpose_f64(G, k, k, W2, c->stream));
  CK(gemm_nn_f64(W2, W, k, k, k, G, c->stream));
  return rotate_rows(c, d_x, k, k, G);
}

}  // namespace

int ortho_device(sep_ctx* c, double* d_psi, long m, long* mkept) {
  const long long n = c->n;
  RET(grow(c, c->w_small, sizeof(double) * (6 * (size_t)m * m + 4 * (size_t)m)));
  double* G = c->w_small.as<double>();
  double* lam = G + (size_t)m * m;
  double* W = lam + m;
  double* W2 = W + (size_t)m * m;
  double* P = W2 + (size_t)m * m;
  double* Pt = P + (size_t)m * m;
  RET(grow(c, c->w_states2, sizeof(double) * (size_t)n * m));  // Q rows
  double* Q = c->w_states2.as<double>();
  const size_t wd = gemm_nt_work_doubles(m, m, n);
  RET(grow(c, c->w_gemm, sizeof(double) * wd));
  (void)wd;
  RET(sub_gemm_nt(c, d_psi, d_psi, m, m, n, c->dv, G, true));
  RET(syevd(c, G, m, lam));
  std::vector<double> hl(m);
  CK(cudaMemcpyAsync(hl.data(), lam, sizeof(double) * m, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  const double top = hl[m - 1];
  if (!(top > 0.0) || !std::isfinite(top)) {
    set_error("ortho: the states are zero or not finite");
    return kErrNumeric;
  }
  const double kRatio = 1.0e-10;                 // filter/ortho.c:41-46
  const double level1 = 2.0e-7;                  // what one Gram pass resolves
  long k0 = 0;
  while (k0 < m && !(std::sqrt(std::max(hl[k0], 0.0) / top) >= level1)) ++k0;
  const long k1 = m - k0;
  CK(scale_eigvecs(G, lam, m, k0, W, c->stream));
  RET(rotate_into(c, d_psi, m, k1, W, Q));
  RET(loewdin(c, Q, k1, G, lam, W, W2));
  long k2 = 0;
  if (k0 > 0) {
    // level 2 on the remainder of psi
    RET(project_out(c, d_psi, m, Q, k1, P, Pt));
    RET(project_out(c, d_psi, m, Q, k1, P, Pt));
    RET(sub_gemm_nt(c, d_psi, d_psi, m, m, n, c->dv, G, true));
    RET(syevd(c, G, m, lam));
    CK(cudaMemcpyAsync(hl.data(), lam, sizeof(double) * m, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    // at most k0 new directions, each with S/S_0 >= 1e-10
    long r0 = m;
    while (r0 > 0 && m - r0 < k0 && std::sqrt(std::max(hl[r0 - 1], 0.0) / top) >= kRatio) --r0;
    k2 = m - r0;
    if (k2 > 0) {
      CK(scale_eigvecs(G, lam, m, r0, W, c->stream));
      RET(rotate_into(c, d_psi, m, k2, W, Q + (size_t)k1 * n));
      double* Q2 = Q + (size_t)k1 * n;
      RET(project_out(c, Q2, k2, Q, k1, P, Pt));
      RET(loewdin(c, Q2, k2, G, lam, W, W2));
    }
  }
  const long k = k1 + k2;
  CK(cudaMemcpyAsync(d_psi, Q, sizeof(double) * (size_t)n * k, cudaMemcpyDeviceToDevice,
                     c->stream));
  *mkept = k;
  return kOk;
}

// filter/Hmat.c:11-86: H_ij = <H psi_i | psi_j> dv over the kept states, the
// symmetric part diagonalised, psi rotated onto the eigenvectors.
int rayleigh_ritz_device(sep_ctx* c, double* d_psi, long m, double* eval_host,
                         double** hpsi) {
  const long long n = c->n;
  RET(grow(c, c->w_small, sizeof(double) * (4 * (size_t)m * m + 4 * (size_t)m)));
  double* A = c->w_small.as<double>();
  double* lam = A + (size_t)m * m;
  // H psi for chunks of states, rows of A accumulated chunk by chunk.  When
  // H psi of all m states fits, it is kept and rotated with psi, so that sigma
  // needs no further H applies (H is linear: H (V psi) = V (H psi)).
  const size_t all = sizeof(double) * (size_t)n * (size_t)m;
  const bool keep = hpsi && (all <= c->w_hpsi.bytes || all <= free_device_bytes() / 3);
  long long chunk = keep ? m : std::min<long long>(m, 256);
  RET(grow(c, c->w_hpsi, sizeof(double) * (size_t)n * chunk));
  double* hps = c->w_hpsi.as<double>();
  for (long long r0 = 0; r0 < m; r0 += chunk) {
    const long long rc = std::min<long long>(chunk, m - r0);
    double* h = keep ? hps + r0 * n : hps;
    RET(apply_h_real(c, d_psi + r0 * n, h, rc));
    RET(sub_gemm_nt(c, h, d_psi, rc, m, n, c->dv, A + r0 * m, false));
  }
  CK(symmetrize_f64(A, m, c->stream));
  RET(syevd(c, A, m, lam));
  // eigenvector j is column j (A[j*m + i]); new state j = sum_i V[i][j] psi_i
  // -> rotation matrix rows = columns of V = the col-major buffer read row-major
  RET(rotate_rows(c, d_psi, m, m, A));
  if (keep) RET(rotate_rows(c, hps, m, m, A));
  if (hpsi) *hpsi = keep ? hps : nullptr;
  CK(cudaMemcpyAsync(eval_host, lam, sizeof(double) * m, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return kOk;
}

// One FP64 block step after Rayleigh-Ritz (no counterpart in the reference,
// whose filter/main.c:118-142 stops at Hmat and sigma): the residuals
// r_i = H psi_i - E_i psi_i of the k Ritz pairs (preconditioned with
// (T + 1 Ha)^-1 after a complex64 filter) are made orthogonal to psi (twice)
// and orthonormal
// (ortho_device, which drops the directions of corrections that are already
// negligible); Rayleigh-Ritz on [psi; t] in a
// workspace of its own gives k + k2 pairs, and the k lowest replace psi.  For
// a pair with residual norm sigma and gap delta the eigenvalue error goes
// from about sigma^2 / delta to about its square.  Skipped when the device
// cannot hold the extended block.
int refine_device(sep_ctx* c, double* d_psi, long k, long m_cap, double* eval_host,
                  double** hpsi, long* k_out) {
  (void)m_cap;
  const long long n = c->n;
  *k_out = k;
  const size_t row = sizeof(double) * (size_t)n;
  const size_t room = (size_t)(0.5 * (double)free_device_bytes()) + c->w_refine.bytes;
  const long kr = std::min<long>(k, (long)((long long)(room / row) - k));
  if (kr < 1) return kOk;
  RET(grow(c, c->w_refine, row * (size_t)(k + kr)));
  double* Z = c->w_refine.as<double>();
  double* R = Z + (size_t)k * n;
  CK(cudaMemcpyAsync(Z, d_psi, row * (size_t)k, cudaMemcpyDeviceToDevice, c->stream));
  RET(grow(c, c->w_small, sizeof(double) * (2 * (size_t)k * kr + (size_t)kr)));
  double* P = c->w_small.as<double>();
  double* Pt = P + (size_t)k * kr;
  double* ed = Pt + (size_t)kr * k;
  CK(cudaMemcpyAsync(ed, eval_host, sizeof(double) * kr, cudaMemcpyHostToDevice, c->stream));
  if (hpsi && *hpsi) {
    CK(residual_rows(Z, *hpsi, ed, kr, n, R, c->stream));
  } else {
    RET(apply_h_real(c, Z, R, kr));
    CK(residual_rows(Z, R, ed, kr, n, R, c->stream));
  }
  // complex64 filters: corrections (T + 1 Ha)^-1 r.  Their residuals are
  // dominated by single-precision noise at high wavenumbers, which the
  // kinetic preconditioner damps (In13_P16: median sigma 4e-5 after one step
  // against 1.1e-4 without).  The residuals of FP64 filters are smooth and go
  // in unpreconditioned (there: 9.7e-11 against 8.7e-10 with it).
  if (c->precision == 1) RET(precond_real(c, R, kr, 1.0));
  RET(project_out(c, R, kr, Z, k, P, Pt));
  RET(project_out(c, R, kr, Z, k, P, Pt));
  long k2 = 0;
  const int r = ortho_device(c, R, kr, &k2);
  if (r == kErrNumeric) return kOk;  // all residuals vanish: nothing to add
  if (r != kOk) return r;
  RET(normalize_device(c, R, k2));
  std::vector<double> ev((size_t)(k + k2));
  RET(rayleigh_ritz_device(c, Z, k + k2, ev.data(), hpsi));
  // the k lowest pairs (ascending) replace psi; H psi keeps its first k rows
  CK(cudaMemcpyAsync(d_psi, Z, row * (size_t)k, cudaMemcpyDeviceToDevice, c->stream));
  std::memcpy(eval_host, ev.data(), sizeof(double) * (size_t)k);
  RET(normalize_device(c, d_psi, k, hpsi ? *hpsi : nullptr));
  return kOk;
}

// FP64 polish of the Ritz pairs in a target window (no counterpart in the
// reference).  After a complex64 filter the Ritz vectors carry single-
// precision rounding noise spread over the whole spectrum, most of it at high
// wavenumbers; it bounds their residuals near 1e-4 Ha although their Ritz
// values already agree with the FP64 path's.  The Ritz vectors whose values
// lie in [elmin - guard, elmax + guard] are filtered once more, in FP64, by a
// wide Gaussian at the window's centre (the Newton filter of
// filter/filter.c:59-83 with one target and c->polish_nc steps), which damps
// the components far from the window and leaves those inside it nearly
// unchanged; the block is then orthonormalised and diagonalised again
// (filter/ortho.c, filter/Hmat.c) and its residuals computed (energy.c:88-119).
// The polished block replaces its rows of psi, eval and sige; *k shrinks when
// ortho drops a direction.  *applies counts the FP64 H applies.
int polish_device(sep_ctx* c, double* d_psi, long* k, double elmin, double elmax, double dE,
                  double vmin, double* eval, double* sige, long* applies) {
  *applies = 0;
  const long nc = c->polish_nc;
  const long m = *k;
  if (nc < 2 || m < 1) return kOk;
  const double lo = elmin - c->polish_guard, hi = elmax + c->polish_guard;
  long i0 = 0;
  while (i0 < m && eval[i0] < lo) ++i0;
  long i1 = i0;
  while (i1 < m && eval[i1] <= hi) ++i1;
  const long kb = i1 - i0;
  if (kb < 1) return kOk;
  const long long n = c->n;
  const size_t row = sizeof(double) * (size_t)n;
  RET(grow(c, c->w_refine, row * (size_t)kb));
  double* F = c->w_refine.as<double>();
  const double center = 0.5 * (elmin + elmax);
  const double dt = ((double)nc / (2.5 * dE)) * ((double)nc / (2.5 * dE));  // main.c:70
  std::vector<double> ar((size_t)nc), ai((size_t)nc), zn((size_t)nc);
  host::coefficients(1, nc, dE, vmin, dt, &center, ar.data(), ai.data(), zn.data());
  if (c->dd_arith) {
    RET(ensure_dd_grid(c));
    RET(filter_impl<ddf>(c, d_psi + (size_t)i0 * n, kb, ar.data(), zn.data(), 1, nc, 4.0 / dE,
                         vmin, F, nullptr));
  } else {
    RET(filter_impl<double>(c, d_psi + (size_t)i0 * n, kb, ar.data(), zn.data(), 1, nc,
                            4.0 / dE, vmin, F, nullptr));
  }
  RET(normalize_device(c, F, kb));
  long kb2 = 0;
  RET(ortho_device(c, F, kb, &kb2));
  RET(normalize_device(c, F, kb2));
  std::vector<double> ev((size_t)kb2), sg((size_t)kb2);
  double* hp = nullptr;
  RET(rayleigh_ritz_device(c, F, kb2, ev.data(), &hp));
  RET(normalize_device(c, F, kb2, hp));
  RET(sigma_device(c, F, kb2, sg.data(), hp));
  CK(cudaMemcpyAsync(d_psi + (size_t)i0 * n, F, row * (size_t)kb2, cudaMemcpyDeviceToDevice,
                     c->stream));
  const long drop = kb - kb2;
  if (drop > 0) {  // rows after the block move up, one row per copy (no overlap)
    for (long r = i1; r < m; ++r)
      CK(cudaMemcpyAsync(d_psi + (size_t)(r - drop) * n, d_psi + (size_t)r * n, row,
                         cudaMemcpyDeviceToDevice, c->stream));
    for (long r = i1; r < m; ++r) {
      eval[r - drop] = eval[r];
      sige[r - drop] = sige[r];
    }
  }
  for (long r = 0; r < kb2; ++r) {
    eval[i0 + r] = ev[(size_t)r];
    sige[i0 + r] = sg[(size_t)r];
  }
  *k = m - drop;
  *applies = kb * (nc - 1) + (hp ? 1 : 2) * kb2;
  return kOk;
}

// filter/energy.c:88-119: sigma = sqrt(<H^2> - <H>^2) = |H psi - E psi| for a
// normalised psi (dv metric) with E = <psi|H|psi>.
int sigma_device(sep_ctx* c, const double* d_psi, long m, double* sige_host,
                 const double* d_hpsi) {
  const long long n = c->n;
  long long chunk = std::min<long long>(m, 256);
  if (!d_hpsi) RET(grow(c, c->w_hpsi, sizeof(double) * (size_t)n * chunk));
  RET(grow(c, c->w_red, sizeof(double) * (reduce_partial_doubles(chunk) + 2 * (size_t)chunk + 64)));
  double* hps = c->w_hpsi.as<double>();
  double* part = c->w_red.as<double>();
  double* e = part + reduce_partial_doubles(chunk);
  double* sg = e + chunk;
  for (long long r0 = 0; r0 < m; r0 += chunk) {
    const long long rc = std::min<long long>(chunk, m - r0);
    const double* h = d_hpsi ? d_hpsi + r0 * n : hps;
    if (!d_hpsi) RET(apply_h_real(c, d_psi + r0 * n, hps, rc));
    CK(row_dots<double>(d_psi + r0 * n, h, rc, n, c->dv, e, part, c->stream));
    CK(residual_norms(d_psi + r0 * n, h, e, rc, n, c->dv, sg, part, c->stream));
    CK(cudaMemcpyAsync(sige_host + r0, sg, sizeof(double) * rc, cudaMemcpyDeviceToHost,
                       c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  return kOk;
}

template <typename T> int time_passes_impl(sep_ctx* c, long npairs, int reps, double* ms_out) {
  GridDev<T>& g = Prec<T>::grid(c);
  const long long n = c->n;
  const int K = c->block_steps;
  const int ms = 8;
  RET(grow(c, c->w_hist, sizeof(cx<T>) * (size_t)n * K * npairs));
  RET(grow(c, c->w_fft, sizeof(cx<T>) * (size_t)n * npairs));
  RET(grow(c, c->w_acc, sizeof(T) * 2 * (size_t)ms * n * npairs));
  RET(grow(c, c->w_coef, sizeof(T) * (size_t)ms * K));
  CK(cudaMemsetAsync(c->w_hist.p, 0, c->w_hist.bytes, c->stream));
  CK(cudaMemsetAsync(c->w_fft.p, 0, c->w_fft.bytes, c->stream));
  CK(cudaMemsetAsync(c->w_coef.p, 0, c->w_coef.bytes, c->stream));
  cx<T>* hist = c->w_hist.as<cx<T>>();
  PassIO<T> io;
  io.data = c->w_fft.as<cx<T>>();
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const int axis[5] = {0, 1, 2, 1, 0};
  const int mode[5] = {kFwd, kFwd, kFwdKInv, kInv, kInvEpiFwd};
  const bool xy = use_xy<T>(c);
  if (xy && !c->xy_ready) {
    CK(xy_prepare(c->g32));
    c->xy_ready = true;
  }
  ms_out[6] = 0.0;
  for (int k = 0; k < (xy ? 7 : 6); ++k) {
    for (int r = -1; r < reps; ++r) {  // r = -1: warm-up
      if (r == 0) CK(cudaEventRecord(e0, c->stream));
      if (k == 6) {
        if constexpr (std::is_same<T, float>::value) {
          PassIO<float> p = io;
          p.psi_in = hist;
          p.psi_out = hist + (long long)n * npairs;
          p.alpha = 0.1f;
          p.beta = -0.5f;
          CK(run_xy_pass(kInvEpiFwd, c->g32, p, (int)npairs, c->stream));
        }
      } else if (k < 5) {
        PassIO<T> p = io;
        if (k == 0) p.src = hist;
        if (k == 4) {
          p.psi_in = hist;
          p.psi_out = hist + (long long)n * npairs;
          p.alpha = T(0.1);
          p.beta = T(-0.5);
        }
        CK(run_pass<T>(axis[k], mode[k], g, p, (int)npairs, c->stream));
      } else {
        CK(newton_accumulate<T, T>(hist, K, (int)npairs, n, 0, K, c->w_coef.as<T>(), K, ms,
                                   c->w_acc.as<T>(), 2 * npairs, false, c->stream));
      }
    }
    CK(cudaEventRecord(e1, c->stream));
    CK(cudaEventSynchronize(e1));
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, e0, e1));
    ms_out[k] = (double)t / reps;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return kOk;
}

// Tile-shape autotuner: time both shapes of every pass kind on npairs grids
// of this context (the filter's precision) and keep the faster.
template <typename T> int autotune_impl(sep_ctx* c, long npairs, int reps, int* choice) {
  GridDev<T>& g = Prec<T>::grid(c);
  const long long n = c->n;
  RET(grow(c, c->w_hist, sizeof(cx<T>) * (size_t)n * 2 * npairs));
  RET(grow(c, c->w_fft, sizeof(cx<T>) * (size_t)n * npairs));
  CK(cudaMemsetAsync(c->w_hist.p, 0, c->w_hist.bytes, c->stream));
  CK(cudaMemsetAsync(c->w_fft.p, 0, c->w_fft.bytes, c->stream));
  cx<T>* hist = c->w_hist.as<cx<T>>();
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const int axis[5] = {0, 1, 2, 1, 0};
  const int mode[5] = {kFwd, kFwd, kFwdKInv, kInv, kInvEpiFwd};
  for (int k = 0; k < 5; ++k) {
    float best = 1e30f;
    int arg = 0;
    for (int v = 0; v < 2; ++v) {
      PassIO<T> p;
      p.data = c->w_fft.as<cx<T>>();
      p.variant = v;
      if (k == 0) p.src = hist;
      if (k == 4) {
        p.psi_in = hist;
        p.psi_out = hist + (long long)n * npairs;
      }
      for (int r = -1; r < reps; ++r) {
        if (r == 0) CK(cudaEventRecord(e0, c->stream));
        CK(run_pass<T>(axis[k], mode[k], g, p, (int)npairs, c->stream));
      }
      CK(cudaEventRecord(e1, c->stream));
      CK(cudaEventSynchronize(e1));
      float t = 0.f;
      CK(cudaEventElapsedTime(&t, e0, e1));
      if (t < best) {
        best = t;
        arg = v;
      }
    }
    g.variant[k] = arg;
    if (choice) choice[k] = arg;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  drop_graphs(c);
  return kOk;
}

int autotune_device(sep_ctx* c, long npairs, int reps, int* choice) {
  if (npairs < 1 || reps < 1) return arg_fail("sep_ctx_autotune: npairs, reps >= 1");
  if (c->precision == 1) return autotune_impl<float>(c, npairs, reps, choice);
  return autotune_impl<double>(c, npairs, reps, choice);
}

// ------------------------------------------------------------------------
// Batched filter over several contexts (grids): one CUDA graph holds every
// job's Newton loop as a parallel branch, so a single launch runs them all.
namespace {
template <typename T> int batch_job_prepare(sep_ctx* c, long ns, long ms, long nc) {
  if (use_xy<T>(c) && !c->xy_ready) {  // kernel attributes, before the batch capture
    CK(xy_prepare(c->g32));
    c->xy_ready = true;
  }
  const long long n = c->n;
  int K = c->block_steps;
  if (K > nc) K = (int)nc;
  const long long B = (ns + 1) / 2;
  RET(grow(c, c->w_hist, sizeof(cx<T>) * (size_t)n * K * B));
  RET(grow(c, c->w_fft, sizeof(cx<T>) * (size_t)n * B));
  RET(grow(c, c->w_acc, sizeof(T) * 2 * (size_t)ms * n * B));
  RET(grow(c, c->w_coef, sizeof(T) * (size_t)ms * nc));
  RET(grow(c, c->w_steps, sizeof(T) * 2 * (size_t)nc));
  return kOk;
}

template <typename T>
int batch_job_capture(sep_ctx* c, const double* d_start, long ns, long ms, long nc,
                      double* d_out) {
  const long long n = c->n;
  int K = c->block_steps;
  if (K > nc) K = (int)nc;
  const int B = (int)((ns + 1) / 2);
  CK(pack_pairs<T, double>(d_start, ns, n, c->w_hist.as<cx<T>>(), c->stream));
  RET(newton_loop<T>(c, B, ns, ms, nc, K));
  CK(unpack_accumulators<T>(c->w_acc.as<T>(), B, n, (int)ms, ns, d_out, c->stream));
  return kOk;
}

template <typename T> int batch_upload(sep_ctx* c, const double* an_re, const double* zn,
                                       long ms, long nc, double dE_1, double vmin,
                                       cudaStream_t s) {
  std::vector<T> a((size_t)ms * nc), st(2 * (size_t)nc, T(0));
  for (size_t i = 0; i < a.size(); ++i) a[i] = (T)an_re[i];
  for (long j = 1; j < nc; ++j) {
    st[2 * j] = (T)dE_1;
    st[2 * j + 1] = (T)(-(2.0 + zn[j - 1] + vmin * dE_1));
  }
  CK(cudaMemcpyAsync(c->w_coef.p, a.data(), sizeof(T) * a.size(), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(c->w_steps.p, st.data(), sizeof(T) * st.size(), cudaMemcpyHostToDevice,
                     s));
  CK(cudaStreamSynchronize(s));
  return kOk;
}
}  // namespace

int batch_create(int njobs, sep_ctx* const* ctxs, const long* ns, long ms, long nc,
                 sep_batch** out) {
  if (njobs < 1 || !ctxs || !ns || !out || ms < 1 || ms > 32 || nc < 1)
    return arg_fail("sep_batch_create: bad argument");
  for (int j = 0; j < njobs; ++j) {
    if (!ctxs[j] || ns[j] < 1 || ns[j] > 2 * 65535) return arg_fail("sep_batch_create: bad job");
    for (int i = 0; i < j; ++i)
      if (ctxs[i] == ctxs[j]) return arg_fail("sep_batch_create: each job needs its own context");
  }
  sep_batch* b = new sep_batch();
  b->ms = ms;
  b->nc = nc;
  auto fail = [&](int r) {
    delete b;
    return r;
  };
  cudaError_t e = cudaStreamCreateWithFlags(&b->master, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  if (e != cudaSuccess) return fail(cuda_fail(e, "batch stream", __LINE__));
  for (int j = 0; j < njobs; ++j) {
    sep_ctx* c = ctxs[j];
    b->ctx.push_back(c);
    b->ns.push_back(ns[j]);
    double *ds = nullptr, *dout = nullptr;
    e = cudaMalloc(&ds, sizeof(double) * (size_t)ns[j] * c->n);
    if (e == cudaSuccess) e = cudaMalloc(&dout, sizeof(double) * (size_t)ns[j] * ms * c->n);
    b->start.push_back(ds);
    b->out.push_back(dout);
    cudaEvent_t ev = nullptr;
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    b->join.push_back(ev);
    if (e != cudaSuccess) return fail(cuda_fail(e, "batch buffers", __LINE__));
    int r = (c->precision == 1) ? batch_job_prepare<float>(c, ns[j], ms, nc)
                                : batch_job_prepare<double>(c, ns[j], ms, nc);
    if (r != kOk) return fail(r);
    CK(cudaMemsetAsync(c->w_coef.p, 0, c->w_coef.bytes, c->stream));
    CK(cudaMemsetAsync(c->w_steps.p, 0, c->w_steps.bytes, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  // capture: master forks to every job's stream, every job joins back
  cudaGraph_t graph = nullptr;
  e = cudaStreamBeginCapture(b->master, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return fail(cuda_fail(e, "batch capture", __LINE__));
  int r = kOk;
  e = cudaEventRecord(b->fork, b->master);
  for (int j = 0; j < njobs && e == cudaSuccess && r == kOk; ++j) {
    sep_ctx* c = b->ctx[j];
    e = cudaStreamWaitEvent(c->stream, b->fork, 0);
    if (e != cudaSuccess) break;
    r = (c->precision == 1)
            ? batch_job_capture<float>(c, b->start[j], b->ns[j], ms, nc, b->out[j])
            : batch_job_capture<double>(c, b->start[j], b->ns[j], ms, nc, b->out[j]);
    if (r != kOk) break;
    e = cudaEventRecord(b->join[j], c->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->master, b->join[j], 0);
  }
  cudaError_t e2 = cudaStreamEndCapture(b->master, &graph);
  if (r != kOk) {
    if (graph) cudaGraphDestroy(graph);
    return fail(r);
  }
  if (e == cudaSuccess) e = e2;
  if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, graph, 0);
  if (graph) cudaGraphDestroy(graph);
  if (e != cudaSuccess) return fail(cuda_fail(e, "batch graph", __LINE__));
  for (sep_ctx* c : b->ctx) c->batch_holds++;
  *out = b;
  return kOk;
}

void batch_release(sep_batch* b) {
  if (b && b->exec)
    for (sep_ctx* c : b->ctx) c->batch_holds--;
}

int batch_set_coefficients(sep_batch* b, int job, const double* an_re, const double* zn,
                           double dE_1, double vmin) {
  if (!b || job < 0 || job >= (int)b->ctx.size() || !an_re || !zn)
    return arg_fail("sep_batch_set_coefficients: bad argument");
  sep_ctx* c = b->ctx[job];
  return (c->precision == 1)
             ? batch_upload<float>(c, an_re, zn, b->ms, b->nc, dE_1, vmin, b->master)
             : batch_upload<double>(c, an_re, zn, b->ms, b->nc, dE_1, vmin, b->master);
}

int batch_run(sep_batch* b) {
  if (!b || !b->exec) return arg_fail("sep_batch_run: no batch");
  CK(cudaGraphLaunch(b->exec, b->master));
  CK(cudaStreamSynchronize(b->master));
  return kOk;
}

// C (m x n) = alpha A B^T and out (m x w) = W X through the subspace
// contraction path of the context (device pointers, dense row-major)
int subspace_gemm_device(sep_ctx* c, const double* A, const double* B, long long m, long long n,
                         long long k, double alpha, bool sym, double* C) {
  return sub_gemm_nt(c, A, sym ? A : B, m, n, k, alpha, C, sym);
}

int subspace_rotate_device(sep_ctx* c, const double* W, const double* X, long long m,
                           long long k, long long w, double* out) {
  RET(sub_gemm_nn_ld(c, W, X, m, w, k, w, out));
  return oz_check(c);
}

// the two passes of the fused complex64 Newton step: ms_out[0] the xy pass
// (plane or sub-plane, step mode), ms_out[1] its z pass (z line pass or zy
// pass); both 0 when the context has no fused step
int time_fused_step_device(sep_ctx* c, long npairs, int reps, double* ms_out) {
  ms_out[0] = ms_out[1] = 0.0;
  if (npairs < 1 || reps < 1) return arg_fail("sep_time_fused_step: npairs, reps >= 1");
  if (c->precision != 1 || !use_xy<float>(c)) return kOk;
  if (!c->xy_ready) {
    CK(xy_prepare(c->g32));
    c->xy_ready = true;
  }
  const long long n = c->n;
  RET(grow(c, c->w_hist, sizeof(cx<float>) * (size_t)n * 2 * npairs));
  RET(grow(c, c->w_fft, sizeof(cx<float>) * (size_t)n * npairs));
  CK(cudaMemsetAsync(c->w_hist.p, 0, c->w_hist.bytes, c->stream));
  CK(cudaMemsetAsync(c->w_fft.p, 0, c->w_fft.bytes, c->stream));
  cx<float>* hist = c->w_hist.as<cx<float>>();
  PassIO<float> io;
  io.data = c->w_fft.as<cx<float>>();
  io.psi_in = hist;
  io.psi_out = hist + (long long)n * npairs;
  io.alpha = 0.1f;
  io.beta = -0.5f;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  int rc = kOk;
  for (int k = 0; k < 2 && rc == kOk; ++k) {
    for (int r = -1; r < reps && rc == kOk; ++r) {  // r = -1: warm-up
      if (r == 0) {
        const cudaError_t er = cudaEventRecord(e0, c->stream);
        if (er != cudaSuccess) rc = cuda_fail(er, "cudaEventRecord", __LINE__);
      }
      const cudaError_t e = k == 0 ? run_xy_pass(kInvEpiFwd, c->g32, io, (int)npairs, c->stream)
                                   : run_xy_zpass(c->g32, io, (int)npairs, c->stream);
      if (e != cudaSuccess) rc = cuda_fail(e, "fused step pass", __LINE__);
    }
    float t = 0.f;
    if (rc == kOk) {
      CK(cudaEventRecord(e1, c->stream));
      CK(cudaEventSynchronize(e1));
      CK(cudaEventElapsedTime(&t, e0, e1));
      ms_out[k] = (double)t / reps;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

int time_passes_device(sep_ctx* c, long npairs, int reps, double* ms_out) {
  if (npairs < 1 || reps < 1 || c->block_steps < 2)
    return arg_fail("sep_time_passes: npairs, reps >= 1 and block steps >= 2");
  if (c->precision == 1) return time_passes_impl<float>(c, npairs, reps, ms_out);
  return time_passes_impl<double>(c, npairs, reps, ms_out);
}

}  // namespace sep
