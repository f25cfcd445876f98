// sep_noalloc.cu -- sep_normalize_states_noalloc: filter/norm.c:40-54 on
// device-resident states, with its reduction scratch in a fixed device array
// of this library instead of memory allocated per call.
//
// Who needs it: callers that must not allocate device memory at the point
// where they normalise -- code running while another allocator (a framework's
// caching pool) holds the device memory, and loops that must not pay
// cudaMalloc/cudaFree, which can wait for work already running on the device.
// sep_normalize_states copies host arrays and allocates on every call; this
// entry point allocates nothing.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/sep_gb300.h"
#include "sep_ctx.cuh"

namespace sep {
int cuda_fail(cudaError_t e, const char* what, int line);
int arg_fail(const char* msg);
}  // namespace sep

using namespace sep;

namespace {

// Row limit of one call and the scratch it needs: first-level partial sums
// (reduce_partial_doubles(rows) doubles) followed by one norm per row.
constexpr long kNoallocMaxRows = 1024;
constexpr long kNoallocPartialPerRow = 256;  // reduce_partial_doubles(1), checked at run time
constexpr long kNoallocScratchDoubles = kNoallocMaxRows * kNoallocPartialPerRow + kNoallocMaxRows;

// 2,105,344 bytes per device, part of the library's module image.  Nothing in
// it has to start at zero: each call writes every slot it reads before it
// reads it.
static __device__ __align__(256) double noalloc_scratch[kNoallocScratchDoubles];

constexpr int kNoallocMaxDevices = 64;
std::mutex noalloc_mu;
double* noalloc_ptr[kNoallocMaxDevices] = {};

// Device address of noalloc_scratch in the current context of device `dev`.
// Outside stream capture it is looked up on every call, so the address stays
// right after cudaDeviceReset (which recreates the module) and in a context
// other than the primary one.  While `s` captures, the address of the last
// lookup on that device is used: the first call on a device, which does the
// lookup, has to come before any capture begins.
int noalloc_scratch_ptr(int dev, cudaStream_t s, double** out) {
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(s, &cap);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();
    cap = cudaStreamCaptureStatusActive;  // treat an unknown state as capturing
  }
  std::lock_guard<std::mutex> lock(noalloc_mu);
  if (cap == cudaStreamCaptureStatusNone) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(noalloc_scratch)", __LINE__);
    noalloc_ptr[dev] = static_cast<double*>(p);
  } else if (!noalloc_ptr[dev]) {
    return arg_fail("sep_normalize_states_noalloc: first call on this device made during "
                    "stream capture; make one call before capturing");
  }
  *out = noalloc_ptr[dev];
  return kOk;
}

}  // namespace

int sep_normalize_states_noalloc(double* psi_dev, long m, long ngrid, double dv,
                                 void* cuda_stream) {
  if (!psi_dev || m < 1 || ngrid < 1 || !(dv > 0.0))
    return arg_fail("sep_normalize_states_noalloc: bad argument");
  if (m > kNoallocMaxRows)
    return arg_fail("sep_normalize_states_noalloc: more than 1024 states in one call; "
                    "split the block into calls of at most 1024 states");
  const size_t need = reduce_partial_doubles(m) + (size_t)m;
  if (need > (size_t)kNoallocScratchDoubles)
    return arg_fail("sep_normalize_states_noalloc: reduction scratch larger than its fixed size");
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    sep::set_error("sep_normalize_states_noalloc: no CUDA device");
    return kErrNoDevice;
  }
  if (dev < 0 || dev >= kNoallocMaxDevices)
    return arg_fail("sep_normalize_states_noalloc: device ordinal above 63");
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  double* scratch = nullptr;
  int r = noalloc_scratch_ptr(dev, s, &scratch);
  if (r != kOk) return r;
  e = normalize_rows<double>(psi_dev, m, ngrid, dv, scratch, scratch + reduce_partial_doubles(m), s);
  if (e != cudaSuccess) return cuda_fail(e, "sep_normalize_states_noalloc", __LINE__);
  return kOk;
}
