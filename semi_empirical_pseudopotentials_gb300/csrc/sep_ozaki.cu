// sep_ozaki.cu -- exact-split FP64 contractions on the tcgen05 tensor cores
// (see sep_ozaki.cuh for the arithmetic).
//
// Kernel shape (k_oz_mma): one CTA per SM, persistent over work items (an
// output tile of 128 x 64 and a range of K), 19 warps with fixed roles:
//  * warp 18, one thread: the copies of each stage, kStages stages ahead: A's
//    pre-tiled slice block in one bulk copy (cp.async.bulk), and for each of
//    the tile's two 32-column halves of B ("sets") the 1 KB pieces of all
//    digits in one 3-D tensor copy (cp.async.bulk.tensor), with mbarrier
//    transaction counts.
//  * warps 16 and 17, one thread each: the tcgen05.mma instructions of set 0
//    and set 1.  Each walks the stages in order with precomputed descriptors;
//    the stage buffer is released when both sets have committed to it.  A
//    single thread issuing both sets kept the tensor pipe about half as busy:
//    its scheduling work ran serially with the MMA issue.
//  * warps 0-7 and 8-15: the drains of set 0 and set 1.  The kSlices level
//    accumulators of a set live in TMEM (kSlices x 32 FP32 columns of 128
//    lanes; set c at columns 256 c).  Every kDrainK of K a set's eight warps
//    read them back with tcgen05.ld (warp w: lanes 32 (w % 4) .. + 31, 16 of
//    the set's columns, two levels per wait) and add them into two int64
//    fixed-point registers per output element: levels 0-3 in units of 2^-24
//    of level 0, levels 4-6 in units of 2^-48.
// The two sets drain kDrainK / 2 of K apart; while one set is drained the
// other set's thread keeps issuing, up to kStages - 1 stages ahead, so the
// tensor cores do not wait for the drains.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdint>
#include <type_traits>

#include "sep_ozaki.cuh"

namespace sep {
namespace oz {
namespace {

constexpr int kSets = 2;                                   // 32-column halves of a tile
constexpr int kSetN = kTileN / kSets;                      // 32
constexpr int kDrainWarps = 8 * kSets;                     // warps 0..15
constexpr int kDrainCols = kSetN / 2;                      // columns per drain thread
constexpr int kMmaWarp = kDrainWarps, kLoadWarp = kDrainWarps + kSets;  // a MMA warp per set
constexpr int kThreads = 32 * (kDrainWarps + kSets + 1);   // + the MMA and copy warps
constexpr int kStages = 4;
constexpr int kStageA = kSlices * kTileM * kChunkK * 2;    // 28672 bytes: one block
constexpr int kStageB = kSlices * kTileN * kChunkK * 2;    // 14336 bytes: 64 rows
constexpr int kStageBytes = kStageA + kStageB;             // 43008 bytes
constexpr uint32_t kRowGroupStride = 256;                  // bytes between 8-row groups
constexpr uint32_t kSliceBytes = 16 * 256;                 // one digit of a 128-row block
constexpr uint32_t kSetSliceBytes = (kSetN / 8) * 256;     // one digit of a set's 32 rows
constexpr int kTmemCols = 512;                              // set c: 256 c .. + 7 * 32
constexpr int kSetCols = 256;
constexpr int kStagesPerDrain = kDrainK / kChunkK;          // 8
constexpr long long kSpin = 1LL << 26;                      // bounded waits
constexpr int kL2Ahead = 8;  // stages between an operand block's L2 prefetch and its copy
static_assert(kSlices * kSetN <= kSetCols && kSets * kSetCols <= kTmemCols, "TMEM columns");
static_assert((kSlices * kSetN) % 16 == 0, "one MMA per digit of A and set");
static_assert((kSlices) * kDrainK * 16384LL < (1LL << 24), "exact FP32 level sums");

// ---- PTX wrappers ----------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

// true once the barrier's phase with the given parity has completed
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait; false (and *err set) if the phase never completes
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err, int code) {
  for (long long it = 0; it < kSpin; ++it)
    if (mbar_try(bar, parity)) return true;
  atomicCAS(err, 0, code);
  return false;
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

// 3-D tensor copy (B operand: the 7 digit pieces of one set, 1 KB each, 4 KB
// apart in global memory, consecutive in shared memory)
__device__ __forceinline__ void tensor3_g2s(uint32_t dst, const CUtensorMap* map, int c0, int c1,
                                            int c2, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, "
      "{%2, %3, %4}], [%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// shared memory matrix descriptor: K-major, no swizzle; LBO = byte distance of
// core matrices along K, SBO = along M/N; bits 46-48 = 0b001 (sm_100 family)
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo & 0x3FFFF) >> 4) << 16;
  d |= (uint64_t)((sbo & 0x3FFFF) >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor, kind::f16: D f32, A and B bf16, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
      : "memory");
}

// 32 lanes x 16 columns of 32-bit TMEM words: thread t of the warp gets lane
// (lane base + t), columns col .. col + 15
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&v)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]),
        "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// two loads of 16 columns (levels at a0 and a1) with one wait: the second
// load's latency runs under the first's
__device__ __forceinline__ void tmem_ld16x2(uint32_t a0, uint32_t a1, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%32];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%33];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
        "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
        "=r"(v[14]), "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]),
        "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]),
        "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(a0), "r"(a1)
      : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// ---- splitting -------------------------------------------------------------
// biased FP64 exponent field of x (0 for zero and denormals)
__device__ __forceinline__ int exp_field(double x) {
  return (int)((__double_as_longlong(x) >> 52) & 0x7FF);
}

// scale exponent of a row whose largest exponent field is ex: |x| < 2^e
__device__ __forceinline__ int scale_of(int ex_max) { return ex_max - 1022; }

// x 2^(55-e) rounded to an integer (|X| <= 2^55), split into kSlices balanced
// base-256 digits, most significant first; integer operations only
__device__ __forceinline__ void split7(double x, int e, int (&d)[kSlices]) {
  const long long bits = __double_as_longlong(x);
  const int ex = (int)((bits >> 52) & 0x7FF);
  long long X = 0;
  if (ex != 0) {
    const long long m = (bits & 0xFFFFFFFFFFFFFLL) | (1LL << 52);
    const int sh = 1020 + e - ex;  // X = m 2^-sh, sh >= -2
    if (sh <= 0)
      X = m << (-sh);
    else if (sh < 62)
      X = (m + (1LL << (sh - 1))) >> sh;
    if (bits < 0) X = -X;
  }
#pragma unroll
  for (int s = 0; s < kSlices - 1; ++s) {
    const int w = 8 * (kSlices - 1 - s);
    const long long q = (X + (1LL << (w - 1))) >> w;
    d[s] = (int)q;
    X -= q << w;
  }
  d[kSlices - 1] = (int)X;
}

__device__ __forceinline__ uint32_t bf16_pair(int lo, int hi) {
  return (__float_as_uint((float)lo) >> 16) | (__float_as_uint((float)hi) & 0xFFFF0000u);
}

// element offset of (row block rb, K chunk kc, slice s) + position (rr, kk) in it
__device__ __forceinline__ long long plane_off(int s, long long kc, long long rb, long long nkc,
                                               long long nrb, int rr, int kk) {
  (void)nrb;
  return (rb * nkc + kc) * kBlockElems + ((s * 16 + (rr >> 3)) * 2 + (kk >> 3)) * 64 +
         (rr & 7) * 8 + (kk & 7);
}

// eight consecutive K values of one row -> kSlices 16-byte stores
__device__ __forceinline__ void store_digits8(const double (&x)[8], int e, uint16_t* planes,
                                              long long kc, long long rb, long long nkc,
                                              long long nrb, int rr, int k0) {
  int d[8][kSlices];
#pragma unroll
  for (int i = 0; i < 8; ++i) split7(x[i], e, d[i]);
#pragma unroll
  for (int s = 0; s < kSlices; ++s) {
    uint4 v;
    v.x = bf16_pair(d[0][s], d[1][s]);
    v.y = bf16_pair(d[2][s], d[3][s]);
    v.z = bf16_pair(d[4][s], d[5][s]);
    v.w = bf16_pair(d[6][s], d[7][s]);
    *reinterpret_cast<uint4*>(planes + plane_off(s, kc, rb, nkc, nrb, rr, k0)) = v;
  }
}

// one block per (padded) row: the largest exponent field of the row
__global__ void k_row_expo(const double* __restrict__ X, long long rows, long long k,
                           long long ld, int* __restrict__ expo) {
  const long long r = blockIdx.x;
  int mx = 0;
  if (r < rows)
    for (long long g = threadIdx.x; g < k; g += blockDim.x) mx = max(mx, exp_field(X[r * ld + g]));
  __shared__ int red[32];
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x < 32) {
    mx = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0;
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (threadIdx.x == 0) expo[r] = (r < rows) ? scale_of(mx) : 0;
  }
}

// one block per (K chunk, row block): 64 rows x kChunkK values of K, eight
// consecutive K values per thread
constexpr int kSliceThreads = kBlockRows * kChunkK / 8;
__global__ void __launch_bounds__(kSliceThreads) k_slice_rows(const double* __restrict__ X, long long rows,
                                                    long long k, long long ld,
                                                    const int* __restrict__ expo,
                                                    uint16_t* __restrict__ planes, long long nkc,
                                                    long long nrb) {
  const long long kc = blockIdx.x, rb = blockIdx.y;
  const int rr = threadIdx.x / (kChunkK / 8), k0 = (threadIdx.x % (kChunkK / 8)) * 8;
  const long long row = rb * kBlockRows + rr;
  const long long g0 = kc * kChunkK + k0;
  double x[8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
    x[i] = (row < rows && g0 + i < k) ? X[row * ld + g0 + i] : 0.0;
  store_digits8(x, expo[row], planes, kc, rb, nkc, nrb, rr, k0);
}

// one thread per (padded) column g of X (kk x cols): exponent over the kk rows
__global__ void k_col_expo(const double* __restrict__ X, long long kk, long long cols,
                           long long ld, long long padded, int* __restrict__ expo) {
  for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < padded;
       g += (long long)gridDim.x * blockDim.x) {
    int mx = 0;
    if (g < cols)
      for (long long j = 0; j < kk; ++j) mx = max(mx, exp_field(X[j * ld + g]));
    expo[g] = (g < cols) ? scale_of(mx) : 0;
  }
}

// one block per (K chunk, row block) of the transpose: X rows j are the K
// index, X columns g the operand rows; staged through shared memory
__global__ void __launch_bounds__(kSliceThreads) k_slice_cols(const double* __restrict__ X, long long kk,
                                                    long long cols, long long ld,
                                                    const int* __restrict__ expo,
                                                    uint16_t* __restrict__ planes, long long nkc,
                                                    long long nrb) {
  __shared__ double tile[kChunkK][kBlockRows + 1];
  const long long kc = blockIdx.x, rb = blockIdx.y;
  for (int e = threadIdx.x; e < kChunkK * kBlockRows; e += blockDim.x) {
    const int j = e / kBlockRows, g = e % kBlockRows;
    const long long jj = kc * kChunkK + j, gg = rb * kBlockRows + g;
    tile[j][g] = (jj < kk && gg < cols) ? X[jj * ld + gg] : 0.0;
  }
  __syncthreads();
  const int rr = threadIdx.x / (kChunkK / 8), k0 = (threadIdx.x % (kChunkK / 8)) * 8;
  double x[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = tile[k0 + i][rr];
  store_digits8(x, expo[rb * kBlockRows + rr], planes, kc, rb, nkc, nrb, rr, k0);
}

// ---- the tensor-core contraction -------------------------------------------
struct MmaArgs {
  const uint16_t* A;
  long long a_nrb;
  const uint16_t* B;
  long long b_nrb;
  long long nkc;
  const int* ea;
  const int* eb;
  int tiles_m, tiles_n, sym, ntiles, nsplit;
  long long kc_per_split;
  long long* part;  // nsplit > 1: part[hi/lo][split][prow][pcol]
  long long prow, pcol;
  double* C;  // nsplit == 1: direct
  long long ldc, m, n;
  double alpha;
  int acc;  // add into C instead of overwriting it
  int* err;
};

// v 2^k without overflow of the intermediate power (k = ea + eb - 38)
__device__ __forceinline__ double pow2i(int k) {
  return (k < -1022) ? 0.0 : __longlong_as_double((long long)(k + 1023) << 52);
}
__device__ __forceinline__ double scale2(double v, int k) {
  const int k1 = k / 2;
  return v * pow2i(k1) * pow2i(k - k1);
}

__device__ __forceinline__ void tile_of(const MmaArgs& a, int t, int& tm, int& tn) {
  if (!a.sym) {
    tm = t / a.tiles_n;
    tn = t - tm * a.tiles_n;
    return;
  }
  // tiles with a column >= a row: tn >= (kTileM / kTileN) tm
  for (tm = 0; tm < a.tiles_m; ++tm) {
    const int first = (kTileM / kTileN) * tm;
    const int cnt = a.tiles_n > first ? a.tiles_n - first : 0;
    if (t < cnt) {
      tn = first + t;
      return;
    }
    t -= cnt;
  }
  tm = tn = 0;
}

// set c's level accumulators are drained after local stage st of an item
__device__ __forceinline__ bool drain_after(int c, int st, int nst) {
  return st == nst - 1 || ((st + (kStagesPerDrain / 2) * c) % kStagesPerDrain) ==
                              kStagesPerDrain - 1;
}

__device__ __forceinline__ void item_of(const MmaArgs& a, int item, int& split, int& tm, int& tn,
                                        long long& kc0, int& nst) {
  // split-major order: CTAs running together share K ranges (and L2 lines)
  split = item / a.ntiles;
  tile_of(a, item - split * a.ntiles, tm, tn);
  kc0 = split * a.kc_per_split;
  long long kc1 = kc0 + a.kc_per_split;
  if (kc1 > a.nkc) kc1 = a.nkc;
  nst = (int)(kc1 > kc0 ? kc1 - kc0 : 0);  // the host leaves no split empty
}

__global__ void __maxnreg__(96) k_oz_mma(const MmaArgs a, const __grid_constant__ CUtensorMap tmb) {
  extern __shared__ __align__(1024) uint8_t stage_mem[];
  __shared__ __align__(8) uint64_t bar_load[kStages];   // copies of a stage landed
  __shared__ __align__(8) uint64_t bar_free[kStages];   // both sets' products of a stage done
  __shared__ __align__(8) uint64_t bar_full[kSets];     // a set's period of products done
  __shared__ __align__(8) uint64_t bar_drained[kSets];  // a set's accumulators read back
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t smem0 = smem_u32(stage_mem);

  if (tid == 0) {
    for (int b = 0; b < kStages; ++b) {
      mbar_init(smem_u32(&bar_load[b]), 1);
      mbar_init(smem_u32(&bar_free[b]), kSets);
    }
    for (int c = 0; c < kSets; ++c) {
      mbar_init(smem_u32(&bar_full[c]), 1);
      mbar_init(smem_u32(&bar_drained[c]), 32 * kDrainWarps / kSets);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const int items = a.ntiles * a.nsplit;
  bool ok = true;

  if (warp == kLoadWarp) {
    // ---------------- copies ----------------
    if ((tid & 31) == 0) {
      long long gs = 0;  // global stage
      for (int item = blockIdx.x; item < items && ok; item += gridDim.x) {
        int split, tm, tn, nst;
        long long kc0;
        item_of(a, item, split, tm, tn, kc0, nst);
        const uint16_t* ablk = a.A + (long long)tm * a.nkc * kBlockElems;
        const uint16_t* bblk = a.B + (long long)(tn >> 1) * a.nkc * kBlockElems;
        // B pieces: 1 KB piece (tn & 1) * kSets + c of every digit of block
        // ((tn >> 1) nkc + kc), the tensor's third coordinate counting digits
        const int piece0 = (tn & 1) * kSets;
        const long long dig0 = (long long)(tn >> 1) * a.nkc * kSlices;
        for (int st = 0; st < nst && ok; ++st, ++gs) {
          const int b = (int)(gs % kStages);
          const long long kc = kc0 + st;
          if (kL2Ahead > 0 && st + kL2Ahead < nst) {  // warm L2 for a later stage
            prefetch_l2(ablk + (kc + kL2Ahead) * kBlockElems, (uint32_t)(kBlockElems * 2));
            prefetch_l2(bblk + (kc + kL2Ahead) * kBlockElems, (uint32_t)(kBlockElems * 2));
          }
          // the buffer's previous stage: both sets' products done
          if (gs >= kStages)
            ok = mbar_wait(smem_u32(&bar_free[b]), (uint32_t)((gs / kStages - 1) & 1), a.err, 2);
          if (!ok) break;
          const uint32_t base = smem0 + b * kStageBytes, bar = smem_u32(&bar_load[b]);
          mbar_expect_tx(bar, kStageBytes);
          bulk_g2s(base, ablk + kc * kBlockElems, kStageA, bar);
          // set c's 32 rows of every digit, digits consecutive: any run of
          // digits of one set is one operand of 32 rows per digit
#pragma unroll
          for (int c = 0; c < kSets; ++c)
            tensor3_g2s(base + kStageA + c * kSlices * kSetSliceBytes, &tmb, 0, piece0 + c,
                        (int)(dig0 + kc * kSlices), bar);
        }
      }
      // the last copies of every buffer land before the shared memory is released
      for (long long g = (gs > kStages ? gs - kStages : 0); g < gs; ++g)
        mbar_wait(smem_u32(&bar_load[g % kStages]), (uint32_t)((g / kStages) & 1), a.err, 4);
    }
  } else if (warp == kMmaWarp || warp == kMmaWarp + 1) {
    // ---------------- products: one thread per set ----------------
    // Each set's thread walks the stages in order: it waits for the stage's
    // copies, issues the set's kSlices MMAs and commits them to the stage
    // buffer's barrier (which the copy thread waits on, for both sets,
    // before it reuses the buffer, so a set runs at most kStages - 1 stages
    // ahead of the other).  Before the first stage of a period it waits for
    // the set's accumulators to be drained.
    auto products = [&](auto cc) {
      constexpr int c = decltype(cc)::value;
      // descriptors of stage buffer 0 (digit 0 of A, set c of B); a buffer
      // and a digit are fixed byte offsets added to the start-address field
      // (shared addresses < 2^18, so the 14-bit field never carries)
      const uint64_t da0 = smem_desc(smem0, 128, kRowGroupStride);
      const uint64_t db0 = smem_desc(smem0 + kStageA + c * kSlices * kSetSliceBytes, 128, kRowGroupStride);
      const uint32_t dt = tmem + (uint32_t)(c * kSetCols);
      long long g0 = 0;        // global stage index of the item's first stage
      uint32_t nf = 0, nd = 0;  // periods ended (bar_full commits), drains seen complete
      for (int item = blockIdx.x; item < items && ok; item += gridDim.x) {
        int split, tm, tn, nst;
        long long kc0;
        item_of(a, item, split, tm, tn, kc0, nst);
        for (int st = 0; st < nst; ++st) {
          const bool fresh = st == 0 || drain_after(c, st - 1, nst);
          if (fresh && nd < nf) {
            ok = mbar_wait(smem_u32(&bar_drained[c]), nd & 1, a.err, 3);
            if (!ok) break;
            ++nd;
          }
          const unsigned long long gs = (unsigned long long)(g0 + st);
          const uint32_t b = (uint32_t)(gs % kStages);
          ok = mbar_wait(smem_u32(&bar_load[b]), (uint32_t)((gs / kStages) & 1), a.err, 1);
          if (!ok) break;
          tc_fence_after();
          const uint64_t so = (uint64_t)((b * (uint32_t)kStageBytes) >> 4);
          // digit s of A times digits 0 .. kSlices-1-s of B: the accumulators
          // of levels s .. kSlices-1, adjacent in TMEM
#pragma unroll
          for (int s = 0; s < kSlices; ++s)
            mma_bf16(dt + (uint32_t)(s * kSetN), da0 + so + (uint64_t)((s * kSliceBytes) >> 4),
                     db0 + so, idesc_bf16(kTileM, (kSlices - s) * kSetN),
                     (fresh && s == 0) ? 0u : 1u);
          mma_commit(smem_u32(&bar_free[b]));
          if (drain_after(c, st, nst)) {
            mma_commit(smem_u32(&bar_full[c]));
            ++nf;
          }
        }
        g0 += nst;
      }
      // the last drain before the accumulators are released
      while (ok && nd < nf) {
        ok = mbar_wait(smem_u32(&bar_drained[c]), nd & 1, a.err, 5);
        if (ok) ++nd;
      }
    };
    if ((tid & 31) == 0) {
      if (warp == kMmaWarp)
        products(std::integral_constant<int, 0>{});
      else
        products(std::integral_constant<int, 1>{});
    }
  } else {
    // ---- drains: set c = warp / 8, lanes 32 (warp % 4) .. + 31, columns
    // kDrainCols h .. + kDrainCols-1 of the set, h = (warp / 4) % 2 ----
    const int c = warp / 8, h = (warp / 4) & 1;
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
    uint32_t nfull_seen = 0;
    for (int item = blockIdx.x; item < items && ok; item += gridDim.x) {
      int split, tm, tn, nst;
      long long kc0;
      item_of(a, item, split, tm, tn, kc0, nst);
      long long Rh[kDrainCols], Rl[kDrainCols];
#pragma unroll
      for (int j = 0; j < kDrainCols; ++j) Rh[j] = Rl[j] = 0;
      for (int st = 0; st < nst && ok; ++st) {
        if (!drain_after(c, st, nst)) continue;
        ok = mbar_wait(smem_u32(&bar_full[c]), nfull_seen & 1, a.err, 6);
        if (!ok) break;
        ++nfull_seen;
        tc_fence_after();
        const uint32_t t0 = tmem + lane_base + (uint32_t)(c * kSetCols + h * kDrainCols);
        // levels in pairs, two loads in flight per wait
#pragma unroll
        for (int l0 = 0; l0 < kSlices; l0 += 2) {
          uint32_t v[2 * kDrainCols];
          if (l0 + 1 < kSlices) {
            tmem_ld16x2(t0 + (uint32_t)(l0 * kSetN), t0 + (uint32_t)((l0 + 1) * kSetN), v);
          } else {
            uint32_t (&v0)[kDrainCols] = *reinterpret_cast<uint32_t(*)[kDrainCols]>(v);
            tmem_ld16(t0 + (uint32_t)(l0 * kSetN), v0);
          }
#pragma unroll
          for (int q = 0; q < 2; ++q) {
            const int l = l0 + q;
            if (l < kSlices) {
#pragma unroll
              for (int j = 0; j < kDrainCols; ++j) {
                const long long w =
                    (long long)__float2int_rn(__uint_as_float(v[q * kDrainCols + j]));
                if (l <= 3)
                  Rh[j] += w << (24 - 8 * l);
                else
                  Rl[j] += w << (48 - 8 * l);
              }
            }
          }
        }
        tc_fence_before();
        mbar_arrive(smem_u32(&bar_drained[c]));
      }
      if (!ok) break;
      // output row 32 (warp % 4) + lane, columns 32 c + 16 h .. + 15 of tile (tm, tn)
      const long long i = (long long)tm * kTileM + (warp & 3) * 32 + (tid & 31);
      const long long j0 = (long long)tn * kTileN + c * kSetN + h * kDrainCols;
      if (a.nsplit > 1) {
        long long* dh = a.part + ((long long)split * a.prow + i) * a.pcol + j0;
        long long* dl = dh + (long long)a.nsplit * a.prow * a.pcol;
#pragma unroll
        for (int j = 0; j < kDrainCols; j += 2) {
          *reinterpret_cast<longlong2*>(dh + j) = make_longlong2(Rh[j], Rh[j + 1]);
          *reinterpret_cast<longlong2*>(dl + j) = make_longlong2(Rl[j], Rl[j + 1]);
        }
      } else if (i < a.m) {
        const int ei = a.ea[i];
#pragma unroll
        for (int jj = 0; jj < kDrainCols; ++jj) {
          const long long j = j0 + jj;
          if (j < a.n && (!a.sym || j >= i)) {
            const double r = (double)Rh[jj] + (double)Rl[jj] * 0x1p-24;
            const double v = scale2(a.alpha * r, ei + a.eb[j] - 38);
            a.C[i * a.ldc + j] = a.acc ? a.C[i * a.ldc + j] + v : v;
            if (a.sym && j > i) a.C[j * a.ldc + i] = a.acc ? a.C[j * a.ldc + i] + v : v;
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(kTmemCols)
                 : "memory");
}

// C = alpha 2^(ea + eb - 38) (hi + lo 2^-24), hi and lo the integer sums of
// the split-K partials
__global__ void k_oz_reduce(const long long* __restrict__ part, int nsplit, long long prow,
                            long long pcol, const int* __restrict__ ea,
                            const int* __restrict__ eb, long long m, long long n, double alpha,
                            int sym, int acc, double* __restrict__ C, long long ldc) {
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < m * n;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long i = idx / n, j = idx - i * n;
    long long ii = i, jj = j;
    if (sym && j < i) {
      ii = j;
      jj = i;
    }
    long long sh = 0, sl = 0;
    const long long lo = (long long)nsplit * prow * pcol;
    for (int sp = 0; sp < nsplit; ++sp) {
      const long long o = ((long long)sp * prow + ii) * pcol + jj;
      sh += part[o];
      sl += part[lo + o];
    }
    const double v = scale2(alpha * ((double)sh + (double)sl * 0x1p-24), ea[ii] + eb[jj] - 38);
    C[i * ldc + j] = acc ? C[i * ldc + j] + v : v;
  }
}

}  // namespace
}  // namespace oz
}  // namespace sep

// ---- host side ---------------------------------------------------------------
namespace sep {
namespace oz {

namespace {
long long cdiv(long long a, long long b) { return (a + b - 1) / b; }
long long padded_blocks(long long rows) { return cdiv(rows, kBlockRows); }  // 128-row blocks
int sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
  return n > 0 ? n : 1;
}
int tile_count(long long m, long long n, bool sym) {
  const int tmc = (int)cdiv(m, kTileM), tnc = (int)cdiv(n, kTileN);
  if (!sym) return tmc * tnc;
  int t = 0;
  constexpr int r = kTileM / kTileN;
  for (int tm = 0; tm < tmc; ++tm) t += tnc > r * tm ? tnc - r * tm : 0;
  return t;
}
// Tensor map of B's digit planes as 1 KB pieces (32 rows x 16 K of one
// digit): dimension 0 the 128 8-byte words of a piece, dimension 1 the four
// pieces of a digit's 128 rows (1 KB apart), dimension 2 the digits of all
// blocks in order (4 KB apart).  A box {128, 1, kSlices} is the run of one
// set's pieces over all digits of a block.
cudaError_t b_pieces_map(const Planes& B, CUtensorMap* map) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    cudaDriverEntryPointQueryResult q;
    void* fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn)
      return cudaErrorNotSupported;
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  const cuuint64_t dims[3] = {128, 4, (cuuint64_t)(B.nrb * B.nkc * kSlices)};
  const cuuint64_t strides[2] = {1024, 4096};
  const cuuint32_t box[3] = {128, 1, (cuuint32_t)kSlices};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, B.d, dims, strides, box, estr,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}
}  // namespace

size_t plane_elems(long long rows, long long k) {
  return (size_t)cdiv(k, kChunkK) * (size_t)padded_blocks(rows) * kBlockElems;
}

cudaError_t slice_rows(const double* X, long long rows, long long k, long long ld, Planes& p,
                       cudaStream_t s) {
  p.rows = rows;
  p.k = k;
  p.nrb = padded_blocks(rows);
  p.nkc = cdiv(k, kChunkK);
  if (p.nkc > 0x7fffffffLL || p.nrb > 65535) return cudaErrorInvalidValue;
  k_row_expo<<<(unsigned)(p.nrb * kBlockRows), 256, 0, s>>>(X, rows, k, ld, p.expo);
  k_slice_rows<<<dim3((unsigned)p.nkc, (unsigned)p.nrb), kSliceThreads, 0, s>>>(X, rows, k, ld, p.expo,
                                                                      p.d, p.nkc, p.nrb);
  return cudaGetLastError();
}

cudaError_t slice_cols(const double* X, long long kk, long long cols, long long ld, Planes& p,
                       cudaStream_t s) {
  p.rows = cols;
  p.k = kk;
  p.nrb = padded_blocks(cols);
  p.nkc = cdiv(kk, kChunkK);
  if (p.nkc > 0x7fffffffLL || p.nrb > 65535) return cudaErrorInvalidValue;
  const long long padded = p.nrb * kBlockRows;
  k_col_expo<<<(unsigned)std::min<long long>(cdiv(padded, 256), 152LL * 16), 256, 0, s>>>(
      X, kk, cols, ld, padded, p.expo);
  k_slice_cols<<<dim3((unsigned)p.nkc, (unsigned)p.nrb), kSliceThreads, 0, s>>>(X, kk, cols, ld, p.expo,
                                                                      p.d, p.nkc, p.nrb);
  return cudaGetLastError();
}

size_t part_elems(long long m, long long n, int nsplit) {
  if (nsplit <= 1) return 0;
  return 2 * (size_t)nsplit * (size_t)(cdiv(m, kTileM) * kTileM) *
         (size_t)(cdiv(n, kTileN) * kTileN);
}

int choose_splits(long long m, long long n, long long k, bool sym) {
  // enough items for every SM, and the item count close to a multiple of the
  // SM count (items run in waves of one per SM); each split covers at least
  // two drain periods of K
  const long long tiles = tile_count(m, n, sym);
  const long long nkc = cdiv(k, kChunkK);
  const long long sms = sm_count();
  const long long cap = std::max<long long>(1, nkc / (2 * (kDrainK / kChunkK)));
  long long best = 1;
  double best_eff = -1.0;
  for (long long ns = 1; ns <= std::min<long long>(cap, 8 * cdiv(sms, tiles)); ++ns) {
    const long long items = tiles * ns;
    const long long waves = cdiv(items, sms);
    const double eff = (double)items / (double)(waves * sms);
    // prefer balance, then fewer splits (less split-K traffic)
    if (eff > best_eff + 0.02) {
      best_eff = eff;
      best = ns;
    }
  }
  return (int)best;
}

cudaError_t gemm_nt(const Planes& A, const Planes& B, double alpha, bool sym, bool accumulate,
                    double* C, long long ldc, long long* part, int nsplit, int* err,
                    cudaStream_t s) {
  if (A.nkc != B.nkc || A.k != B.k) return cudaErrorInvalidValue;
  if (nsplit > 1 && !part) return cudaErrorInvalidValue;
  static bool attr_set[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 0 && dev < 64 && !attr_set[dev]) {
    e = cudaFuncSetAttribute(k_oz_mma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             kStages * kStageBytes);
    if (e != cudaSuccess) return e;
    attr_set[dev] = true;
  }
  MmaArgs a{};
  a.A = A.d;
  a.a_nrb = A.nrb;
  a.B = B.d;
  a.b_nrb = B.nrb;
  a.nkc = A.nkc;
  a.ea = A.expo;
  a.eb = B.expo;
  a.m = A.rows;
  a.n = B.rows;
  a.tiles_m = (int)cdiv(A.rows, kTileM);
  a.tiles_n = (int)cdiv(B.rows, kTileN);
  a.sym = sym ? 1 : 0;
  a.ntiles = tile_count(A.rows, B.rows, sym);
  a.nsplit = nsplit < 1 ? 1 : nsplit;
  a.kc_per_split = cdiv(A.nkc, a.nsplit);
  // no split without K chunks: every split writes its partial sums
  a.nsplit = (int)cdiv(A.nkc, a.kc_per_split);
  a.part = part;
  a.prow = (long long)a.tiles_m * kTileM;
  a.pcol = (long long)a.tiles_n * kTileN;
  a.C = C;
  a.ldc = ldc;
  a.alpha = alpha;
  a.acc = accumulate ? 1 : 0;
  a.err = err;
  const long long items = (long long)a.ntiles * a.nsplit;
  if (items < 1) return cudaSuccess;
  CUtensorMap tmb;
  e = b_pieces_map(B, &tmb);
  if (e != cudaSuccess) return e;
  const unsigned grid = (unsigned)std::min<long long>(items, sm_count());
  k_oz_mma<<<grid, kThreads, kStages * kStageBytes, s>>>(a, tmb);
  e = cudaGetLastError();
  if (e != cudaSuccess || a.nsplit == 1) return e;
  const long long mn = A.rows * B.rows;
  k_oz_reduce<<<(unsigned)std::min<long long>(cdiv(mn, 256), 152LL * 8), 256, 0, s>>>(
      part, a.nsplit, a.prow, a.pcol, A.expo, B.expo, A.rows, B.rows, alpha, a.sym, a.acc, C, ldc);
  return cudaGetLastError();
}

cudaError_t check_status(const int* err, cudaStream_t s, int* host_status) {
  cudaError_t e = cudaMemcpyAsync(host_status, err, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e;
}

}  // namespace oz
}  // namespace sep
