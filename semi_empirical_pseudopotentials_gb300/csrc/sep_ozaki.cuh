// sep_ozaki.cuh -- FP64-accurate contractions of the subspace stages on the
// tcgen05 tensor cores.
//
// The Gram, projection and rotation products of the orthogonalisation
// (filter/ortho.c:11-52) and of Rayleigh-Ritz (filter/Hmat.c:11-86) are dense
// state-by-grid contractions.  On GB300 the FP64 pipe gives about 1.25
// TFLOP/s, while the bf16 tensor cores give about 2 PFLOP/s.  These routines
// compute the products to FP64 accuracy on the bf16 tensor cores by exact
// splitting (the Ozaki scheme):
//
//  * Each row (or, for the rotation's grid operand, each column) of an
//    operand gets a power-of-two scale 2^e with |x| < 2^e.  Every element is
//    rounded to a 55-bit fixed-point integer X = round(x 2^(55-e)) and split
//    into kSlices balanced base-256 digits d_s in [-128, 128]:
//    X = sum_s d_s 2^(8 (kSlices-1-s)).  A digit is exact in bf16.
//  * Products of digits are exact (|d d'| <= 2^14).  The tensor core sums
//    them in FP32 for at most kDrainK values of K per level l = s + t, and
//    (l + 1) kDrainK 2^14 < 2^24, so every partial sum is an exact integer.
//  * Each level's exact sum is drained from TMEM into two 64-bit fixed-point
//    accumulators held in registers (levels 0-3 in units of 2^-24 of level
//    0, levels 4-6 in units of 2^-48), and split-K partials are added as
//    integers: the result does not depend on the order of the additions.
//  * Levels l >= kSlices are dropped: the error is below 2^-53 of the
//    product of the two row maxima, per term, like an FP64 product.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace sep {
namespace oz {

constexpr int kSlices = 7;          // digits per value (55 bits)
constexpr int kTileM = 128;         // rows of A per tile (TMEM lanes)
constexpr int kTileN = 64;          // rows of B per tile (two sets of 32 TMEM columns per level)
constexpr int kChunkK = 16;         // K per pipeline stage (one MMA per digit pair)
constexpr int kBlockRows = 128;     // rows per pre-tiled block in global memory
constexpr int kDrainK = 128;        // K accumulated per level before a drain
constexpr int kBlockElems = kSlices * kBlockRows * kChunkK;  // 14336 bf16: all digits of a block

// Pre-tiled digit planes of one operand.  Row block rb (128 rows) and K chunk
// kc (16 values) hold all kSlices digits in one 28,672-byte block, in the
// tensor cores' K-major no-swizzle layout, digit-major: the 8x8 core matrix of
// digit s, row group i (0..15), K group j (0..1) at ((s * 16 + i) * 2 + j) *
// 128 bytes, row r of it at r * 16 bytes.  So a block is one contiguous copy,
// digit s of it a matrix with row-group stride 256 bytes starting s * 4096
// bytes in, and each 32 rows of a digit one 1024-byte piece.
// Element offset (uint16) of (row rr of the block, k, digit s):
//   (rb * nkc + kc) * 14336 + ((s * 16 + i) * 2 + j) * 64 + r * 8 + (k % 8).
struct Planes {
  uint16_t* d = nullptr;  // nrb * nkc * 14336 values
  int* expo = nullptr;    // scale exponent per row (nrb * 128 entries)
  long long rows = 0, k = 0;
  long long nrb = 0, nkc = 0;
};

size_t plane_elems(long long rows, long long k);  // uint16 values of one operand

// Slices of the rows of X (rows x k, leading dimension ld): row scaling.
cudaError_t slice_rows(const double* X, long long rows, long long k, long long ld, Planes& p,
                       cudaStream_t s);
// Slices of the transpose of X (kk x cols, leading dimension ld): operand row
// g = column g of X, its K index = row of X; column scaling.
cudaError_t slice_cols(const double* X, long long kk, long long cols, long long ld, Planes& p,
                       cudaStream_t s);

// C (m x n, leading dimension ldc) = alpha A B^T for sliced A (m rows) and B
// (n rows) over the same K.  sym: A and B are the same operand; only tiles on
// or above the diagonal are computed and the result is mirrored.  accumulate:
// C += alpha A B^T.  part: int64 split-K partials (part_elems(...) values,
// unused when nsplit == 1).  err: device int, set non-zero if a wait inside
// the kernel runs out.
size_t part_elems(long long m, long long n, int nsplit);
int choose_splits(long long m, long long n, long long k, bool sym);
cudaError_t gemm_nt(const Planes& A, const Planes& B, double alpha, bool sym, bool accumulate,
                    double* C, long long ldc, long long* part, int nsplit, int* err,
                    cudaStream_t s);

// Launch-level check of the kernel's device-side status word (err).
cudaError_t check_status(const int* err, cudaStream_t s, int* host_status);

}  // namespace oz
}  // namespace sep
