// FP64-accurate GEMM on the BF16 tensor cores by exact digit splitting (the Ozaki
// scheme: K. Ozaki, T. Ogita, S. Oishi, S. M. Rump, "Error-free transformations of
// matrix multiplication by using fast routines of matrix multiplication and its
// applications", Numer. Algorithms 59 (2012)).
//
// Every row of A (every column of B) is scaled by a power of two 2^e so that its
// entries lie in (-1, 1), and the scaled value is cut into kOzSlices signed digits of
// kOzBits bits: x = 2^e sum_i d_i 2^(-kOzBits i), |d_i| <= 63, each exactly a BF16.
// A digit product sum_k a_i(m,k) b_j(k,n) is an integer below 2^24 in magnitude when K
// is cut into chunks of kOzChunkTiles K tiles, so the FP32 tensor-memory accumulator
// holds it exactly; the digit pairs of one level l = i + j share an accumulator.
// Levels up to kOzSlices + 1 are kept (45 digit products); the dropped tail is below
// 2^-52 of K max|A(m,.)| max|B(.,n)|.  The levels of one chunk are combined in two
// 64-bit integers and converted to FP64 once.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace ccx {

constexpr int kOzSlices = 9;       // digits per operand
constexpr int kOzBits = 6;         // bits per digit
constexpr int kOzLevels = kOzSlices;  // levels 2 .. kOzSlices + 1
constexpr int kOzN = 32;           // columns per CTA: kOzLevels accumulators at 32-column offsets
constexpr int kOzChunkTiles = 7;   // K tiles (64 each) per exact accumulation chunk

// Digit planes of one operand in the canonical K-major tiling of the split-precision
// kernel (A: 128-row tiles, B: npad-row tiles), plane p at planes + p * plane_elems.
struct OzProb {
  const uint16_t *A;   // A digit planes of this problem (first tile of plane 0)
  const int *eA;       // row exponents of A (M)
  const uint16_t *B;   // B digit planes of this problem
  const int *eB;       // column exponents of B (N)
  int64_t a_plane, b_plane;  // elements between digit planes
  int M, N, nk, npad;
  double *C;           // C(m, n) += alpha * (A B)(m, n) at C[m * sCm + n * sCn]
  int64_t sCm, sCn;
  double alpha;
};
struct OzTile {
  int prob, mt, n0;    // 128-row tile mt, columns n0 .. n0 + min(kOzN, npad - n0)
};
// error codes written to *err: 1 load wait, 2 MMA wait, 3 drain wait timed out, 4 bad shape
void launch_oz_gemm(const OzProb *probs, const OzTile *tiles, int ntiles, int *err, cudaStream_t st);

// Exponents and digit planes of an FP64 matrix (rows x cols, element (r, k) at
// src[r * sr + k * sk]), tiled like TcSplitJob (tile_rows 128 for A, npad for B).
struct OzSplitJob {
  const double *src;
  int64_t sr, sk;
  int rows, cols, tile_rows, nk, rows_pad;
  uint16_t *planes;
  int64_t plane_elems;
  int *exps;           // rows exponents (written by the exponent pass, read by the digit pass)
};
std::vector<int4> oz_split_chunks(const std::vector<OzSplitJob> &jobs);
// exps: one warp per row; rowtab: (job, row) pairs; chunks as the split kernel's (the
// digit planes are zeroed once when allocated)
void launch_oz_split(const OzSplitJob *jobs, const int2 *rowtab, int nrows, const int4 *chunks, int nchunks,
                     cudaStream_t st);
std::vector<int2> oz_row_table(const std::vector<OzSplitJob> &jobs);

}  // namespace ccx
