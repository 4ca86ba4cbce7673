// Tensor-core (tcgen05) split-precision GEMM: C(fp64) += alpha * A B with A, B given
// as hi/lo pairs of BF16 (or TF32) in a pre-tiled K-major layout.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace ccx {

// Pre-tiled operand layout (both operands K-major, 128-byte K tiles):
//   A (M x K): tile (mt, kt) of 128 rows x 128 bytes of K at element offset
//              (mt * nk + kt) * 128 * kTileK, rows padded to a multiple of 128;
//   B (N x K): tile kt of npad rows x 128 bytes at element offset kt * npad * kTileK.
// Inside a tile the rows form 8-row groups of eight 8x16-byte core matrices along K:
//   byte offset of (row, kbyte) = ((row/8)*8 + kbyte/16)*128 + (row%8)*16 + kbyte%16,
// i.e. the canonical SWIZZLE_NONE K-major layout with LBO = 128 B, SBO = 1024 B.
enum TcKind { kTcBF16 = 0, kTcTF32 = 1 };

// A further product accumulated into the same output tile (same M, N): its own operands
// and K-tile count, optionally subtracted (the MMAs negate B).
struct TcSeg {
  const void *Ahi, *Alo, *Bhi, *Blo;
  int nk;
  int64_t bstride;  // as TcProb::bstride
  int neg;          // 1: the product is subtracted
};
constexpr int kTcMaxSegs = 6;  // products per output tile (the problem's own and ext)

struct TcProb {
  const void *Ahi, *Alo;  // pre-tiled A (this problem), nullptr Alo: A taken as hi only
  const void *Bhi, *Blo;  // pre-tiled B
  int M, N, nk, npad;     // rows, columns, K tiles, padded columns (multiple of 16, <= 256)
  double *C;              // C(m, n) at C[m * sCm + n * sCn]
  int64_t sCm, sCn;
  double alpha;
  int64_t bstride;        // bytes between B K tiles (0: npad * 128, the whole B operand); a
                          // column block of a wider B points Bhi/Blo at its first row and
                          // steps by the full operand's K-tile size
  TcSeg ext[kTcMaxSegs - 1];  // further products into the same accumulator (next of them)
  int next;
  const double *C0;       // optional term added once, at C's strides
  int overwrite;          // 1: C = C0 + alpha acc; 0: C += C0 + alpha acc
};
struct TcTile {
  int prob, mt;
};

// elements of one 128-byte K tile row
inline int tc_tile_k(int kind) { return kind == kTcBF16 ? 64 : 32; }

// error codes written to *err (0 = ok): 1 load wait timed out, 2 MMA wait timed out,
// 3 final wait timed out, 4 bad problem (npad > 256 or not a multiple of 16, no K tiles)
// max_nk: largest K-tile count (all segments) among the tiles (unused: the persistent
// kernel's stage ring runs on across tiles).  wait_budget: clock cycles each pipeline
// wait may take before the kernel gives up with an error code (<= 0: the default of
// about 2 s); the final waits for copies and MMAs in flight always keep the default.
void launch_tc_gemm(int kind, const TcProb *probs, const TcTile *tiles, int ntiles, int npad_max, int max_nk, int *err,
                    cudaStream_t st, long long wait_budget = 0);
// shared-memory stages launch_tc_gemm uses for tiles up to npad_max columns
int tc_stages(int npad_max);

// FP64 matrix (rows x cols, element (r, k) at src[r*sr + k*sk], optionally minus sub at
// the same strides, or plus sub (one FP64 addition) when add is 1) -> pre-tiled hi/lo
// pair, zero padded.  add = 2: src itself into hi/lo and src + sub into hi2/lo2 (two
// operands of the same tile geometry from one read of src).
// tile_rows = 128 for an A operand, npad for a B operand; nk = ceil(cols / tile_k).
struct TcSplitJob {
  const double *src, *sub;
  int64_t sr, sk;
  int rows, cols, tile_rows, nk, rows_pad, add;
  void *hi, *lo, *hi2, *lo2;
};
// Work list of the split kernels: (job, first unit, end unit) per block, at most
// kSplitChunk 16-byte units, covering only the row groups of each tile that hold rows of
// the matrix.  Units of all-padding row groups are never written: the tile buffers are
// zeroed once when they are allocated.
constexpr int kSplitChunk = 1024;
void split_ranges(int job, int rows, int rows_pad, int tile_rows, int nk, std::vector<int4> &out);
std::vector<int4> tc_split_chunks(const std::vector<TcSplitJob> &jobs);
void launch_tc_split(int kind, const TcSplitJob *jobs, const int4 *chunks, int nchunks, cudaStream_t st);

// Split once, place many times.  An operand whose entries are signed copies of one
// packed vector (T' and its particle-hole rearrangement T_ph hold every packed amplitude
// up to four times, in two tilings each) is split once into packed hi/lo arrays, and
// each tiled operand is then filled by a gather through a per-element map parallel to
// the tile buffer: m > 0 takes packed entry m - 1, m < 0 its negation, 0 a zero.
//
// Map building, once per layout: element (r, k) of a TcSplitJob-shaped region maps to
// ind ? ind[base + r sr + k sk] : base + r sr + k sk + 1 (indices in scalar elements).
struct TcMapJob {
  int64_t base, sr, sk;
  int rows, cols, tile_rows, nk, rows_pad;
  const int32_t *ind;
  int32_t *map;  // parallel to the tile region: element j of unit u at map[u * per16 + j]
};
void launch_tc_build_map(int kind, const TcMapJob *jobs, const int4 *chunks, int nchunks, cudaStream_t st);
// the gather: unit u of job j from its map and the packed arrays of its scalar component
struct TcGatherJob {
  const int32_t *map;
  const void *phl;  // packed hi/lo pairs: BF16 hi | lo << 16 (32 bits), TF32 hi | lo << 32 (64 bits)
  void *hi, *lo;    // tile region
};
void launch_tc_gather(int kind, const TcGatherJob *jobs, const int4 *chunks, int nchunks, cudaStream_t st);
// packed split of src - sub, n entries at a stride of `stride` doubles (the scalar
// components of complex data are split as separate vectors by their offsets)
void launch_tc_split_packed(int kind, const double *src, const double *sub, int64_t n, int stride, void *phl,
                            cudaStream_t st);

}  // namespace ccx
