// Host-callable launchers of the CCD kernels (implemented in kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"
#include "devlayout.hpp"

namespace ccx {

// ---- grouped GEMM (FP64 / complex FP64) ------------------------------------
// C(m,n) [+]= sum_s alpha_s * sum_k A_s(m,k) B_s(k,n), element strides per operand.
template <typename S>
struct GemmSeg {
  const S *A, *B;
  int64_t sAm, sAk, sBk, sBn;
  int K;
  double alpha;
};
template <typename S>
struct GemmProb {
  GemmSeg<S> seg[2];
  int nseg;
  int M, N;
  S *C;
  const S *C0;  // initial value when accumulate == 0 (nullptr: zero)
  int64_t sCm, sCn;
  int accumulate;
  int kchunk;   // > 0: split-K over one segment; tile.kslice picks the chunk
  S *part;      // split-K partial products, kslice-major, each M x N column-major
};
struct GemmTile {
  int prob, m0, n0, kslice;
};
constexpr int kGemmBK = 16;
// two tile shapes: 64x64 (4x4 per thread) and 128x32 (8x2 per thread, for N <= 32)
enum GemmShape { kShape64x64 = 0, kShape128x32 = 1 };
inline int gemm_bm(int shape) { return shape == kShape64x64 ? 64 : 128; }
inline int gemm_bn(int shape) { return shape == kShape64x64 ? 64 : 32; }

template <typename S>
void launch_gemm(int shape, const GemmProb<S> *probs, const GemmTile *tiles, int ntiles, cudaStream_t st);
// C = (accumulate ? C : C0 or 0) + sum over the split-K partials, fixed order
template <typename S>
void launch_splitk_reduce(const GemmProb<S> *probs, const int *plist, int n, cudaStream_t st);

// ---- potentials -----------------------------------------------------------
struct DevPotential {
  int kind;            // 0 Minnesota, 1 chiral-like
  int f32_literals;
  double lec[9];       // CS, CT, C1..C7 (MeV units)
};

// ---- residual pieces --------------------------------------------------------
template <typename S> void launch_gather_tph(const DevLayout &L, const S *T, S *Tph, cudaStream_t st);
// where each T_ph entry comes from: +/-(packed T' index + 1), 0 for a zero entry
void launch_tph_map(const DevLayout &L, int32_t *map, cudaStream_t st);
// X' = V_hhpp'^T T' per channel; work items (channel, first row, first column, 0)
constexpr int kXM = 32, kXJ = 8, kXK = 256;
constexpr int kXSlice = 512;  // K per X work item: long channels are split, partials summed in order
// X = V_hhpp'^T T' as K-sliced column-dot items into partial slots, then the slices
// summed in order (work and groups built by the engine)
template <typename S>
void launch_xdot(const DevLayout &L, const int4 *work, int nwork, const int4 *groups, int ngroups, const S *V,
                 const S *T, S *part, S *X, cudaStream_t st);
template <typename S> void launch_i7(const DevLayout &L, const S *X, const S *fdiag, const S *f7, S *d2ij, S *i7off, cudaStream_t st);
template <typename S> void launch_i9(const DevLayout &L, int64_t n, const S *Vhh, const S *X, S *I9, cudaStream_t st);
// I7 without X: the X entries it reads as 2 A^2 column dots of V_hhpp' and T' into xd
// (2 A^2 scalars), then summed as launch_i7 does
template <typename S>
void launch_i7_direct(const DevLayout &L, const S *V, const S *T, S *xd, const S *fdiag, const S *f7, S *d2ij, S *i7off,
                      cudaStream_t st);
// I9 = Vhh + (Xb + dX), n entries
template <typename S> void launch_i9b(int64_t n, const S *Vhh, const S *Xb, const S *dX, S *I9, cudaStream_t st);
// I6 in two passes; rowtile: (channel, first packed pp row) per block of kI6Rows rows;
// D: 3 values per packed row, at 3 * (t_off[ch] + row)
constexpr int kI6Rows = 128;
constexpr int kI6Parts = 4;  // threads per row: interleaved slices of the hole-pair sum
template <typename S> void launch_i6(const DevLayout &L, const int2 *rowtile, int nrowtile, S *D, const S *T, const S *Vhp,
                                     const S *fdiag, const S *f6, S *d2ab, S *i6off, cudaStream_t st);
// R' initialisation; omap / rmap (int4 per packed amplitude) from launch_rinit_maps.
// The ring term gathered from Rph is stored per amplitude into ring_out when given, and
// ring_base (per amplitude) is added to it when given: a ring split as R_ph,b + dR_ph.
void launch_rinit_maps(const DevLayout &L, int4 *omap, int4 *rmap, cudaStream_t st);
template <typename S>
void launch_rinit(const DevLayout &L, const int4 *omap, const int4 *rmap, const S *T, const S *Vhp, const S *Rph,
                  const S *i6off, const S *i7off, const S *ring_base, S *ring_out, S *R, cudaStream_t st);

// ---- update / energy / norms (per-block partial sums, then a fixed-order finish) --
// mode 0: reference update T <- 0.75 T + 0.25 R/D, history column written
// mode 1: Jacobi T_jac = R/D into hist_t, step into hist_e, T untouched
// mode 2: energy only (no update); mode 3: residual norm + energy, no update
// the DIIS step vectors of the standard mode: the step is computed to FP32 accuracy and
// stored in FP32 (real engines) or as FP32 (re, im) pairs (complex engines)
struct __align__(8) cplxf {
  float re, im;
};
template <typename S> struct StepOf;
template <> struct StepOf<double> { using type = float; };
template <> struct StepOf<cplx> { using type = cplxf; };
template <typename S>
void launch_update(const DevLayout &L, int mode, S *T, const S *R, const S *Vhp, const S *d2ij, const S *d2ab,
                   S *hist_t, typename StepOf<S>::type *hist_e, double *partial, double *out4, cudaStream_t st);
// dot products: out[j] = sum_x w(a[x]) * b_j[x] for j < nb; conj on a when conj_a
template <typename S>
void launch_dots(int64_t n, const S *a, const S *const *bs, int nb, int conj_a, double *partial, double *out, cudaStream_t st);
// mode-1 update and the Gram row of its step in one pass:
// out[0] = E (re), out[1] = E (im, 0 for real engines), out[2] = |R - D T|^2, out[3] = *err (0 when err is null),
// out[4 + j] = Re(conj(step) . es[j]) for j < nb (1 <= nb <= 16); es[self] is hist_e, the step
// this pass writes.  partial holds 20 doubles for each of up to 608 blocks.
template <typename S>
void launch_update_std(const DevLayout &L, const S *T, const S *R, const S *Vhp, const S *d2ij, const S *d2ab, S *hist_t,
                       typename StepOf<S>::type *hist_e, const typename StepOf<S>::type *const *es, int nb, int self,
                       const int *err, double *partial, double *out, cudaStream_t st);
// reference DIIS Gram matrix of differences of nstep history columns (no conjugation)
template <typename S>
void launch_diis_gram(int64_t n, const S *const *cols, int nstep, double *partial, double *out, cudaStream_t st);
// y = sum_i c_i x_i
template <typename S>
void launch_combine(int64_t n, const S *const *xs, const double *coef /* host, 2 per term */, int m, S *y, cudaStream_t st);

// ---- interaction -----------------------------------------------------------
template <typename S>
void launch_pack_vblock(const DevLayout &L, int kind, int ch, int n_rows, const double *stage, S *dst, int *flag, cudaStream_t st);
// The same packing read straight from host memory the device can address (pinned and
// mapped): reads follow the block's column-major order (consecutive rows), through a
// shared-memory transpose where the packed layout is row-major (kinds 3 and 6).
// rows_packed / cols_packed: the channel's packed extents (kind 3: H, P; 6: P, P; 1: H, H).
template <typename S>
void launch_pack_vblock_host(const DevLayout &L, int kind, int ch, int n_rows, int rows_packed, int cols_packed,
                             const double *src, S *dst, int *flag, cudaStream_t st);
// Copies of many blocks in one launch (n doubles from src to dst per job); src may be
// mapped host memory.
struct CopyJob {
  const double *src;
  double *dst;
  int64_t n;
};
void launch_copy_jobs(const CopyJob *jobs, int njobs, cudaStream_t st);
template <typename S>
void launch_build_w(const DevLayout &L, const int2 *hp4_slot, const int64_t *v4_off, const int *n4, const double *v4,
                    S *W, int *flag, cudaStream_t st);
template <typename S> void launch_build_vph(const DevLayout &L, const S *Vhp, S *Vph, cudaStream_t st);
template <typename S>
// pairf: npp + nhh + A (ns - A) doubles of scratch for the per-pair factors of the
// chiral-like kind (complex engines; null: every element evaluated in full)
void launch_generate(const DevLayout &L, const DevOrbits &O, const DevPotential &pot, S *Vhp, S *Vpp, S *Vhh, S *W,
                     S *fdiag, S *f6, S *f7, double *e0, double *pairf, int npp, int nhh, cudaStream_t st);
// ordered block of <row|V|col> (or <col|V|row> when swap) into interleaved doubles
template <typename S>
void launch_gen_ordered(const DevOrbits &O, const DevPotential &pot, const int2 *rows, const int2 *cols, int nr, int nc,
                        int swap, double *out, cudaStream_t st);
// packed V' -> ordered reference block (kind 3 V_hhpp, 6 V_pppp, 1 V_hhhh of hhpp channel ch)
template <typename S>
void launch_unpack_vblock(const DevLayout &L, int kind, int ch, int n_rows, int n_cols, const int *row_sgn,
                          const int *col_sgn, const S *src, double *out, cudaStream_t st);
double measure_fp64_peak(int device);
// y += x (n elements)
template <typename S> void launch_axpy(int64_t n, const S *x, S *y, cudaStream_t st);
template <typename S> void launch_mp2(const DevLayout &L, const S *Vhp, const S *fdiag, S *T, cudaStream_t st);
template <typename S> void launch_pack_t(const DevLayout &L, int ch, int n_pp, const double *stage, S *T, int *flag, cudaStream_t st);
template <typename S>
void launch_unpack_t(const DevLayout &L, int ch, int n_pp, const int *pp_signed, const int *hh_signed, int n_hh, const S *T,
                     double *stage, cudaStream_t st);

}  // namespace ccx
