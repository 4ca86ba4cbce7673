// Tensor-core split-precision GEMM on sm_103a (tcgen05 + TMEM + bulk async copies).
//
// C(fp64) += alpha * (A_hi B_hi + A_hi B_lo + A_lo B_hi), with the hi/lo pairs of BF16
// (kind::f16) or TF32 (kind::tf32) operands, FP32 accumulation in tensor memory.
// Persistent: one CTA per SM walks the tile list (a tile = 128 rows of one problem, all N
// <= 256 columns); a tile may sum up to six products with the same M, N (segments), each
// added or subtracted.
// Lane 0 of warp 8 streams the pre-tiled K tiles of A and B into a ring of shared-memory
// stages with cp.async.bulk (one contiguous copy per operand tile, completion on an
// mbarrier); the ring runs on across tiles.  Lane 0 of warp 9 issues the MMAs into one
// of two tensor-memory halves, alternating by tile, and tcgen05.commit hands each stage
// back.  Warps 0-3 drain the tiles of half 0 and warps 4-7 those of half 1: each reads
// its 32 TMEM lanes (rows) with tcgen05.ld and adds into C while the next tile
// accumulates in the other half.
// Every mbarrier wait is bounded by a clock budget: on expiry the kernel records an
// error code, lets its own copies land, frees its TMEM and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>

#include "tc_ptx.cuh"
#include "tcgemm.cuh"

namespace ccx {

namespace {

using namespace tcptx;

constexpr int kTcThreads = 320;   // warps 0-7 epilogue, warp 8 producer, warp 9 MMA issuer
constexpr int kTcHalfCols = 256;  // tensor-memory columns of one accumulator half
constexpr int kTcMaxStages = 8;

// FP32 bit pattern -> the same value as FP64, exactly, with integer operations only (a
// float-to-double conversion would run on this GPU's narrow FP64 pipe)
__device__ __forceinline__ double f32_bits_to_f64(uint32_t u) {
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  const uint32_t e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  unsigned long long bits;
  if (e == 0xffu) {  // infinities and NaNs
    bits = sign | (0x7ffull << 52) | ((unsigned long long)m << 29);
  } else if (e != 0) {  // normal: exponent rebiased from 127 to 1023
    bits = sign | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29);
  } else if (m == 0) {
    bits = sign;
  } else {  // subnormal m 2^-149, normalised on its leading bit p
    const int p = 31 - __clz((int)m);
    bits = sign | ((unsigned long long)(p - 149 + 1023) << 52) | (((unsigned long long)m << (52 - p)) & 0xFFFFFFFFFFFFFull);
  }
  return __longlong_as_double((long long)bits);
}

// K tiles of segment e of a problem (e = 0: the problem's own operands)
__device__ __forceinline__ TcSeg tc_segment(const TcProb *__restrict__ pp, int e) {
  if (e == 0) return TcSeg{pp->Ahi, pp->Alo, pp->Bhi, pp->Blo, pp->nk, pp->bstride, 0};
  return pp->ext[e - 1];
}

// What every role of the kernel derives from a tile's problem, identically.
struct TcGeom {
  int npad, nseg, ncols, nacc;
  bool ok;
};
__device__ __forceinline__ TcGeom tc_geom(const TcProb *__restrict__ pp, int npad_max) {
  TcGeom g;
  g.npad = pp->npad;
  g.nseg = 1 + min(max(pp->next, 0), kTcMaxSegs - 1);
  int nk = 0;
  for (int e = 0; e < g.nseg; ++e) nk += tc_segment(pp, e).nk;
  g.ok = g.npad >= 16 && g.npad <= 256 && (g.npad & 15) == 0 && g.npad <= npad_max && nk >= 1;
  g.ncols = 32;
  while (g.ncols < g.npad) g.ncols <<= 1;
  // one FP32 accumulator per segment while they fit in half of the tensor memory (the
  // other half holds the next tile's accumulators); a segment beyond that adds into the
  // last one.  Each product then keeps the rounding of its own accumulation, and the
  // epilogue sums them in FP64.
  g.nacc = g.nseg;
  while (g.nacc > 1 && g.nacc * g.ncols > kTcHalfCols) --g.nacc;
  return g;
}

template <int KIND>
__global__ void __launch_bounds__(kTcThreads, 1) k_tc_gemm(const TcProb *__restrict__ probs,
                                                          const TcTile *__restrict__ tiles, int ntiles, int stages,
                                                          int npad_max, int *err, long long budget) {
  extern __shared__ __align__(1024) uint8_t smem[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr uint32_t a_bytes = 128u * 128u;
  const uint32_t stage_bytes = 2u * a_bytes + 2u * (uint32_t)npad_max * 128u;
  uint64_t *full = (uint64_t *)(smem + (size_t)stages * stage_bytes);
  uint64_t *empty = full + stages;
  uint64_t *tfull = empty + stages, *tempty = tfull + 2, *fin = tempty + 2;
  uint32_t *tmem_slot = (uint32_t *)(fin + 1);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);

  if (warp == 0) {
    tmem_alloc(smem_u32(tmem_slot), 2 * kTcHalfCols);
    tmem_relinquish();
  }
  if (tid == 0) {
    for (int s = 0; s < stages; ++s) {
      mbar_init(smem_u32(&full[s]), 1);
      mbar_init(smem_u32(&empty[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&tfull[b]), 1);
      mbar_init(smem_u32(&tempty[b]), 4);  // the four warps of drain group b
    }
    mbar_init(smem_u32(fin), 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  // bounded wait (budget cycles) that also ends when another thread has given up; the
  // final waits for copies and MMAs in flight keep the full kWaitBudget
  auto wait = [&](uint64_t *bar, uint32_t parity) -> bool {
    const uint32_t b = smem_u32(bar);
    const long long t0 = clock64();
    while (!mbar_try_wait(b, parity)) {
      if (*abort_flag) return false;
      if (clock64() - t0 > budget) {
        *abort_flag = 1;
        return false;
      }
    }
    return true;
  };

  if (warp == 8) {
    if (lane == 0) {
      // producer: one bulk copy per operand tile into the stage ring, which runs on
      // across tiles; a stage is refilled once the MMAs that read it have completed
      int cnt = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const TcTile tl = tiles[t];
        const TcProb *__restrict__ pp = probs + tl.prob;
        const TcGeom G = tc_geom(pp, npad_max);
        if (!G.ok) continue;
        const uint32_t b_bytes = (uint32_t)G.npad * 128u;
        // live 8-row groups of the A tile (1 KiB each); the MMA's rows beyond them read
        // stale shared memory and produce rows that are never stored
        const int live_rows = min(128, pp->M - tl.mt * 128);
        const uint32_t a_copy = (uint32_t)((live_rows + 7) / 8) * 1024u;
        for (int e = 0; e < G.nseg && ok; ++e) {
          const TcSeg g = tc_segment(pp, e);
          const bool two_a = g.Alo != nullptr;
          const size_t bst = g.bstride ? (size_t)g.bstride : (size_t)b_bytes;
          const uint8_t *Ahi = (const uint8_t *)g.Ahi + (size_t)tl.mt * g.nk * a_bytes;
          const uint8_t *Alo = two_a ? (const uint8_t *)g.Alo + (size_t)tl.mt * g.nk * a_bytes : nullptr;
          const uint8_t *Bhi = (const uint8_t *)g.Bhi, *Blo = (const uint8_t *)g.Blo;
          const uint32_t tx = (two_a ? 2u : 1u) * a_copy + 2u * b_bytes;
          for (int kl = 0; kl < g.nk; ++kl, ++cnt) {
            const int s = cnt % stages;
            // fill j = cnt / stages of stage s waits for consumption j - 1
            if (cnt >= stages && !wait(&empty[s], (uint32_t)((cnt / stages - 1) & 1))) {
              ok = false;
              break;
            }
            uint8_t *st = smem + (size_t)s * stage_bytes;
            const uint32_t fb = smem_u32(&full[s]);
            mbar_expect_tx(fb, tx);
            bulk_g2s(smem_u32(st), Ahi + (size_t)kl * a_bytes, a_copy, fb);
            if (two_a) bulk_g2s(smem_u32(st + a_bytes), Alo + (size_t)kl * a_bytes, a_copy, fb);
            bulk_g2s(smem_u32(st + 2 * a_bytes), Bhi + (size_t)kl * bst, b_bytes, fb);
            bulk_g2s(smem_u32(st + 2 * a_bytes + (size_t)npad_max * 128), Blo + (size_t)kl * bst, b_bytes, fb);
          }
        }
      }
      if (!ok) atomicExch(err, 1);
      // every copy this CTA issued lands before the shared memory goes away: stage s
      // received fills 0 .. n_s - 1, the last completing phase n_s - 1 of full[s]
      for (int s = 0; s < stages; ++s) {
        const int n_s = cnt > s ? (cnt - s + stages - 1) / stages : 0;
        if (n_s > 0) mbar_wait(smem_u32(&full[s]), (uint32_t)((n_s - 1) & 1));
      }
    }
  } else if (warp == 9) {
    if (lane == 0) {
      // MMA issuer: the K tiles of every segment of a tile into its accumulators in
      // tensor-memory half b = (local tile) & 1, then tcgen05.commit to tfull[b]
      int cnt = 0, lt = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const TcTile tl = tiles[t];
        const TcProb *__restrict__ pp = probs + tl.prob;
        const TcGeom G = tc_geom(pp, npad_max);
        if (!G.ok) {
          atomicExch(err, 4);
          continue;
        }
        const int b = lt & 1;
        if (lt >= 2 && !wait(&tempty[b], (uint32_t)(((lt >> 1) - 1) & 1))) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t idesc = instr_desc<KIND>(128, G.npad);
        for (int e = 0; e < G.nseg && ok; ++e) {
          const TcSeg g = tc_segment(pp, e);
          const bool two_a = g.Alo != nullptr;
          // instruction-descriptor bit 14 negates B: a subtracted product
          const uint32_t id = idesc | (g.neg ? (1u << 14) : 0u);
          const uint32_t acc = tmem + (uint32_t)(b * kTcHalfCols + min(e, G.nacc - 1) * G.ncols);
          bool first = e < G.nacc;  // this segment opens its accumulator
          for (int kl = 0; kl < g.nk; ++kl, ++cnt) {
            const int s = cnt % stages;
            if (!wait(&full[s], (uint32_t)((cnt / stages) & 1))) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t sa = smem_u32(smem + (size_t)s * stage_bytes);
            const uint32_t sal = sa + a_bytes;
            const uint32_t sb = sa + 2 * a_bytes;
            const uint32_t sbl = sb + (uint32_t)npad_max * 128u;
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
              const uint32_t o = (uint32_t)ks * 256u;
              tc_mma<KIND>(acc, smem_desc(sa + o), smem_desc(sb + o), id, first ? 0u : 1u);
              first = false;
              tc_mma<KIND>(acc, smem_desc(sa + o), smem_desc(sbl + o), id, 1u);
              if (two_a) tc_mma<KIND>(acc, smem_desc(sal + o), smem_desc(sb + o), id, 1u);
            }
            tc_commit(smem_u32(&empty[s]));
          }
        }
        if (ok) tc_commit(smem_u32(&tfull[b]));
        ++lt;
      }
      if (!ok) atomicExch(err, 2);
      // every MMA this thread issued completes before the tensor memory is freed
      tc_commit(smem_u32(fin));
      mbar_wait(smem_u32(fin), 0);
    }
  } else {
    // warps 0-7: two groups of four, group g draining the tiles of tensor-memory half g,
    // so two tiles' C updates are in flight; warp w reads lanes 32 (w % 4) .. + 31
    const int grp = warp >> 2, quad = warp & 3;
    const int row = quad * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(quad * 32) << 16);
    int lt = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
      const TcTile tl = tiles[t];
      const TcProb *__restrict__ pp = probs + tl.prob;
      const TcGeom G = tc_geom(pp, npad_max);
      if (!G.ok) continue;
      const int b = lt & 1;
      if (b != grp) {
        ++lt;
        continue;
      }
      const bool got = __all_sync(0xffffffffu, wait(&tfull[b], (uint32_t)((lt >> 1) & 1)));
      if (!got) {
        if (lane == 0) atomicExch(err, 3);
        break;
      }
      tc_fence_after();
      const int m = tl.mt * 128 + row;
      const int64_t sCm = pp->sCm, sCn = pp->sCn;
      double *__restrict__ crow = pp->C + (int64_t)m * sCm;
      const double *C0 = pp->C0;
      const double *__restrict__ c0row = C0 ? C0 + (int64_t)m * sCm : nullptr;
      const bool keep = pp->overwrite == 0;
      const double alpha = pp->alpha;
      const int nvalid = pp->N;
      const bool live = m < pp->M;
      if (tl.mt * 128 + quad * 32 >= pp->M) {  // no row of this warp's lanes is stored
        if (lane == 0) mbar_arrive(smem_u32(&tempty[b]));
        ++lt;
        continue;
      }
      const uint32_t accb = lane_base + (uint32_t)(b * kTcHalfCols);
      // 32 columns per read (npad rounded up to 32 stays inside each accumulator)
      for (int c0 = 0; c0 < G.npad; c0 += 32) {
        // the C and C0 loads go first, so that their latency overlaps the tensor-memory
        // reads; the mode is uniform over the tile, so the branches sit outside the
        // unrolled loops and the 32 loads of a row issue back to back
        double v[32];
        if (live && keep) {
#pragma unroll
          for (int j = 0; j < 32; ++j) v[j] = (c0 + j < nvalid) ? crow[(int64_t)(c0 + j) * sCn] : 0.0;
        } else {
#pragma unroll
          for (int j = 0; j < 32; ++j) v[j] = 0.0;
        }
        if (live && c0row) {
          double add[32];
#pragma unroll
          for (int j = 0; j < 32; ++j) add[j] = (c0 + j < nvalid) ? c0row[(int64_t)(c0 + j) * sCn] : 0.0;
          if (keep) {
#pragma unroll
            for (int j = 0; j < 32; ++j) v[j] += add[j];
          } else {
#pragma unroll
            for (int j = 0; j < 32; ++j) v[j] = add[j];
          }
        }
        // one FP64 multiply-add per accumulator and element: the FP32 values widen on
        // the integer pipe
        for (int a = 0; a < G.nacc; ++a) {
          uint32_t r[32];
          tmem_ld32(accb + (uint32_t)(a * G.ncols + c0), r);
          tmem_ld_wait();
#pragma unroll
          for (int j = 0; j < 32; ++j) v[j] = fma(alpha, f32_bits_to_f64(r[j]), v[j]);
        }
        if (c0 + 32 >= G.npad) {
          // the accumulators of this half are read: hand it back to the MMA issuer
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(smem_u32(&tempty[b]));
        }
        if (live) {
#pragma unroll
          for (int j = 0; j < 32; ++j)
            if (c0 + j < nvalid) crow[(int64_t)(c0 + j) * sCn] = v[j];
        }
      }
      ++lt;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 2 * kTcHalfCols);
  }
}

// ---- operand preparation ---------------------------------------------------------
// x = hi + lo split of an FP64 value (or of a difference a - b of two) into two narrow
// floats (BF16: 8 significant bits each; TF32: 11), computed on the bit patterns with
// integer operations only: the FP64 pipe of this GPU is narrow, and both a float
// conversion of a double and an FP64 subtraction run on it.  hi is x rounded to NB
// significant bits (half away from zero), lo the remainder rounded the same way, so
// |x - hi - lo| <= 2^(-2 NB) |x| (plus 2^-60 |a| for a difference, whose smaller
// operand is truncated below the larger one's 62-bit grid).  Values below the float
// range (2^-126) and FP64 subnormals become zero.
template <int NB>
struct BitSplit {
  // float bit pattern of sign * sig * 2^(e2 - (NB - 1)), sig in [2^(NB-1), 2^NB)
  __device__ static uint32_t pack(uint32_t sign, int e2, uint32_t sig) {
    const int biased = e2 + 127;
    if (biased <= 0) return sign << 31;
    return (sign << 31) | ((uint32_t)biased << 23) | ((sig & ((1u << (NB - 1)) - 1)) << (24 - NB));
  }
  // one NB-bit rounding of mag 2^ex (mag > 0, up to 63 bits): its significand, the
  // exponent e2 of pack(), and the signed remainder mag - sig 2^drop
  __device__ static void round_nb(unsigned long long mag, int ex, uint32_t &sig, int &e2, long long &rem) {
    const int p = 63 - __clzll((long long)mag);  // leading bit
    const int drop = p + 1 - NB;
    if (drop <= 0) {
      sig = (uint32_t)(mag << (-drop));
      e2 = ex + p;
      rem = 0;
      return;
    }
    unsigned long long h = (mag + (1ull << (drop - 1))) >> drop;
    rem = (long long)(mag - (h << drop));
    e2 = ex + p;
    if (h == (1ull << NB)) {  // rounded up to the next power of two
      h >>= 1;
      ++e2;
    }
    sig = (uint32_t)h;
  }
  // x = (-1)^sign mag 2^ex
  __device__ static void split_mag(uint32_t sign, unsigned long long mag, int ex, uint32_t &hi, uint32_t &lo) {
    if (mag == 0) {
      hi = lo = sign << 31;
      return;
    }
    uint32_t h, l;
    int eh, el;
    long long rem, rem2;
    round_nb(mag, ex, h, eh, rem);
    hi = pack(sign, eh, h);
    if (rem == 0) {
      lo = 0;
      return;
    }
    round_nb((unsigned long long)(rem < 0 ? -rem : rem), ex, l, el, rem2);
    lo = pack(sign ^ (rem < 0 ? 1u : 0u), el, l);
  }
  // sign, 53-bit significand and exponent (value = sig 2^ex) of an FP64 bit pattern;
  // zero and subnormals give sig = 0
  __device__ static void decode(unsigned long long u, uint32_t &sign, unsigned long long &sig, int &ex) {
    sign = (uint32_t)(u >> 63);
    const int e = (int)((u >> 52) & 0x7ff);
    sig = e == 0 ? 0ull : (u & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    ex = e - 1075;
  }
  __device__ static void split(double x, uint32_t &hi, uint32_t &lo) {
    uint32_t sign;
    unsigned long long sig;
    int ex;
    decode((unsigned long long)__double_as_longlong(x), sign, sig, ex);
    split_mag(sign, sig, ex, hi, lo);
  }
  // split of a - b: both significands on the 62-bit grid of the larger exponent, added
  // as signed 64-bit integers (the magnitudes stay below 2^62, their sum below 2^63)
  __device__ static void split_diff(double a, double b, uint32_t &hi, uint32_t &lo) {
    uint32_t sa, sb;
    unsigned long long ma, mb;
    int ea, eb;
    decode((unsigned long long)__double_as_longlong(a), sa, ma, ea);
    decode((unsigned long long)__double_as_longlong(b), sb, mb, eb);
    sb ^= 1u;  // a + (-b)
    if (mb == 0) {
      split_mag(sa, ma, ea, hi, lo);
      return;
    }
    if (ma == 0) {
      split_mag(sb, mb, eb, hi, lo);
      return;
    }
    const int e = max(ea, eb);
    const int da = e - ea, db = e - eb;
    const long long va = da >= 62 ? 0 : (long long)((ma << 9) >> da);
    const long long vb = db >= 62 ? 0 : (long long)((mb << 9) >> db);
    const long long r = (sa ? -va : va) + (sb ? -vb : vb);
    split_mag(r < 0 ? 1u : 0u, (unsigned long long)(r < 0 ? -r : r), e - 9, hi, lo);
  }
};
// elements per 16-byte unit and the float bit patterns of one unit
template <int KIND> struct Half;
template <> struct Half<kTcBF16> {
  static constexpr int per16 = 8;
  static constexpr int nb = 8;
  __device__ static uint4 pack(const uint32_t (&f)[8]) {  // the upper halves of 8 floats
    return make_uint4((f[0] >> 16) | (f[1] & 0xFFFF0000u), (f[2] >> 16) | (f[3] & 0xFFFF0000u),
                      (f[4] >> 16) | (f[5] & 0xFFFF0000u), (f[6] >> 16) | (f[7] & 0xFFFF0000u));
  }
};
template <> struct Half<kTcTF32> {
  static constexpr int per16 = 4;
  static constexpr int nb = 11;
  __device__ static uint4 pack(const uint32_t (&f)[4]) { return make_uint4(f[0], f[1], f[2], f[3]); }
};

// One thread per 16-byte unit of the tiled output (one core-matrix row: 8 BF16 or 4
// TF32 values of one operand row).  Inside a tile the units are ordered
// (row group, K chunk, row in group), so a warp reads 8 rows x 4 consecutive K chunks
// and writes 512 contiguous bytes.  Blocks cover kSplitChunk units of one job.  No FP64
// arithmetic: a job with sub splits src - sub through BitSplit::split_diff.
template <int KIND>
__global__ void __launch_bounds__(256) k_tc_split(const TcSplitJob *__restrict__ jobs, const int4 *__restrict__ chunks) {
  using H = Half<KIND>;
  using B = BitSplit<H::nb>;
  constexpr int cme = H::per16;  // elements per unit
  constexpr int tk = 8 * cme;    // elements per 128-byte tile row
  const int4 ck = chunks[blockIdx.x];
  const TcSplitJob J = jobs[ck.x];
  const int tile_units = J.tile_rows * 8;
  const int end = ck.z;
  uint4 *hi = (uint4 *)J.hi, *lo = (uint4 *)J.lo;
  for (int u = ck.y + threadIdx.x; u < end; u += blockDim.x) {
    const int t = u / tile_units, w = u - t * tile_units;
    const int rt = t / J.nk, kt = t - rt * J.nk;
    const int g = w >> 6, kc = (w >> 3) & 7, r8 = w & 7;
    const int row = rt * J.tile_rows + g * 8 + r8;
    const int k0 = kt * tk + kc * cme;
    const bool live = row < J.rows && k0 < J.cols;
    if (live) {
      const double *src = J.src + (int64_t)row * J.sr;
      double a[cme], b[cme];
#pragma unroll
      for (int j = 0; j < cme; ++j) a[j] = (k0 + j < J.cols) ? src[(int64_t)(k0 + j) * J.sk] : 0.0;
      uint32_t h[cme], l[cme];
      if (J.sub && J.add) {  // the FP64 sum, then the plain split
        const double *sub = J.sub + (int64_t)row * J.sr;
#pragma unroll
        for (int j = 0; j < cme; ++j) b[j] = (k0 + j < J.cols) ? sub[(int64_t)(k0 + j) * J.sk] : 0.0;
        if (J.add == 2) {  // src itself as well, into the second tile pair
          uint32_t h2[cme], l2[cme];
#pragma unroll
          for (int j = 0; j < cme; ++j) B::split(a[j] + b[j], h2[j], l2[j]);
          ((uint4 *)J.hi2)[u] = H::pack(h2);
          ((uint4 *)J.lo2)[u] = H::pack(l2);
#pragma unroll
          for (int j = 0; j < cme; ++j) B::split(a[j], h[j], l[j]);
        } else {
#pragma unroll
          for (int j = 0; j < cme; ++j) B::split(a[j] + b[j], h[j], l[j]);
        }
      } else if (J.sub) {
        const double *sub = J.sub + (int64_t)row * J.sr;
#pragma unroll
        for (int j = 0; j < cme; ++j) b[j] = (k0 + j < J.cols) ? sub[(int64_t)(k0 + j) * J.sk] : 0.0;
#pragma unroll
        for (int j = 0; j < cme; ++j) B::split_diff(a[j], b[j], h[j], l[j]);
      } else {
#pragma unroll
        for (int j = 0; j < cme; ++j) B::split(a[j], h[j], l[j]);
      }
      hi[u] = H::pack(h);
      if (lo) lo[u] = H::pack(l);
    } else {
      hi[u] = make_uint4(0, 0, 0, 0);
      if (lo) lo[u] = make_uint4(0, 0, 0, 0);
      if (J.add == 2) {
        ((uint4 *)J.hi2)[u] = make_uint4(0, 0, 0, 0);
        ((uint4 *)J.lo2)[u] = make_uint4(0, 0, 0, 0);
      }
    }
  }
}

// element (row, k) of unit u of a job with the split kernels' tile geometry
template <int CME>
__device__ __forceinline__ void unit_rc(int u, int tile_rows, int nk, int &row, int &k0) {
  constexpr int tk = 8 * CME;
  const int tile_units = tile_rows * 8;
  const int t = u / tile_units, w = u - t * tile_units;
  const int rt = t / nk, kt = t - rt * nk;
  const int g = w >> 6, kc = (w >> 3) & 7, r8 = w & 7;
  row = rt * tile_rows + g * 8 + r8;
  k0 = kt * tk + kc * CME;
}

template <int KIND>
__global__ void __launch_bounds__(256) k_tc_build_map(const TcMapJob *__restrict__ jobs, const int4 *__restrict__ chunks) {
  constexpr int cme = Half<KIND>::per16;
  const int4 ck = chunks[blockIdx.x];
  const TcMapJob J = jobs[ck.x];
  for (int u = ck.y + threadIdx.x; u < ck.z; u += blockDim.x) {
    int row, k0;
    unit_rc<cme>(u, J.tile_rows, J.nk, row, k0);
#pragma unroll
    for (int j = 0; j < cme; ++j) {
      int32_t m = 0;
      if (row < J.rows && k0 + j < J.cols) {
        const int64_t e = J.base + (int64_t)row * J.sr + (int64_t)(k0 + j) * J.sk;
        m = J.ind ? J.ind[e] : (int32_t)(e + 1);
      }
      J.map[(int64_t)u * cme + j] = m;
    }
  }
}

// the hi and lo bit patterns of packed entry |m| - 1 (hi and lo interleaved in one word:
// BF16 hi | lo << 16, TF32 hi | lo << 32), sign flipped for m < 0
template <int KIND>
__device__ __forceinline__ void gather_one(const void *phl, int32_t m, uint32_t &h, uint32_t &l) {
  if (m == 0) {
    h = l = 0;
    return;
  }
  const int64_t i = (m > 0 ? m : -m) - 1;
  if (KIND == kTcBF16) {
    const uint32_t w = ((const uint32_t *)phl)[i] ^ (m < 0 ? 0x80008000u : 0u);
    h = w & 0xFFFFu;
    l = w >> 16;
  } else {
    const unsigned long long w = ((const unsigned long long *)phl)[i] ^ (m < 0 ? 0x8000000080000000ull : 0ull);
    h = (uint32_t)w;
    l = (uint32_t)(w >> 32);
  }
}

template <int KIND>
__global__ void __launch_bounds__(256) k_tc_gather(const TcGatherJob *__restrict__ jobs, const int4 *__restrict__ chunks) {
  constexpr int cme = Half<KIND>::per16;
  const int4 ck = chunks[blockIdx.x];
  const TcGatherJob J = jobs[ck.x];
  uint4 *hi = (uint4 *)J.hi, *lo = (uint4 *)J.lo;
  for (int u = ck.y + threadIdx.x; u < ck.z; u += blockDim.x) {
    int32_t m[cme];
    const int4 *mp = (const int4 *)J.map + (int64_t)u * (cme / 4);  // the unit's map entries
#pragma unroll
    for (int q = 0; q < cme / 4; ++q) {
      const int4 a = mp[q];
      m[4 * q] = a.x;
      m[4 * q + 1] = a.y;
      m[4 * q + 2] = a.z;
      m[4 * q + 3] = a.w;
    }
    uint32_t h[cme], l[cme];
#pragma unroll
    for (int j = 0; j < cme; ++j) gather_one<KIND>(J.phl, m[j], h[j], l[j]);
    uint32_t hw[4], lw[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if constexpr (cme == 8) {  // two BF16 per word
        hw[q] = h[2 * q] | (h[2 * q + 1] << 16);
        lw[q] = l[2 * q] | (l[2 * q + 1] << 16);
      } else {
        hw[q] = h[q];
        lw[q] = l[q];
      }
    }
    hi[u] = make_uint4(hw[0], hw[1], hw[2], hw[3]);
    lo[u] = make_uint4(lw[0], lw[1], lw[2], lw[3]);
  }
}

template <int KIND>
__global__ void __launch_bounds__(256) k_tc_split_packed(const double *__restrict__ src, const double *__restrict__ sub,
                                                         int64_t n, int stride, void *phl) {
  using B = BitSplit<Half<KIND>::nb>;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t h, l;
    if (sub) B::split_diff(src[i * stride], sub[i * stride], h, l);
    else B::split(src[i * stride], h, l);
    if (KIND == kTcBF16) ((uint32_t *)phl)[i] = (h >> 16) | (l & 0xFFFF0000u);
    else ((unsigned long long *)phl)[i] = (unsigned long long)h | ((unsigned long long)l << 32);
  }
}

}  // namespace

void launch_tc_build_map(int kind, const TcMapJob *jobs, const int4 *chunks, int nchunks, cudaStream_t st) {
  if (nchunks <= 0) return;
  if (kind == kTcBF16) k_tc_build_map<kTcBF16><<<nchunks, 256, 0, st>>>(jobs, chunks);
  else k_tc_build_map<kTcTF32><<<nchunks, 256, 0, st>>>(jobs, chunks);
}
void launch_tc_gather(int kind, const TcGatherJob *jobs, const int4 *chunks, int nchunks, cudaStream_t st) {
  if (nchunks <= 0) return;
  if (kind == kTcBF16) k_tc_gather<kTcBF16><<<nchunks, 256, 0, st>>>(jobs, chunks);
  else k_tc_gather<kTcTF32><<<nchunks, 256, 0, st>>>(jobs, chunks);
}
void launch_tc_split_packed(int kind, const double *src, const double *sub, int64_t n, int stride, void *phl,
                            cudaStream_t st) {
  if (n <= 0) return;
  const int grid = (int)std::min<int64_t>((n + 255) / 256, 4096);
  if (kind == kTcBF16) k_tc_split_packed<kTcBF16><<<grid, 256, 0, st>>>(src, sub, n, stride, phl);
  else k_tc_split_packed<kTcTF32><<<grid, 256, 0, st>>>(src, sub, n, stride, phl);
}

int tc_stages(int npad_max) {
  const size_t stage_bytes = 2 * 128 * 128 + 2 * (size_t)npad_max * 128;
  const size_t budget = 227 * 1024 - 256;
  return std::max(1, (int)std::min<size_t>(kTcMaxStages, budget / stage_bytes));
}

void launch_tc_gemm(int kind, const TcProb *probs, const TcTile *tiles, int ntiles, int npad_max, int max_nk, int *err,
                    cudaStream_t st, long long wait_budget) {
  if (wait_budget <= 0) wait_budget = tcptx::kWaitBudget;
  (void)max_nk;  // the stage ring runs on across tiles
  if (ntiles <= 0) return;
  const size_t stage_bytes = 2 * 128 * 128 + 2 * (size_t)npad_max * 128;
  const int stages = tc_stages(npad_max);
  const size_t smem = (size_t)stages * stage_bytes + (2 * stages + 5) * 8 + 16;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms <= 0) sms = 1;
  const int grid = std::min(ntiles, sms);  // persistent: one CTA per SM walks the tile list
  if (kind == kTcBF16) {
    cudaFuncSetAttribute(k_tc_gemm<kTcBF16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_tc_gemm<kTcBF16><<<grid, kTcThreads, smem, st>>>(probs, tiles, ntiles, stages, npad_max, err, wait_budget);
  } else {
    cudaFuncSetAttribute(k_tc_gemm<kTcTF32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_tc_gemm<kTcTF32><<<grid, kTcThreads, smem, st>>>(probs, tiles, ntiles, stages, npad_max, err, wait_budget);
  }
}

void split_ranges(int job, int rows, int rows_pad, int tile_rows, int nk, std::vector<int4> &out) {
  const int tile_units = tile_rows * 8;
  for (int rt = 0; rt < rows_pad / tile_rows; ++rt) {
    const int live_rows = std::min(tile_rows, rows - rt * tile_rows);
    if (live_rows <= 0) continue;
    const int live_units = (live_rows + 7) / 8 * 64;
    for (int kt = 0; kt < nk; ++kt) {
      const int base = (rt * nk + kt) * tile_units;
      for (int u = 0; u < live_units; u += kSplitChunk)
        out.push_back(make_int4(job, base + u, base + std::min(live_units, u + kSplitChunk), 0));
    }
  }
}

std::vector<int4> tc_split_chunks(const std::vector<TcSplitJob> &jobs) {
  std::vector<int4> out;
  for (size_t j = 0; j < jobs.size(); ++j)
    split_ranges((int)j, jobs[j].rows, jobs[j].rows_pad, jobs[j].tile_rows, jobs[j].nk, out);
  return out;
}

void launch_tc_split(int kind, const TcSplitJob *jobs, const int4 *chunks, int nchunks, cudaStream_t st) {
  if (nchunks <= 0) return;
  if (kind == kTcBF16) k_tc_split<kTcBF16><<<nchunks, 256, 0, st>>>(jobs, chunks);
  else k_tc_split<kTcTF32><<<nchunks, 256, 0, st>>>(jobs, chunks);
}

}  // namespace ccx
