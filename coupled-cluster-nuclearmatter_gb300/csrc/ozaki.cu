// FP64-accurate GEMM by exact digit products on the BF16 tensor cores (sm_103a).
//
// Persistent: one CTA per SM walks the (128-row tile, up to kOzN columns) tiles of the
// problem list; six warps:
//   warp 4 (one lane) streams the digit tiles with cp.async.bulk: per K tile, the
//     kOzSlices B digit tiles into one of two B buffers, then the kOzSlices A digit
//     tiles one by one through a ring of kOzStages stages;
//   warp 5 (one lane) issues tcgen05.mma: A digit i times B digits j = 0 .. 8 - i into
//     the tensor-memory accumulators of levels i + j, all j in one MMA over the stacked
//     B digit tiles, and commits each stage back;
//   warps 0-3 drain the kOzLevels accumulators after every K chunk (kOzChunkTiles K
//     tiles, short enough for every level sum to stay an exact FP32 integer) into two
//     64-bit integer sums per row and column, and after the tile's last chunk convert
//     them to FP64 once, scale by 2^(eA + eB) and add into C.
// Every wait is bounded: on expiry the waiting thread records an error code and raises
// a shared abort flag that ends every other wait at once; the producer lets its own
// copies land before the CTA frees its tensor memory and exits.
#include <cuda_runtime.h>

#include <algorithm>

#include "ozaki.cuh"
#include "tc_ptx.cuh"

namespace ccx {

namespace {

using namespace tcptx;

constexpr int kOzStages = 6;
constexpr uint32_t kATile = 128u * 128u;                   // one A digit tile: 128 rows x 64 BF16
constexpr uint32_t kBSlot = (uint32_t)kOzN * 128u;         // one B digit tile of kOzN rows
constexpr uint32_t kBBuf = (uint32_t)kOzSlices * kBSlot;   // all B digits of one K tile
constexpr uint32_t kBarOff = kOzStages * kATile + 2 * kBBuf;
constexpr int kOzBars = 2 * kOzStages + 8;  // afull, aempty, bfull[2], bempty[2], done, drained, fin
constexpr size_t kOzSmem = kBarOff + kOzBars * 8 + 16;
constexpr int kOzThreads = 192;

__device__ __forceinline__ double pow2(int e) {
  e = max(-1022, min(1023, e));
  return __longlong_as_double((long long)(e + 1023) << 52);
}

__device__ __forceinline__ bool oz_tile_ok(const OzProb &P, const OzTile &tl) {
  const int nc = min(kOzN, P.npad - tl.n0);
  return nc >= 16 && !(nc & 15) && !(P.npad & 15) && !(tl.n0 & 7) && P.nk >= 1;
}

// Persistent: CTA b handles tiles b, b + gridDim.x, ...  The producer, the MMA issuer and
// the drain warps walk the same tile sequence; stage, B-buffer and chunk counters run on
// across tiles, so the next tile's digits stream in while the last chunk drains.
__global__ void __launch_bounds__(kOzThreads, 1) k_oz_gemm(const OzProb *__restrict__ probs,
                                                           const OzTile *__restrict__ tiles, int ntiles, int *err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  uint8_t *abuf = smem;
  uint8_t *bbuf = smem + kOzStages * kATile;
  uint64_t *bars = (uint64_t *)(smem + kBarOff);
  uint64_t *afull = bars, *aempty = bars + kOzStages, *bfull = bars + 2 * kOzStages, *bempty = bfull + 2,
           *done = bempty + 2, *drained = done + 1, *fin = done + 2;
  uint32_t *tmem_slot = (uint32_t *)(bars + kOzBars);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);

  if (warp == 0) {
    tmem_alloc(smem_u32(tmem_slot), 512);
    tmem_relinquish();
  }
  if (tid == 0) {
    for (int s = 0; s < kOzStages; ++s) {
      mbar_init(smem_u32(&afull[s]), 1);
      mbar_init(smem_u32(&aempty[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&bfull[b]), 1);
      mbar_init(smem_u32(&bempty[b]), 1);
    }
    mbar_init(smem_u32(done), 1);
    mbar_init(smem_u32(drained), 4);
    mbar_init(smem_u32(fin), 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  // bounded wait that also ends when another thread has given up
  auto wait = [&](uint64_t *bar, uint32_t parity) -> bool {
    const uint32_t b = smem_u32(bar);
    const long long t0 = clock64();
    while (!mbar_try_wait(b, parity)) {
      if (*abort_flag) return false;
      if (clock64() - t0 > kWaitBudget) {
        *abort_flag = 1;
        return false;
      }
    }
    return true;
  };

  if (warp == 4) {
    if (lane == 0) {  // producer
      int na[kOzStages] = {}, nb[2] = {0, 0};
      int cnt = 0, bk = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const OzTile tl = tiles[t];
        const OzProb P = probs[tl.prob];
        if (!oz_tile_ok(P, tl)) continue;
        const int nc = min(kOzN, P.npad - tl.n0), nk = P.nk;
        const uint8_t *A0 = (const uint8_t *)P.A + (size_t)tl.mt * nk * kATile;
        const uint8_t *B0 = (const uint8_t *)P.B + (size_t)tl.n0 * 128;
        const size_t ap = (size_t)P.a_plane * 2, bp = (size_t)P.b_plane * 2, bt = (size_t)P.npad * 128;
        const uint32_t bbytes = (uint32_t)nc * 128u;
        // live 8-row groups of each A digit tile (1 KiB each); the MMA's rows beyond them
        // read stale shared memory and give level sums that are never stored
        const int live_rows = min(128, P.M - tl.mt * 128);
        const uint32_t a_copy = (uint32_t)((live_rows + 7) / 8) * 1024u;
        for (int kt = 0; kt < nk && ok; ++kt, ++bk) {
          const int bb = bk & 1;
          if (bk >= 2 && !wait(&bempty[bb], (uint32_t)(((bk >> 1) - 1) & 1))) { ok = false; break; }
          const uint32_t fb = smem_u32(&bfull[bb]);
          mbar_expect_tx(fb, (uint32_t)kOzSlices * bbytes);
          for (int j = 0; j < kOzSlices; ++j)
            bulk_g2s(smem_u32(bbuf + bb * kBBuf + j * kBSlot), B0 + j * bp + (size_t)kt * bt, bbytes, fb);
          ++nb[bb];
          for (int i = 0; i < kOzSlices; ++i) {
            const int s = cnt % kOzStages;
            if (cnt >= kOzStages && !wait(&aempty[s], (uint32_t)((cnt / kOzStages - 1) & 1))) { ok = false; break; }
            const uint32_t fa = smem_u32(&afull[s]);
            mbar_expect_tx(fa, a_copy);
            bulk_g2s(smem_u32(abuf + s * kATile), A0 + i * ap + (size_t)kt * kATile, a_copy, fa);
            ++na[s];
            ++cnt;
          }
        }
      }
      if (!ok) atomicExch(err, 1);
      // every issued copy lands before this CTA's shared memory can go away
      for (int s = 0; s < kOzStages; ++s)
        if (na[s]) mbar_wait(smem_u32(&afull[s]), (uint32_t)((na[s] - 1) & 1));
      for (int b = 0; b < 2; ++b)
        if (nb[b]) mbar_wait(smem_u32(&bfull[b]), (uint32_t)((nb[b] - 1) & 1));
    }
  } else if (warp == 5) {
    if (lane == 0) {  // MMA issuer
      int cnt = 0, bk = 0, ck = 0;
      bool ok = true;
      for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
        const OzTile tl = tiles[t];
        const OzProb P = probs[tl.prob];
        if (!oz_tile_ok(P, tl)) {
          atomicExch(err, 4);
          continue;
        }
        const int nk = P.nk;
        const int nchunk = (nk + kOzChunkTiles - 1) / kOzChunkTiles;
        for (int c = 0; c < nchunk && ok; ++c, ++ck) {
          if (ck > 0 && !wait(drained, (uint32_t)((ck - 1) & 1))) { ok = false; break; }
          tc_fence_after();
          const int k_beg = c * kOzChunkTiles, k_end = min(nk, k_beg + kOzChunkTiles);
          for (int kt = k_beg; kt < k_end && ok; ++kt, ++bk) {
            const int bb = bk & 1;
            if (!wait(&bfull[bb], (uint32_t)((bk >> 1) & 1))) { ok = false; break; }
            tc_fence_after();
            const uint32_t sb = smem_u32(bbuf + bb * kBBuf);
            for (int i = 0; i < kOzSlices; ++i) {
              const int s = cnt % kOzStages;
              if (!wait(&afull[s], (uint32_t)((cnt / kOzStages) & 1))) { ok = false; break; }
              tc_fence_after();
              // A digit i times B digits j = 0 .. 8 - i lands in levels i .. 8: the B digit
              // tiles sit one after the other (kOzN rows each) and the level accumulators
              // kOzN columns apart, so one MMA of N = kOzN (9 - i) covers them all (two
              // when that exceeds 256 columns).  Columns beyond a narrow tile's nc come
              // from stale B rows and are never drained.
              const uint64_t da = smem_desc(smem_u32(abuf + s * kATile));
#pragma unroll
              for (int ks = 0; ks < 4; ++ks) {
                const uint32_t acc = (kt > k_beg || i > 0 || ks > 0) ? 1u : 0u;
                for (int j0 = 0; j0 < kOzSlices - i; j0 += 256 / kOzN) {
                  const int nj = min(kOzSlices - i - j0, 256 / kOzN);
                  tc_mma<kTcBF16>(tmem + (uint32_t)((i + j0) * kOzN), da + (uint64_t)(ks * 16),
                                  smem_desc(sb + (uint32_t)j0 * kBSlot) + (uint64_t)(ks * 16),
                                  instr_desc<kTcBF16>(128, nj * kOzN), acc);
                }
              }
              tc_commit(smem_u32(&aempty[s]));
              ++cnt;
            }
            if (ok) tc_commit(smem_u32(&bempty[bb]));
          }
          if (ok) tc_commit(smem_u32(done));
        }
      }
      if (!ok) atomicExch(err, 2);
      // every MMA this thread issued completes before the tensor memory is freed
      tc_commit(smem_u32(fin));
      mbar_wait(smem_u32(fin), 0);
    }
  } else {  // warps 0-3: drain the level accumulators of every chunk, C once per tile
    const int row = warp * 32 + lane;
    const uint32_t tbase = tmem + ((uint32_t)(warp * 32) << 16);
    int ck = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
      const OzTile tl = tiles[t];
      const OzProb P = probs[tl.prob];
      if (!oz_tile_ok(P, tl)) continue;
      const int nc = min(kOzN, P.npad - tl.n0), nk = P.nk;
      const int nchunk = (nk + kOzChunkTiles - 1) / kOzChunkTiles;
      const int m = tl.mt * 128 + row;
      const bool live = m < P.M;
      // a warp none of whose rows is stored skips the drain
      const bool warp_live = tl.mt * 128 + warp * 32 < P.M;
      // The tile's row sums so far as exact integers in units of 2^-30 (levels 0-3) and
      // 2^-60 (levels 4-8, kept below 2^30 by carrying into the first): each chunk adds
      // its level sums with integer operations only, so the accumulators are free for the
      // next chunk's MMAs after a few integer operations per level and column, and the
      // FP64 work (conversion, scaling, the read-modify-write of C) runs once per tile,
      // beside the next tile's MMAs.
      long long ah[kOzN], al[kOzN];
#pragma unroll
      for (int q = 0; q < kOzN; ++q) ah[q] = al[q] = 0;
      for (int c = 0; c < nchunk; ++c, ++ck) {
        const bool got = __all_sync(0xffffffffu, wait(done, (uint32_t)(ck & 1)));
        if (!got) {
          if (lane == 0) atomicExch(err, 3);
          ok = false;
          break;
        }
        tc_fence_after();
#pragma unroll
        for (int cb = 0; cb < kOzN; cb += 4) {
          if (!warp_live || cb >= nc) break;
          // all levels of 4 columns in flight at once, one wait
          uint32_t r[kOzLevels][4];
#pragma unroll
          for (int lv = 0; lv < kOzLevels; ++lv) tmem_ld4(tbase + (uint32_t)(lv * kOzN + cb), r[lv]);
          tmem_ld_wait();
#pragma unroll
          for (int lv = 0; lv < kOzLevels; ++lv) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              // an exact integer below 2^24 in magnitude
              const long long x = (long long)__float2int_rz(__uint_as_float(r[lv][q]));
              if (lv < 4) ah[cb + q] += x * (1ll << (kOzBits * (3 - lv)));
              else al[cb + q] += x * (1ll << (kOzBits * (8 - lv)));
            }
          }
        }
        // the level accumulators are read: the next chunk's MMAs may start
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(drained));
#pragma unroll
        for (int q = 0; q < kOzN; ++q) {
          const long long carry = al[q] >> 30;  // floor: al stays in [0, 2^30)
          ah[q] += carry;
          al[q] -= carry * (1ll << 30);
        }
      }
      if (ok && live) {
        const int eAm = P.eA[m];
        double *crow = P.C + (int64_t)m * P.sCm;
        // 8 columns at a time: their loads of C in flight together, then the stores
#pragma unroll
        for (int q0 = 0; q0 < kOzN; q0 += 8) {
          double old[8];
#pragma unroll
          for (int q = q0; q < q0 + 8; ++q) {
            const int n = tl.n0 + q;
            old[q - q0] = (q < nc && n < P.N) ? crow[(int64_t)n * P.sCn] : 0.0;
          }
#pragma unroll
          for (int q = q0; q < q0 + 8; ++q) {
            const int n = tl.n0 + q;
            if (q < nc && n < P.N) {
              const double z = fma((double)ah[q], 0x1p-30, (double)al[q] * 0x1p-60);
              crow[(int64_t)n * P.sCn] = old[q - q0] + P.alpha * (z * pow2(eAm + P.eB[n]));
            }
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

// ---- digit planes ---------------------------------------------------------------
// Row exponent: the smallest e with |x| < 2^e over the row (0 for an all-zero row).
__global__ void k_oz_exps(const OzSplitJob *__restrict__ jobs, const int2 *__restrict__ rowtab, int nrows) {
  const int w = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (w >= nrows) return;
  const int2 jr = rowtab[w];
  const OzSplitJob &J = jobs[jr.x];
  const double *src = J.src + (int64_t)jr.y * J.sr;
  int mx = 0;
  for (int k = lane; k < J.cols; k += 32)
    mx = max(mx, (int)(((unsigned long long)__double_as_longlong(src[(int64_t)k * J.sk]) >> 52) & 0x7ff));
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) J.exps[jr.y] = mx == 0 ? 0 : mx - 1022;
}

// kOzSlices signed 6-bit digits of x 2^-e (truncated after 54 bits), as BF16 bit patterns
__device__ __forceinline__ void oz_digits(double x, int e, uint32_t (&d)[kOzSlices]) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const int ex = (int)((u >> 52) & 0x7ff);
  unsigned long long y = 0;
  if (ex != 0) {
    const unsigned long long mant = (u & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    const int sh = ex - 1021 - e;  // y = |x| 2^(54 - e) = mant 2^sh < 2^54, sh <= 1
    y = sh >= 0 ? (mant << sh) : (-sh >= 64 ? 0ull : (mant >> -sh));
  }
  const bool neg = (u >> 63) != 0;
#pragma unroll
  for (int i = 0; i < kOzSlices; ++i) {
    const int v = (int)((y >> (kOzBits * (kOzSlices - 1 - i))) & 63);
    d[i] = __float_as_uint((float)(neg ? -v : v)) >> 16;
  }
}

__global__ void __launch_bounds__(256) k_oz_digits(const OzSplitJob *__restrict__ jobs, const int4 *__restrict__ chunks) {
  const int4 ck = chunks[blockIdx.x];
  const OzSplitJob J = jobs[ck.x];
  const int tile_units = J.tile_rows * 8;
  const int end = ck.z;
  uint4 *planes = (uint4 *)J.planes;
  const int64_t pstride = J.plane_elems / 8;  // uint4 units between planes
  for (int u = ck.y + threadIdx.x; u < end; u += blockDim.x) {
    const int t = u / tile_units, w = u - t * tile_units;
    const int rt = t / J.nk, kt = t - rt * J.nk;
    const int g = w >> 6, kc = (w >> 3) & 7, r8 = w & 7;
    const int row = rt * J.tile_rows + g * 8 + r8;
    const int k0 = kt * 64 + kc * 8;
    uint32_t dg[8][kOzSlices];
    if (row < J.rows && k0 < J.cols) {
      const int e = J.exps[row];
      const double *src = J.src + (int64_t)row * J.sr;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int k = k0 + j;
        oz_digits(k < J.cols ? src[(int64_t)k * J.sk] : 0.0, e, dg[j]);
      }
    } else {
#pragma unroll
      for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int i = 0; i < kOzSlices; ++i) dg[j][i] = 0;
    }
#pragma unroll
    for (int i = 0; i < kOzSlices; ++i)
      planes[i * pstride + u] = make_uint4(dg[0][i] | (dg[1][i] << 16), dg[2][i] | (dg[3][i] << 16),
                                           dg[4][i] | (dg[5][i] << 16), dg[6][i] | (dg[7][i] << 16));
  }
}

}  // namespace

void launch_oz_gemm(const OzProb *probs, const OzTile *tiles, int ntiles, int *err, cudaStream_t st) {
  if (ntiles <= 0) return;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms <= 0) sms = 1;
  cudaFuncSetAttribute(k_oz_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kOzSmem);
  k_oz_gemm<<<std::min(ntiles, sms), kOzThreads, kOzSmem, st>>>(probs, tiles, ntiles, err);
}

std::vector<int4> oz_split_chunks(const std::vector<OzSplitJob> &jobs) {
  std::vector<int4> out;
  for (size_t j = 0; j < jobs.size(); ++j)
    split_ranges((int)j, jobs[j].rows, jobs[j].rows_pad, jobs[j].tile_rows, jobs[j].nk, out);
  return out;
}

std::vector<int2> oz_row_table(const std::vector<OzSplitJob> &jobs) {
  std::vector<int2> out;
  for (size_t j = 0; j < jobs.size(); ++j)
    for (int r = 0; r < jobs[j].rows; ++r) out.push_back(make_int2((int)j, r));
  return out;
}

void launch_oz_split(const OzSplitJob *jobs, const int2 *rowtab, int nrows, const int4 *chunks, int nchunks,
                     cudaStream_t st) {
  if (nrows > 0) k_oz_exps<<<(nrows * 32 + 255) / 256, 256, 0, st>>>(jobs, rowtab, nrows);
  if (nchunks > 0) k_oz_digits<<<nchunks, 256, 0, st>>>(jobs, chunks);
}

}  // namespace ccx
