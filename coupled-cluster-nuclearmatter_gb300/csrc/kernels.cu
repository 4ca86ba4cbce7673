// CCD kernels of the FP64 path (real or complex scalars).
//
// The engine stores T2 packed: one block per hhpp channel over pairs a<b and i<j
// (column-major, P x H).  Every term of the reference residual
// (ccm_t2_eqn.f90:4-1304) is restated on that representation:
//   ordered sums 1/2 sum_cd over (c,d) become sums over c<d with weight 1, and
//   the reference's antisymmetrising scatters become gathers with signs.
#include <algorithm>
#include <cstdio>

#include "common.cuh"
#include "devlayout.hpp"
#include "kernels.hpp"
#include "potential.cuh"

namespace ccx {

namespace {

__device__ inline double2 warp_sum2(double2 v) {
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  return v;
}
__device__ inline double shfl_xor(double x, int o) { return __shfl_xor_sync(0xffffffffu, x, o); }
__device__ inline cplx shfl_xor(cplx x, int o) { return cplx(shfl_xor(x.re, o), shfl_xor(x.im, o)); }
// Butterfly reduce-scatter of 32 values per lane over the warp: afterwards v[0] of lane
// l holds the warp total of value l.  31 additions per lane instead of 5 per value.
template <typename S>
__device__ inline void warp_reduce_scatter32(S (&v)[32], int lane) {
#pragma unroll
  for (int o = 16, n = 32; o >= 1; o >>= 1, n >>= 1) {
    const bool upper = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < n / 2; ++i) {
      const S give = upper ? v[i] : v[i + n / 2];
      const S keep = upper ? v[i + n / 2] : v[i];
      v[i] = keep + shfl_xor(give, o);
    }
  }
}
__device__ inline double2 to2(double x) { return make_double2(x, 0.0); }
__device__ inline double2 to2(cplx x) { return make_double2(x.re, x.im); }
template <typename S> __device__ inline S from2(double2 v);
template <> __device__ inline double from2<double>(double2 v) { return v.x; }
template <> __device__ inline cplx from2<cplx>(double2 v) { return cplx(v.x, v.y); }

// Block-wide sum of NV doubles per thread into partial[blockIdx.x*NV + k].
template <int NV>
__device__ void block_partial(double (&v)[NV], double *partial) {
  __shared__ double red[NV][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if constexpr (NV == 32) {
    // butterfly reduce-scatter: lane k ends with the warp total of value k (31 additions
    // per lane instead of 5 per value)
    warp_reduce_scatter32(v, lane);
    red[lane][wid] = v[0];
  } else {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double x = warp_sum(v[k]);
      if (lane == 0) red[k][wid] = x;
    }
  }
  __syncthreads();
  if (wid == 0) {
    if constexpr (NV == 32) {  // lane k sums value k over the warps, in warp order
      double x = 0.0;
      for (int w = 0; w < nw; ++w) x += red[lane][w];
      partial[(int64_t)blockIdx.x * NV + lane] = x;
    } else {
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        double x = lane < nw ? red[k][lane] : 0.0;
        x = warp_sum(x);
        if (lane == 0) partial[(int64_t)blockIdx.x * NV + k] = x;
      }
    }
  }
}

// Fixed-order finish of nb partial rows of nv values: out[k] = sum_b partial[b*nv+k].
__global__ void k_finish(const double *partial, int nb, int nv, double *out) {
  const int k = blockIdx.x;
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) s += partial[(int64_t)b * nv + k];
  __shared__ double red[32];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double x = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    x = warp_sum(x);
    if (threadIdx.x == 0) out[k] = x;
  }
}

void finish(const double *partial, int nb, int nv, double *out, cudaStream_t st) {
  k_finish<<<nv, 256, 0, st>>>(partial, nb, nv, out);
}

// An input value (re, im) in the engine's scalar.  Flag bits: 1 a non-zero imaginary
// part given to a real engine, 2 a NaN or Inf.
template <typename S> __device__ inline S cvt_in(const double *p, int *flag);
template <> __device__ inline double cvt_in<double>(const double *p, int *flag) {
  if (p[1] != 0.0) atomicOr(flag, 1);
  if (!isfinite(p[0]) || !isfinite(p[1])) atomicOr(flag, 2);
  return p[0];
}
template <> __device__ inline cplx cvt_in<cplx>(const double *p, int *flag) {
  if (!isfinite(p[0]) || !isfinite(p[1])) atomicOr(flag, 2);
  return cplx(p[0], p[1]);
}

}  // namespace

// ============================================================================
// grouped GEMM, FP64 FMA.  One CTA per BM x BN output tile of one problem; up to two
// K segments share the accumulator (the pp-ladder and hh-ladder both add into R).
// Thread (tm, tn) owns a TM x TN register tile, tm fastest; threads whose columns
// lie beyond N skip the FMA loop, so narrow problems waste few FP64 lanes.
// ============================================================================
template <typename S, int BM, int BN, int TM, int TN>
__global__ void __launch_bounds__(256) k_gemm(const GemmProb<S> *__restrict__ probs, const GemmTile *__restrict__ tiles) {
  constexpr int BK = kGemmBK;
  constexpr int NTM = BM / TM;  // threads along M
  static_assert(NTM * (BN / TN) == 256, "256 threads");
  __shared__ S As[BK][BM + 1];
  __shared__ S Bs[BK][BN + 1];
  const GemmTile tl = tiles[blockIdx.x];
  const GemmProb<S> &pr = probs[tl.prob];
  const int M = pr.M, N = pr.N, nseg = pr.nseg, kchunk = pr.kchunk;
  const int tid = threadIdx.x;
  const int tm = tid % NTM, tn = tid / NTM;
  const bool active = (tl.m0 + tm * TM < M) && (tl.n0 + tn * TN < N);
  S acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = S(0.0);
  for (int s = 0; s < nseg; ++s) {
    const S *A = pr.seg[s].A, *B = pr.seg[s].B;
    const int64_t sAm = pr.seg[s].sAm, sAk = pr.seg[s].sAk, sBk = pr.seg[s].sBk, sBn = pr.seg[s].sBn;
    const double alpha = pr.seg[s].alpha;
    int kbeg = 0, kend = pr.seg[s].K;
    if (kchunk > 0) {
      kbeg = tl.kslice * kchunk;
      kend = min(kend, kbeg + kchunk);
    }
    for (int k0 = kbeg; k0 < kend; k0 += BK) {
      for (int x = tid; x < BM * BK; x += 256) {
        int m, k;
        if (sAm == 1) { m = x % BM; k = x / BM; } else { k = x % BK; m = x / BK; }
        const int gm = tl.m0 + m, gk = k0 + k;
        S v = S(0.0);
        if (gm < M && gk < kend) v = alpha * A[(int64_t)gm * sAm + (int64_t)gk * sAk];
        As[k][m] = v;
      }
      for (int x = tid; x < BK * BN; x += 256) {
        int k, n;
        if (sBk == 1) { k = x % BK; n = x / BK; } else { n = x % BN; k = x / BN; }
        const int gk = k0 + k, gn = tl.n0 + n;
        S v = S(0.0);
        if (gk < kend && gn < N) v = B[(int64_t)gk * sBk + (int64_t)gn * sBn];
        Bs[k][n] = v;
      }
      __syncthreads();
      if (active) {
#pragma unroll
        for (int k = 0; k < BK; ++k) {
          S a[TM], b[TN];
#pragma unroll
          for (int i = 0; i < TM; ++i) a[i] = As[k][tm * TM + i];
#pragma unroll
          for (int j = 0; j < TN; ++j) b[j] = Bs[k][tn * TN + j];
#pragma unroll
          for (int i = 0; i < TM; ++i)
#pragma unroll
            for (int j = 0; j < TN; ++j) acc[i][j] += a[i] * b[j];
        }
      }
      __syncthreads();
    }
  }
  if (!active) return;
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int m = tl.m0 + tm * TM + i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int n = tl.n0 + tn * TN + j;
      if (n >= N) continue;
      if (kchunk > 0) {
        pr.part[(int64_t)tl.kslice * M * N + m + (int64_t)M * n] = acc[i][j];
        continue;
      }
      const int64_t o = (int64_t)m * pr.sCm + (int64_t)n * pr.sCn;
      if (pr.accumulate) pr.C[o] += acc[i][j];
      else pr.C[o] = (pr.C0 ? pr.C0[o] : S(0.0)) + acc[i][j];
    }
  }
}

template <typename S>
void launch_gemm(int shape, const GemmProb<S> *probs, const GemmTile *tiles, int ntiles, cudaStream_t st) {
  if (ntiles <= 0) return;
  if (shape == kShape64x64) k_gemm<S, 64, 64, 4, 4><<<ntiles, 256, 0, st>>>(probs, tiles);
  else k_gemm<S, 128, 32, 8, 2><<<ntiles, 256, 0, st>>>(probs, tiles);
}

template <typename S>
__global__ void k_splitk_reduce(const GemmProb<S> *__restrict__ probs, const int *__restrict__ plist) {
  const GemmProb<S> &pr = probs[plist[blockIdx.x]];
  const int M = pr.M, N = pr.N;
  const int ns = (pr.seg[0].K + pr.kchunk - 1) / pr.kchunk;
  for (int e = threadIdx.x; e < M * N; e += blockDim.x) {
    S acc = S(0.0);
    for (int s = 0; s < ns; ++s) acc += pr.part[(int64_t)s * M * N + e];
    const int m = e % M, n = e / M;
    const int64_t o = (int64_t)m * pr.sCm + (int64_t)n * pr.sCn;
    if (pr.accumulate) pr.C[o] += acc;
    else pr.C[o] = (pr.C0 ? pr.C0[o] : S(0.0)) + acc;
  }
}
template <typename S>
void launch_splitk_reduce(const GemmProb<S> *probs, const int *plist, int n, cudaStream_t st) {
  if (n > 0) k_splitk_reduce<S><<<n, 256, 0, st>>>(probs, plist);
}

// ============================================================================
// T_ph(ai, jb) = T(ab, ij): gather of ccm_t2_eqn.f90:37-62
// ============================================================================
template <typename S>
__global__ void k_gather_tph(DevLayout L, const S *__restrict__ T, S *__restrict__ Tph) {
  const int2 tl = L.phtile[blockIdx.x];
  const int q = tl.x;
  const int nph = L.n_ph[q], nhp = L.n_hp[q];
  const int n = nph * nhp;  // < 2^31 per channel
  const int end = min(tl.y + kTileElems, n);
  for (int e = tl.y + threadIdx.x; e < end; e += blockDim.x) {
    const int c = e / nph, r = e - c * nph;
    const int2 ai = L.ph_orb[L.ph_off[q] + r];
    const int2 jb = L.hp_orb[L.hp_off[q] + c];
    const int2 sab = L.pp_slot[(int64_t)(ai.x - L.A) * L.NP + (jb.y - L.A)];
    const int2 sij = L.hh_slot[ai.y * L.A + jb.x];
    S v = S(0.0);
    if (sab.y != 0 && sij.y != 0) {
      const int ch = sab.x;
      v = (ssign(sab.y) * ssign(sij.y)) * T[L.t_off[ch] + sidx(sab.y) + (int64_t)L.P[ch] * sidx(sij.y)];
    }
    Tph[L.tph_off[q] + e] = v;
  }
}
template <typename S> void launch_gather_tph(const DevLayout &L, const S *T, S *Tph, cudaStream_t st) {
  if (L.nphtile) k_gather_tph<S><<<L.nphtile, 256, 0, st>>>(L, T, Tph);
}
// the same walk as k_gather_tph, recording the signed source index instead of the value
__global__ void k_tph_map(DevLayout L, int32_t *__restrict__ map) {
  const int2 tl = L.phtile[blockIdx.x];
  const int q = tl.x;
  const int nph = L.n_ph[q], nhp = L.n_hp[q];
  const int n = nph * nhp;
  const int end = min(tl.y + kTileElems, n);
  for (int e = tl.y + threadIdx.x; e < end; e += blockDim.x) {
    const int c = e / nph, r = e - c * nph;
    const int2 ai = L.ph_orb[L.ph_off[q] + r];
    const int2 jb = L.hp_orb[L.hp_off[q] + c];
    const int2 sab = L.pp_slot[(int64_t)(ai.x - L.A) * L.NP + (jb.y - L.A)];
    const int2 sij = L.hh_slot[ai.y * L.A + jb.x];
    int32_t m = 0;
    if (sab.y != 0 && sij.y != 0) {
      const int ch = sab.x;
      const int32_t idx = (int32_t)(L.t_off[ch] + sidx(sab.y) + (int64_t)L.P[ch] * sidx(sij.y)) + 1;
      m = (ssign(sab.y) * ssign(sij.y)) < 0 ? -idx : idx;
    }
    map[L.tph_off[q] + e] = m;
  }
}
void launch_tph_map(const DevLayout &L, int32_t *map, cudaStream_t st) {
  if (L.nphtile) k_tph_map<<<L.nphtile, 256, 0, st>>>(L, map);
}

// ============================================================================
// X'(m, j) = sum_k V'(k, m) T'(k, j) per hhpp channel (the V_hhpp T product of the I9
// ZGEMM, ccm_t2_eqn.f90:459, on packed pairs).  V_hhpp' and T' are P x H column-major,
// so X(m, j) is the dot product of two contiguous columns of length P.  One CTA per
// (channel, kXM rows, kXJ columns): the kXJ columns of T' are staged in shared memory
// in K chunks, each warp owns rows m (lanes stride over k), and the lane partials are
// reduced with shuffles at the end, in a fixed order.
// ============================================================================
template <typename S, int NJ>
__device__ __forceinline__ void xdot_rows(const S *__restrict__ V, const S (*Ts)[kXK], int64_t off, int P, int H, int m0,
                                          int k0, int kn, int warp, int lane, S (&acc)[kXM / 8][kXJ]) {
  constexpr int RPW = kXM / 8;
#pragma unroll
  for (int r = 0; r < RPW; ++r) {
    const int m = m0 + warp + 8 * r;
    if (m >= H) break;
    const S *vc = V + off + (int64_t)P * m + k0;
    int k = lane;
    // two independent loads in flight per iteration
    for (; k + 32 < kn; k += 64) {
      const S v0 = vc[k], v1 = vc[k + 32];
#pragma unroll
      for (int j = 0; j < NJ; ++j) {
        acc[r][j] += v0 * Ts[j][k];
        acc[r][j] += v1 * Ts[j][k + 32];
      }
    }
    if (k < kn) {
      const S v = vc[k];
#pragma unroll
      for (int j = 0; j < NJ; ++j) acc[r][j] += v * Ts[j][k];
    }
  }
}

template <typename S>
__global__ void __launch_bounds__(256) k_xdot(DevLayout L, const int4 *__restrict__ work, const S *__restrict__ V,
                                              const S *__restrict__ T, S *__restrict__ part) {
  constexpr int RPW = kXM / 8;  // rows per warp
  __shared__ S Ts[kXJ][kXK];
  const int4 w = work[blockIdx.x];  // (channel, m0 | j0 << 16, K slice, partial slot)
  const int ch = w.x, m0 = w.y & 0xffff, j0 = w.y >> 16;
  const int H = L.H[ch];
  const int kbeg = w.z * kXSlice;
  const int P = min(L.P[ch], kbeg + kXSlice);  // this item's K range is [kbeg, P)
  const int64_t off = L.t_off[ch];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nj = min(kXJ, H - j0);
  S acc[RPW][kXJ];
#pragma unroll
  for (int r = 0; r < RPW; ++r)
#pragma unroll
    for (int j = 0; j < kXJ; ++j) acc[r][j] = S(0.0);
  const int ld = L.P[ch];  // column length of V' and T'
  for (int k0 = kbeg; k0 < P; k0 += kXK) {
    const int kn = min(kXK, P - k0);
    for (int x = threadIdx.x; x < kXJ * kXK; x += blockDim.x) {
      const int j = x / kXK, k = x % kXK;
      Ts[j][k] = (j < nj && k < kn) ? T[off + (int64_t)ld * (j0 + j) + k0 + k] : S(0.0);
    }
    __syncthreads();
    // no FP64 work on the padding columns of a partial column block
    switch (nj) {
      case 8: xdot_rows<S, 8>(V, Ts, off, ld, H, m0, k0, kn, warp, lane, acc); break;
      case 7: xdot_rows<S, 7>(V, Ts, off, ld, H, m0, k0, kn, warp, lane, acc); break;
      case 6: xdot_rows<S, 6>(V, Ts, off, ld, H, m0, k0, kn, warp, lane, acc); break;
      case 5: xdot_rows<S, 5>(V, Ts, off, ld, H, m0, k0, kn, warp, lane, acc); break;
      case 4: xdot_rows<S, 4>(V, Ts, off, ld, H, m0, k0, kn, warp, lane, acc); break;
      case 3: xdot_rows<S, 3>(V, Ts, off, ld, H, m0, k0, kn, warp, lane, acc); break;
      case 2: xdot_rows<S, 2>(V, Ts, off, ld, H, m0, k0, kn, warp, lane, acc); break;
      default: xdot_rows<S, 1>(V, Ts, off, ld, H, m0, k0, kn, warp, lane, acc); break;
    }
    __syncthreads();
  }
  // the item's kXM x kXJ partial tile, row-major, in its slot: lane l of the warp ends
  // with value l = (r, j) = (l / kXJ, l % kXJ) of the warp's rows
  static_assert(RPW * kXJ == 32, "one value per lane after the reduce-scatter");
  S vals[32];
#pragma unroll
  for (int r = 0; r < RPW; ++r)
#pragma unroll
    for (int j = 0; j < kXJ; ++j) vals[r * kXJ + j] = acc[r][j];
  warp_reduce_scatter32(vals, lane);
  part[(int64_t)w.w * (kXM * kXJ) + (warp + 8 * (lane / kXJ)) * kXJ + lane % kXJ] = vals[0];
}
// X tile (channel, m0 | j0 << 16, first slot, slices): the K-slice partials summed in
// slice order, so the result does not depend on which item finished first
template <typename S>
__global__ void __launch_bounds__(kXM * kXJ) k_xreduce(DevLayout L, const int4 *__restrict__ groups,
                                                       const S *__restrict__ part, S *__restrict__ X) {
  const int4 g = groups[blockIdx.x];
  const int ch = g.x, m0 = g.y & 0xffff, j0 = g.y >> 16, H = L.H[ch];
  const int mr = threadIdx.x / kXJ, j = threadIdx.x % kXJ;
  if (m0 + mr >= H || j0 + j >= H) return;
  S tot = part[(int64_t)g.z * (kXM * kXJ) + threadIdx.x];
  for (int s = 1; s < g.w; ++s) tot += part[(int64_t)(g.z + s) * (kXM * kXJ) + threadIdx.x];
  X[L.hh2_off[ch] + (m0 + mr) + (int64_t)H * (j0 + j)] = tot;
}
template <typename S>
void launch_xdot(const DevLayout &L, const int4 *work, int nwork, const int4 *groups, int ngroups, const S *V,
                 const S *T, S *part, S *X, cudaStream_t st) {
  if (nwork <= 0) return;
  k_xdot<S><<<nwork, 256, 0, st>>>(L, work, V, T, part);
  k_xreduce<S><<<ngroups, kXM * kXJ, 0, st>>>(L, groups, part, X);
}

// ============================================================================
// I7(k,i) = f(k,i) + 1/2 sum V(kl,cd) T(cd,il), ccm_t2_eqn.f90:1352-1392, from the
// packed X = V_hhpp' T'; only k in {i, partner(i)} is non-zero.  The diagonal
// becomes d2ij (ccm_t2_eqn.f90:81-84).
// ============================================================================
// one warp per (y, which): the lanes take the l of the sum, reduced in a fixed order
template <typename S>
__global__ void k_i7(DevLayout L, const S *__restrict__ X, const S *__restrict__ fdiag, const S *__restrict__ f7,
                     S *d2ij, S *i7off) {
  const int t = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (t >= 2 * L.A) return;
  const int y = t >> 1, which = t & 1;
  const int c = which ? L.partner[y] : y;
  if (which && (c < 0 || c >= L.A)) {
    if (lane == 0) i7off[y] = S(0.0);
    return;
  }
  S acc = S(0.0);
  for (int l = lane; l < L.A; l += 32) {
    const int2 s1 = L.hh_slot[c * L.A + l], s2 = L.hh_slot[y * L.A + l];
    if (s1.y == 0 || s2.y == 0) continue;
    const int ch = s1.x;
    acc += (ssign(s1.y) * ssign(s2.y)) * X[L.hh2_off[ch] + sidx(s1.y) + (int64_t)L.H[ch] * sidx(s2.y)];
  }
  const S tot = from2<S>(warp_sum2(to2(acc)));
  if (lane == 0) {
    const S val = (which ? f7[y] : fdiag[y]) + tot;
    if (which) i7off[y] = val;
    else d2ij[y] = val;
  }
}
template <typename S>
void launch_i7(const DevLayout &L, const S *X, const S *fdiag, const S *f7, S *d2ij, S *i7off, cudaStream_t st) {
  const int64_t threads = (int64_t)2 * L.A * 32;
  k_i7<S><<<(int)((threads + 127) / 128), 128, 0, st>>>(L, X, fdiag, f7, d2ij, i7off);
}

// The same I7 without X: the entries of X it reads, X(slot(c,l), slot(y,l)) for c in
// {y, partner(y)}, as dots of column slot(c,l) of V_hhpp' with column slot(y,l) of T'
// over the channel's packed pp rows (one warp per dot, the sign of both slots applied),
// then the sums over l in the order of k_i7.  About 2 A^2 dots instead of all of X.
template <typename S>
__global__ void k_i7dots(DevLayout L, const S *__restrict__ V, const S *__restrict__ T, S *__restrict__ xd) {
  const int64_t t = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31, A = L.A;
  if (t >= (int64_t)2 * A * A) return;
  const int yw = (int)(t / A), l = (int)(t - (int64_t)yw * A);
  const int y = yw >> 1, which = yw & 1;
  const int c = which ? L.partner[y] : y;
  S acc = S(0.0);
  if (!which || (c >= 0 && c < A)) {
    const int2 s1 = L.hh_slot[c * A + l], s2 = L.hh_slot[y * A + l];
    if (s1.y != 0 && s2.y != 0) {
      const int ch = s1.x, P = L.P[ch];
      const S *v = V + L.t_off[ch] + (int64_t)P * sidx(s1.y);
      const S *u = T + L.t_off[ch] + (int64_t)P * sidx(s2.y);
      for (int k = lane; k < P; k += 32) acc += v[k] * u[k];
      acc = (ssign(s1.y) * ssign(s2.y)) * from2<S>(warp_sum2(to2(acc)));
    }
  }
  if (lane == 0) xd[t] = acc;
}
template <typename S>
__global__ void k_i7sum(DevLayout L, const S *__restrict__ xd, const S *__restrict__ fdiag, const S *__restrict__ f7,
                        S *d2ij, S *i7off) {
  const int t = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (t >= 2 * L.A) return;
  const int y = t >> 1, which = t & 1;
  const int c = which ? L.partner[y] : y;
  if (which && (c < 0 || c >= L.A)) {
    if (lane == 0) i7off[y] = S(0.0);
    return;
  }
  S acc = S(0.0);
  for (int l = lane; l < L.A; l += 32) acc += xd[(int64_t)t * L.A + l];
  const S tot = from2<S>(warp_sum2(to2(acc)));
  if (lane == 0) {
    const S val = (which ? f7[y] : fdiag[y]) + tot;
    if (which) i7off[y] = val;
    else d2ij[y] = val;
  }
}
template <typename S>
void launch_i7_direct(const DevLayout &L, const S *V, const S *T, S *xd, const S *fdiag, const S *f7, S *d2ij, S *i7off,
                      cudaStream_t st) {
  const int64_t t1 = (int64_t)2 * L.A * L.A * 32, t2 = (int64_t)2 * L.A * 32;
  if (t1 == 0) return;
  k_i7dots<S><<<(int)((t1 + 255) / 256), 256, 0, st>>>(L, V, T, xd);
  k_i7sum<S><<<(int)((t2 + 127) / 128), 128, 0, st>>>(L, xd, fdiag, f7, d2ij, i7off);
}
// I9 = V_hhhh + (X_b + dX)
template <typename S>
__global__ void k_i9b(int64_t n, const S *__restrict__ Vhh, const S *__restrict__ Xb, const S *__restrict__ dX, S *I9) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    I9[i] = Vhh[i] + (Xb[i] + dX[i]);
}
template <typename S>
void launch_i9b(int64_t n, const S *Vhh, const S *Xb, const S *dX, S *I9, cudaStream_t st) {
  if (n > 0) k_i9b<S><<<(int)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, st>>>(n, Vhh, Xb, dX, I9);
}

template <typename S>
__global__ void k_i9(int64_t n, const S *__restrict__ Vhh, const S *__restrict__ X, S *I9) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    I9[i] = Vhh[i] + X[i];
}
template <typename S> void launch_i9(const DevLayout &, int64_t n, const S *Vhh, const S *X, S *I9, cudaStream_t st) {
  if (n > 0) k_i9<S><<<(int)std::min<int64_t>((n + 255) / 256, 4096), 256, 0, st>>>(n, Vhh, X, I9);
}

// ============================================================================
// I6(a,c) = f(a,c) - 1/2 sum V(kl,dc) T(da,kl), ccm_t2_eqn.f90:1399-1441, for
// c in {a, partner(a)}; the diagonal becomes d2ab (:86-89).  Two passes:
//  1. k_i6_rows, one thread per packed pp row rho = (p, q), p < q: the three column
//     dots over the packed hole pairs that row feeds, D0 = T_rho . V_rho (into
//     I6(p,p) and I6(q,q)), D1 = T_rho . V_(q,p') (into I6(p,p')) and
//     D2 = T_rho . V_(p,q') (into I6(q,q')), with the antisymmetry signs of the
//     pair slots.  Rows of one channel are adjacent, so the T and V_rho reads are
//     coalesced; they are stored at the row's first element of the T layout.
//  2. k_i6_sum, one warp per (a, c): the sum over d of the dots of the rows (a, d).
// ============================================================================
template <typename S>
__global__ void k_i6_rows(DevLayout L, const int2 *__restrict__ rowtile, const S *__restrict__ T,
                          const S *__restrict__ Vhp, S *__restrict__ D) {
  __shared__ S red[kI6Parts][kI6Rows][3];
  const int2 rt = rowtile[blockIdx.x];
  const int r = threadIdx.x % kI6Rows, part = threadIdx.x / kI6Rows;  // a warp: 32 rows, one part
  const int ch = rt.x, rho = rt.y + r;
  const int P = L.P[ch];
  if (rho >= P) {
    __syncthreads();  // every thread of the block reaches the barrier
    return;
  }
  const int H = L.H[ch], A = L.A, NP = L.NP;
  const int64_t off = L.t_off[ch];
  const int2 po = L.pp_orb[L.pp_off[ch] + rho];
  const int p = po.x, q = po.y;
  // I6(p, p'): d = q, pairs (q, p) and (q, p')
  int i1 = -1, i2 = -1;
  double sg1 = 0.0, sg2 = 0.0;
  const int pp = L.partner[p], qq = L.partner[q];
  if (pp >= A) {
    const int2 s1 = L.pp_slot[(int64_t)(q - A) * NP + (p - A)], s2 = L.pp_slot[(int64_t)(q - A) * NP + (pp - A)];
    if (s1.y != 0 && s2.y != 0) { i1 = sidx(s2.y); sg1 = ssign(s1.y) * ssign(s2.y); }
  }
  // I6(q, q'): d = p, pairs (p, q) and (p, q')
  if (qq >= A) {
    const int2 s1 = L.pp_slot[(int64_t)(p - A) * NP + (q - A)], s2 = L.pp_slot[(int64_t)(p - A) * NP + (qq - A)];
    if (s1.y != 0 && s2.y != 0) { i2 = sidx(s2.y); sg2 = ssign(s1.y) * ssign(s2.y); }
  }
  S d0 = S(0.0), d1 = S(0.0), d2 = S(0.0);
  const S *tc = T + off, *vc = Vhp + off;
  for (int k = part; k < H; k += kI6Parts) {
    const int64_t o = (int64_t)P * k;
    const S t = tc[o + rho];
    d0 += t * vc[o + rho];
    if (i1 >= 0) d1 += t * vc[o + i1];
    if (i2 >= 0) d2 += t * vc[o + i2];
  }
  // the kI6Parts interleaved k partials of a row, summed in part order
  red[part][r][0] = d0;
  red[part][r][1] = d1;
  red[part][r][2] = d2;
  __syncthreads();
  if (part == 0) {
#pragma unroll
    for (int q = 1; q < kI6Parts; ++q) {
      d0 += red[q][r][0];
      d1 += red[q][r][1];
      d2 += red[q][r][2];
    }
    S *dr = D + 3 * (off + rho);
    dr[0] = d0;
    dr[1] = sg1 * d1;
    dr[2] = sg2 * d2;
  }
}

// one block of kI6SumThreads per (a, c): the threads take the d of the sum, reduced in a
// fixed order (lanes by shuffles, then the warps in order)
constexpr int kI6SumThreads = 128;
template <typename S>
__global__ void __launch_bounds__(kI6SumThreads) k_i6_sum(DevLayout L, const S *__restrict__ D,
                                                          const S *__restrict__ fdiag, const S *__restrict__ f6,
                                                          S *d2ab, S *i6off) {
  __shared__ S red[kI6SumThreads / 32];
  const int w = blockIdx.x;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int u = w >> 1, which = w & 1;
  const int x = L.A + u;
  const int c = which ? L.partner[x] : x;
  if (which && c < L.A) {
    if (threadIdx.x == 0) i6off[u] = S(0.0);
    return;
  }
  S acc = S(0.0);
  for (int d = threadIdx.x; d < L.NP; d += kI6SumThreads) {
    const int2 s = L.pp_slot[(int64_t)u * L.NP + d];
    if (s.y == 0) continue;
    const int ch = s.x, rho = sidx(s.y);
    const S *dr = D + 3 * (L.t_off[ch] + rho);
    if (!which) acc += dr[0];
    else acc += (L.pp_orb[L.pp_off[ch] + rho].x == x) ? dr[1] : dr[2];
  }
  const S ws = from2<S>(warp_sum2(to2(acc)));
  if (lane == 0) red[wid] = ws;
  __syncthreads();
  if (threadIdx.x == 0) {
    S tot = red[0];
    for (int q = 1; q < kI6SumThreads / 32; ++q) tot += red[q];
    const S val = (which ? f6[u] : fdiag[x]) - tot;
    if (which) i6off[u] = val;
    else d2ab[u] = val;
  }
}
template <typename S>
void launch_i6(const DevLayout &L, const int2 *rowtile, int nrowtile, S *D, const S *T, const S *Vhp, const S *fdiag,
               const S *f6, S *d2ab, S *i6off, cudaStream_t st) {
  if (nrowtile > 0) k_i6_rows<S><<<nrowtile, kI6Rows * kI6Parts, 0, st>>>(L, rowtile, T, Vhp, D);
  if (L.NP > 0) k_i6_sum<S><<<2 * L.NP, kI6SumThreads, 0, st>>>(L, D, fdiag, f6, d2ab, i6off);
}

// ============================================================================
// R' = conj(V(ij,ab)) (:106-138) + one-body I6/I7 terms (:144-211) + the P(ab)P(ij)
// ring scatter (:840-892) written as a gather of four R_ph entries.
// ============================================================================
template <typename S>
__device__ inline S ring_at(const DevLayout &L, const S *__restrict__ Rph, int a, int i, int j, int b) {
  const int2 s1 = L.ph_slot[(int64_t)(a - L.A) * L.A + i];
  const int2 s2 = L.hp_slot[(int64_t)j * L.NP + (b - L.A)];
  if (s1.x < 0 || s2.x < 0) return S(0.0);
  const int q = s1.x;
  return Rph[L.tph_off[q] + s1.y + (int64_t)L.n_ph[q] * s2.y];
}

// Where the one-body and ring terms of each packed element come from, once per layout:
// omap = signed T' positions (+-(index + 1), 0 = absent) of the I6(b, b'), I6(a, a'),
// I7(j, j') and I7(i, i') terms; rmap = R_ph positions (+1, 0 = absent) of the four
// P(ab)P(ij) ring entries (a i j b), (b i j a), (a j i b), (b j i a).
__global__ void k_rinit_maps(DevLayout L, int4 *__restrict__ omap, int4 *__restrict__ rmap) {
  const int2 tl = L.ttile[blockIdx.x];
  const int ch = tl.x;
  const int P = L.P[ch], H = L.H[ch];
  const int n = P * H;
  const int end = min(tl.y + kTileElems, n);
  const int A = L.A, NP = L.NP;
  const int64_t base = L.t_off[ch];
  auto tpos = [&](int2 s, int64_t rel) -> int {  // signed position of T' entry base + rel
    const int v = (int)(base + rel) + 1;
    return s.y > 0 ? v : -v;
  };
  auto rpos = [&](int a, int i, int j, int b) -> int {
    const int2 s1 = L.ph_slot[(int64_t)(a - A) * A + i];
    const int2 s2 = L.hp_slot[(int64_t)j * NP + (b - A)];
    if (s1.x < 0 || s2.x < 0) return 0;
    return (int)(L.tph_off[s1.x] + s1.y + (int64_t)L.n_ph[s1.x] * s2.y) + 1;
  };
  for (int e = tl.y + threadIdx.x; e < end; e += blockDim.x) {
    const int ij = e / P, ab = e - ij * P;
    const int2 po = L.pp_orb[L.pp_off[ch] + ab];
    const int2 ho = L.hh_orb[L.hh_off[ch] + ij];
    const int a = po.x, b = po.y, i = ho.x, j = ho.y;
    int4 o = make_int4(0, 0, 0, 0);
    const int bb = L.partner[b];
    if (bb >= A) {
      const int2 s = L.pp_slot[(int64_t)(a - A) * NP + (bb - A)];
      if (s.y) o.x = tpos(s, sidx(s.y) + (int64_t)P * ij);
    }
    const int aa = L.partner[a];
    if (aa >= A) {
      const int2 s = L.pp_slot[(int64_t)(b - A) * NP + (aa - A)];
      if (s.y) o.y = tpos(s, sidx(s.y) + (int64_t)P * ij);
    }
    const int jj = L.partner[j];
    if (jj >= 0 && jj < A) {
      const int2 s = L.hh_slot[i * A + jj];
      if (s.y) o.z = tpos(s, ab + (int64_t)P * sidx(s.y));
    }
    const int ii = L.partner[i];
    if (ii >= 0 && ii < A) {
      const int2 s = L.hh_slot[j * A + ii];
      if (s.y) o.w = tpos(s, ab + (int64_t)P * sidx(s.y));
    }
    omap[base + e] = o;
    rmap[base + e] = make_int4(rpos(a, i, j, b), rpos(b, i, j, a), rpos(a, j, i, b), rpos(b, j, i, a));
  }
}
void launch_rinit_maps(const DevLayout &L, int4 *omap, int4 *rmap, cudaStream_t st) {
  if (L.nttile) k_rinit_maps<<<L.nttile, 256, 0, st>>>(L, omap, rmap);
}

template <typename S>
__device__ __forceinline__ S signed_at(const S *__restrict__ T, int m) {
  return m > 0 ? T[m - 1] : S(0.0) - T[-m - 1];
}
template <typename S>
__device__ __forceinline__ S at_or_zero(const S *__restrict__ X, int m) {
  return m ? X[m - 1] : S(0.0);
}

// R' = conj(V) + the one-body I6 / I7 terms + the ring scatter, through the maps
template <typename S>
__global__ void k_rinit(DevLayout L, const int4 *__restrict__ omap, const int4 *__restrict__ rmap, const S *__restrict__ T,
                        const S *__restrict__ Vhp, const S *__restrict__ Rph, const S *__restrict__ i6off,
                        const S *__restrict__ i7off, const S *__restrict__ ring_base, S *__restrict__ ring_out,
                        S *__restrict__ R) {
  const int2 tl = L.ttile[blockIdx.x];
  const int ch = tl.x;
  const int P = L.P[ch], H = L.H[ch];
  const int n = P * H;  // < 2^31 per channel
  const int end = min(tl.y + kTileElems, n);
  const int A = L.A;
  const int64_t base = L.t_off[ch];
  for (int e = tl.y + threadIdx.x; e < end; e += blockDim.x) {
    const int4 o = omap[base + e];
    const int4 m = rmap[base + e];
    S r = conj_(Vhp[base + e]);
    if (o.x | o.y) {
      const int ab = e % P;
      const int2 po = L.pp_orb[L.pp_off[ch] + ab];
      if (o.x) r += i6off[po.y - A] * signed_at(T, o.x);
      if (o.y) r -= i6off[po.x - A] * signed_at(T, o.y);
    }
    if (o.z | o.w) {
      const int ij = e / P;
      const int2 ho = L.hh_orb[L.hh_off[ch] + ij];
      if (o.z) r -= i7off[ho.y] * signed_at(T, o.z);
      if (o.w) r += i7off[ho.x] * signed_at(T, o.w);
    }
    const S ring = at_or_zero(Rph, m.x) - at_or_zero(Rph, m.y) - at_or_zero(Rph, m.z) + at_or_zero(Rph, m.w);
    if (ring_out) ring_out[base + e] = ring;  // the ring term of this R_ph, kept per amplitude
    r += ring_base ? ring_base[base + e] + ring : ring;
    R[base + e] = r;
  }
}
template <typename S>
void launch_rinit(const DevLayout &L, const int4 *omap, const int4 *rmap, const S *T, const S *Vhp, const S *Rph,
                  const S *i6off, const S *i7off, const S *ring_base, S *ring_out, S *R, cudaStream_t st) {
  if (L.nttile)
    k_rinit<S><<<L.nttile, 256, 0, st>>>(L, omap, rmap, T, Vhp, Rph, i6off, i7off, ring_base, ring_out, R);
}

// ============================================================================
// Update / energy / residual norm (diis_t1t2 :93-126, ccd_energy_save, and
// ||R - D T||).  Partials: [E.re, E.im, |R-DT|^2] per block.  Dressed denominator
// d2ij(i)+d2ij(j)-d2ab(a)-d2ab(b) in the reference's evaluation order.
// ============================================================================
template <typename S>
__global__ void k_update(DevLayout L, int mode, S *__restrict__ T, const S *__restrict__ R, const S *__restrict__ Vhp,
                         const S *__restrict__ d2ij, const S *__restrict__ d2ab, S *__restrict__ hist_t,
                         typename StepOf<S>::type *__restrict__ hist_e, double *partial) {
  const int2 tl = L.ttile[blockIdx.x];
  const int ch = tl.x;
  const int P = L.P[ch], H = L.H[ch];
  const int n = P * H;  // < 2^31 per channel
  const int end = min(tl.y + kTileElems, n);
  double v[3] = {0.0, 0.0, 0.0};
  const int A = L.A;
  for (int e = tl.y + threadIdx.x; e < end; e += blockDim.x) {
    const int64_t g = L.t_off[ch] + e;
    const S t = T[g];
    const S vij = Vhp[g];
    if (mode == 2) {
      const S pr = t * vij;
      v[0] += real_(pr);
      if constexpr (ScalarOf<S>::complex) v[1] += imag_(pr);
      continue;
    }
    const int ij = e / P, ab = e - ij * P;
    const int2 po = L.pp_orb[L.pp_off[ch] + ab];
    const int2 ho = L.hh_orb[L.hh_off[ch] + ij];
    const S D = ((d2ij[ho.x] + d2ij[ho.y]) - d2ab[po.x - A]) - d2ab[po.y - A];
    const S r = R[g];
    const S q = r - D * t;  // the Jacobi step times D
    v[2] += abs2(q);
    S tn = t;
    if (mode == 0) {
      tn = 0.75 * t + 0.25 * (r / D);
      T[g] = tn;
      hist_t[g] = tn;
    } else if (mode == 1) {
      if constexpr (ScalarOf<S>::complex) {
        const S tj = r / D;
        hist_t[g] = tj;
        const S st = tj - t;
        hist_e[g] = cplxf{__double2float_rn(st.re), __double2float_rn(st.im)};
      } else {
        // the step q / D to FP32 accuracy (an FP64 division is a long sequence on this
        // GPU's narrow FP64 pipe); t + step keeps the fixed point exact, since the step
        // vanishes with the residual
        const float step = __fdiv_rn(__double2float_rn(q), __double2float_rn(D));
        hist_t[g] = t + (S)step;
        hist_e[g] = step;
      }
    }
    const S pr = tn * vij;
    v[0] += real_(pr);
    if constexpr (ScalarOf<S>::complex) v[1] += imag_(pr);
  }
  block_partial<3>(v, partial);
}
template <typename S>
void launch_update(const DevLayout &L, int mode, S *T, const S *R, const S *Vhp, const S *d2ij, const S *d2ab, S *hist_t,
                   typename StepOf<S>::type *hist_e, double *partial, double *out4, cudaStream_t st) {
  if (!L.nttile) return;
  k_update<S><<<L.nttile, 256, 0, st>>>(L, mode, T, R, Vhp, d2ij, d2ab, hist_t, hist_e, partial);
  finish(partial, L.nttile, 3, out4, st);
}

// ============================================================================
// dot products and DIIS helpers
// ============================================================================
constexpr int kMaxDots = 16;
template <typename S>
struct PtrPack {
  const S *p[kMaxDots];
};

template <typename S>
__global__ void k_dots(int64_t n, const S *__restrict__ a, PtrPack<S> bs, int nb, int conj_a, double *partial) {
  double v[2 * kMaxDots];
#pragma unroll
  for (int k = 0; k < 2 * kMaxDots; ++k) v[k] = 0.0;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    const S av = conj_a ? conj_(a[x]) : a[x];
#pragma unroll
    for (int k = 0; k < kMaxDots; ++k) {
      if (k < nb) {
        if constexpr (ScalarOf<S>::complex) {
          const S pr = av * bs.p[k][x];
          v[2 * k] += real_(pr);
          v[2 * k + 1] += imag_(pr);
        } else {  // no FP64 additions of a zero imaginary part
          v[2 * k] = fma(real_(av), real_(bs.p[k][x]), v[2 * k]);
        }
      }
    }
  }
  block_partial<2 * kMaxDots>(v, partial);
}
template <typename S>
void launch_dots(int64_t n, const S *a, const S *const *bs, int nb, int conj_a, double *partial, double *out, cudaStream_t st) {
  PtrPack<S> pk{};
  for (int k = 0; k < nb && k < kMaxDots; ++k) pk.p[k] = bs[k];
  const int blocks = 608;
  k_dots<S><<<blocks, 256, 0, st>>>(n, a, pk, nb, conj_a, partial);
  finish(partial, blocks, 2 * kMaxDots, out, st);
}

// Standard-mode update with the Gram row of its step in the same pass.  Per amplitude:
// D from the dressed denominators (hole-pair sums staged per tile in shared memory, the
// same association as k_update), q = R - D t in FP64, the step q/D to FP32 accuracy,
// hist_t = t + step, hist_e = step; the energy sum t V in FP64, and |q|^2 and
// Re(conj(step) hist_e[j]) in FP32 per thread (FP64 across warps and blocks).  One pass,
// one launch and one host copy per iteration instead of an update and a dots pass.  The
// FP32 step vanishes with the residual, so the fixed point is the FP64 one.
constexpr int kUpdStdBlocks = 608;
constexpr int kUpdStdNV = 4 + kMaxDots;  // E re, E im, |q|^2, error word, Gram row
__device__ inline float warp_sum_f(float x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}
// the step q / D to FP32 accuracy (an FP64 division is a long sequence on this GPU's
// narrow FP64 pipe), its |q|^2 contribution and its Gram products
__device__ inline float upd_step(double q, double D, float &r2) {
  const float qf = __double2float_rn(q);
  r2 = fmaf(qf, qf, r2);
  return __fdiv_rn(qf, __double2float_rn(D));
}
__device__ inline cplxf upd_step(cplx q, cplx D, float &r2) {
  const float qr = __double2float_rn(q.re), qi = __double2float_rn(q.im);
  const float dr = __double2float_rn(D.re), di = __double2float_rn(D.im);
  r2 = fmaf(qr, qr, fmaf(qi, qi, r2));
  const float den = fmaf(dr, dr, di * di);
  return cplxf{__fdiv_rn(fmaf(qr, dr, qi * di), den), __fdiv_rn(fmaf(qi, dr, -qr * di), den)};
}
__device__ inline double add_step(double t, float s) { return t + (double)s; }
__device__ inline cplx add_step(cplx t, cplxf s) { return cplx(t.re + (double)s.re, t.im + (double)s.im); }
__device__ inline float gram_dot(float a, float b) { return a * b; }
__device__ inline float gram_dot(cplxf a, cplxf b) { return fmaf(a.re, b.re, a.im * b.im); }
template <typename S>
__global__ void __launch_bounds__(256) k_update_std(DevLayout L, const S *__restrict__ T, const S *__restrict__ R,
                                                    const S *__restrict__ Vhp, const S *__restrict__ d2ij,
                                                    const S *__restrict__ d2ab, S *__restrict__ hist_t,
                                                    typename StepOf<S>::type *__restrict__ hist_e,
                                                    PtrPack<typename StepOf<S>::type> es, int nb, int self,
                                                    const int *err, double *partial) {
  using E = typename StepOf<S>::type;
  __shared__ S sdij[kTileElems];  // hole-pair sums of one tile (at most kTileElems rows)
  __shared__ double red[kUpdStdNV][8];
  double e_re = 0.0, e_im = 0.0;
  float r2 = 0.0f, f[kMaxDots];
#pragma unroll
  for (int k = 0; k < kMaxDots; ++k) f[k] = 0.0f;
  const int A = L.A;
  for (int tix = blockIdx.x; tix < L.nttile; tix += gridDim.x) {
    const int2 tl = L.ttile[tix];
    const int ch = tl.x;
    const int P = L.P[ch];
    const int end = min(tl.y + kTileElems, P * L.H[ch]);
    const int ij0 = tl.y / P, nij = (end - 1) / P - ij0 + 1;
    __syncthreads();  // the previous tile's sums are no longer read
    for (int i = threadIdx.x; i < nij; i += blockDim.x) {
      const int2 ho = L.hh_orb[L.hh_off[ch] + ij0 + i];
      sdij[i] = d2ij[ho.x] + d2ij[ho.y];
    }
    __syncthreads();
    const int64_t base = L.t_off[ch];
    const int2 *pporb = L.pp_orb + L.pp_off[ch];
    for (int el = tl.y + threadIdx.x; el < end; el += blockDim.x) {
      const int64_t g = base + el;
      const S t = T[g], vij = Vhp[g], r = R[g];
      const int ij = el / P, ab = el - ij * P;
      const int2 po = pporb[ab];
      const S D = (sdij[ij - ij0] - d2ab[po.x - A]) - d2ab[po.y - A];
      const S q = r - D * t;
      const E step = upd_step(q, D, r2);
      hist_t[g] = add_step(t, step);
      hist_e[g] = step;
      if constexpr (ScalarOf<S>::complex) {
        const S pr = t * vij;
        e_re += real_(pr);
        e_im += imag_(pr);
      } else {
        e_re = fma(t, vij, e_re);
      }
#pragma unroll
      for (int k = 0; k < kMaxDots; ++k)
        if (k < nb) f[k] += gram_dot(step, k == self ? step : es.p[k][g]);
    }
  }
  // warp sums (FP32 values in FP32), then FP64 across the warps
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  e_re = warp_sum(e_re);
  e_im = warp_sum(e_im);
  r2 = warp_sum_f(r2);
#pragma unroll
  for (int k = 0; k < kMaxDots; ++k)
    if (k < nb) f[k] = warp_sum_f(f[k]);
  if (lane == 0) {
    red[0][wid] = e_re;
    red[1][wid] = e_im;
    red[2][wid] = (double)r2;
    red[3][wid] = (err && blockIdx.x == 0 && wid == 0) ? (double)*err : 0.0;  // carried to the host in the same copy
#pragma unroll
    for (int k = 0; k < kMaxDots; ++k) red[4 + k][wid] = k < nb ? (double)f[k] : 0.0;
  }
  __syncthreads();
  if (threadIdx.x < kUpdStdNV) {
    double x = 0.0;
    for (int w = 0; w < nw; ++w) x += red[threadIdx.x][w];
    partial[(int64_t)blockIdx.x * kUpdStdNV + threadIdx.x] = x;
  }
}
template <typename S>
void launch_update_std(const DevLayout &L, const S *T, const S *R, const S *Vhp, const S *d2ij, const S *d2ab, S *hist_t,
                       typename StepOf<S>::type *hist_e, const typename StepOf<S>::type *const *es, int nb, int self,
                       const int *err, double *partial, double *out, cudaStream_t st) {
  if (!L.nttile) return;
  PtrPack<typename StepOf<S>::type> pk{};
  for (int k = 0; k < nb; ++k) pk.p[k] = es[k];
  const int blocks = std::min(L.nttile, kUpdStdBlocks);
  k_update_std<S><<<blocks, 256, 0, st>>>(L, T, R, Vhp, d2ij, d2ab, hist_t, hist_e, pk, nb, self, err, partial);
  finish(partial, blocks, kUpdStdNV, out, st);
}

// Gram matrix of consecutive differences d_i = t_{i+1} - t_i, B_ij = sum d_i d_j
// without conjugation (ccm_diis.f90:134-150).  Upper triangle, 2 doubles per entry.
template <typename S>
__global__ void k_diis_gram(int64_t n, PtrPack<S> cols, int nstep, double *partial) {
  constexpr int MAXD = 5;
  double v[2 * 15];
#pragma unroll
  for (int k = 0; k < 30; ++k) v[k] = 0.0;
  const int nd = nstep - 1;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    S d[MAXD];
#pragma unroll
    for (int i = 0; i < MAXD; ++i) d[i] = (i < nd) ? cols.p[i + 1][x] - cols.p[i][x] : S(0.0);
    int k = 0;
#pragma unroll
    for (int i = 0; i < MAXD; ++i)
#pragma unroll
      for (int j = i; j < MAXD; ++j) {
        const S pr = d[i] * d[j];
        v[2 * k] += real_(pr);
        v[2 * k + 1] += imag_(pr);
        ++k;
      }
  }
  block_partial<30>(v, partial);
}
template <typename S>
void launch_diis_gram(int64_t n, const S *const *cols, int nstep, double *partial, double *out, cudaStream_t st) {
  PtrPack<S> pk{};
  for (int k = 0; k < nstep && k < kMaxDots; ++k) pk.p[k] = cols[k];
  const int blocks = 608;
  k_diis_gram<S><<<blocks, 256, 0, st>>>(n, pk, nstep, partial);
  finish(partial, blocks, 30, out, st);
}

template <typename S>
struct CoefPack {
  double re[kMaxDots], im[kMaxDots];
};
template <typename S>
__global__ void k_combine(int64_t n, PtrPack<S> xs, CoefPack<S> c, int m, S *y) {
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    S acc = S(0.0);
    for (int i = 0; i < m; ++i) acc += make_scalar<S>(c.re[i], c.im[i]) * xs.p[i][x];
    y[x] = acc;
  }
}
template <typename S>
void launch_combine(int64_t n, const S *const *xs, const double *coef, int m, S *y, cudaStream_t st) {
  PtrPack<S> pk{};
  CoefPack<S> c{};
  for (int k = 0; k < m && k < kMaxDots; ++k) {
    pk.p[k] = xs[k];
    c.re[k] = coef[2 * k];
    c.im[k] = coef[2 * k + 1];
  }
  k_combine<S><<<1216, 256, 0, st>>>(n, pk, c, m, y);
}

// ============================================================================
// Interaction blocks handed over in the reference's ordered layout
// ============================================================================
// kind 3: V_hhpp(n_hh, n_pp) -> Vhp'(ij', ab') at [ij'*P + ab']
// kind 6: V_pppp(n_pp, n_pp) -> Vpp'(ab', cd') at [ab'*P + cd']
// kind 1: V_hhhh(n_hh, n_hh) of the matching hhhh channel -> Vhh'(kl', ij') col-major
template <typename S>
__global__ void k_pack_vblock(DevLayout L, int kind, int ch, int n_rows, const double *__restrict__ stage,
                              S *__restrict__ dst, int *flag) {
  const int P = L.P[ch], H = L.H[ch];
  int64_t n;
  if (kind == 3) n = (int64_t)H * P;
  else if (kind == 6) n = (int64_t)P * P;
  else n = (int64_t)H * H;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t src, o;
    if (kind == 3) {
      const int ij = (int)(e / P), ab = (int)(e % P);
      src = L.hh_row[L.hh_off[ch] + ij] + (int64_t)n_rows * L.pp_row[L.pp_off[ch] + ab];
      o = L.t_off[ch] + e;
    } else if (kind == 6) {
      const int r = (int)(e / P), c = (int)(e % P);
      src = L.pp_row[L.pp_off[ch] + r] + (int64_t)n_rows * L.pp_row[L.pp_off[ch] + c];
      o = L.vpp_off[ch] + e;
    } else {
      const int r = (int)(e % H), c = (int)(e / H);
      src = L.hh_row[L.hh_off[ch] + r] + (int64_t)n_rows * L.hh_row[L.hh_off[ch] + c];
      o = L.hh2_off[ch] + e;
    }
    dst[o] = cvt_in<S>(stage + 2 * src, flag);
  }
}
template <typename S>
void launch_pack_vblock(const DevLayout &L, int kind, int ch, int n_rows, const double *stage, S *dst, int *flag, cudaStream_t st) {
  k_pack_vblock<S><<<1216, 256, 0, st>>>(L, kind, ch, n_rows, stage, dst, flag);
}

// Kinds 3 and 6 from host memory: dst(r, c) at base + r * P + c (row-major) from the
// reference block's (row_map[r], col_map[c]) element (column-major, leading dimension
// n_rows).  A 32 x 32 tile is read down its columns (consecutive source rows, so each
// host cache line is fetched once) and written along its rows.
template <typename S>
__global__ void __launch_bounds__(256) k_pack_vblock_tr(DevLayout L, int kind, int ch, int n_rows, int R, int P,
                                                        const double *__restrict__ src, S *__restrict__ dst, int *flag) {
  __shared__ S tile[32][33];
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  const int *row_map = kind == 3 ? L.hh_row + L.hh_off[ch] : L.pp_row + L.pp_off[ch];
  const int *col_map = L.pp_row + L.pp_off[ch];
  const int64_t base = kind == 3 ? L.t_off[ch] : L.vpp_off[ch];
  const int r = r0 + tx;
  const int64_t srow = r < R ? row_map[r] : 0;
#pragma unroll
  for (int j = 0; j < 32; j += 8) {
    const int c = c0 + ty + j;
    if (r < R && c < P) tile[ty + j][tx] = cvt_in<S>(src + 2 * (srow + (int64_t)n_rows * col_map[c]), flag);
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < 32; j += 8) {
    const int rr = r0 + ty + j, c = c0 + tx;
    if (rr < R && c < P) dst[base + (int64_t)rr * P + c] = tile[tx][ty + j];
  }
}
// Kind 6 from host memory, one source column at a time: a block reads the rows of packed
// column c from the reference block's column col_map[c] (contiguous in host memory) and
// writes them down the packed column (stride P; the blocks on neighbouring columns fill
// the same destination lines in L2).  The blocks in flight read a few contiguous columns
// each, so the host pages they touch at once stay few: reads spread over 32 columns per
// block (the tile kernel above) reach a fraction of the link rate on a family of tens of
// GB.
template <typename S>
__global__ void __launch_bounds__(512) k_pack_vpp_cols(DevLayout L, int ch, int n_rows, int P,
                                                       const double *__restrict__ src, S *__restrict__ dst, int *flag) {
  const int *row_map = L.pp_row + L.pp_off[ch];
  const int *col_map = L.pp_row + L.pp_off[ch];
  const int64_t base = L.vpp_off[ch];
  for (int c = blockIdx.x; c < P; c += gridDim.x) {
    const double *col = src + 2 * (int64_t)n_rows * col_map[c];
    for (int r = threadIdx.x; r < P; r += blockDim.x) dst[base + (int64_t)r * P + c] = cvt_in<S>(col + 2 * row_map[r], flag);
  }
}
template <typename S>
void launch_pack_vblock_host(const DevLayout &L, int kind, int ch, int n_rows, int rows_packed, int cols_packed,
                             const double *src, S *dst, int *flag, cudaStream_t st) {
  if (rows_packed <= 0 || cols_packed <= 0) return;
  if (kind == 6) {
    k_pack_vpp_cols<S><<<std::min(cols_packed, 304), 512, 0, st>>>(L, ch, n_rows, cols_packed, src, dst, flag);
  } else if (kind == 3) {
    const dim3 grid((cols_packed + 31) / 32, (rows_packed + 31) / 32);
    k_pack_vblock_tr<S><<<grid, dim3(32, 8), 0, st>>>(L, kind, ch, n_rows, rows_packed, cols_packed, src, dst, flag);
  } else {
    // kind 1 reads consecutive source rows already
    k_pack_vblock<S><<<1216, 256, 0, st>>>(L, kind, ch, n_rows, src, dst, flag);
  }
}

// one CTA per job; 16-byte copies where both ends and the length allow
__global__ void k_copy_jobs(const CopyJob *__restrict__ jobs) {
  const CopyJob j = jobs[blockIdx.x];
  const bool vec = ((reinterpret_cast<uintptr_t>(j.src) | reinterpret_cast<uintptr_t>(j.dst)) & 15) == 0;
  if (vec) {
    const int64_t n2 = j.n / 2;
    const double2 *s2 = reinterpret_cast<const double2 *>(j.src);
    double2 *d2 = reinterpret_cast<double2 *>(j.dst);
    for (int64_t i = threadIdx.x; i < n2; i += blockDim.x) d2[i] = s2[i];
    if ((j.n & 1) && threadIdx.x == 0) j.dst[j.n - 1] = j.src[j.n - 1];
  } else {
    for (int64_t i = threadIdx.x; i < j.n; i += blockDim.x) j.dst[i] = j.src[i];
  }
}
void launch_copy_jobs(const CopyJob *jobs, int njobs, cudaStream_t st) {
  if (njobs > 0) k_copy_jobs<<<njobs, 256, 0, st>>>(jobs);
}

// W(ia, jb) = -V_hphp(ib, ja), the constant part of I4 (ccm_t2_eqn.f90:740-780)
template <typename S>
__global__ void k_build_w(DevLayout L, const int2 *__restrict__ hp4_slot, const int64_t *__restrict__ v4_off,
                          const int *__restrict__ n4, const double *__restrict__ v4, S *__restrict__ W, int *flag) {
  for (int q = blockIdx.x; q < L.nph; q += gridDim.x) {
    const int nhp = L.n_hp[q];
    const int64_t n = (int64_t)nhp * nhp;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
      const int r = (int)(e % nhp), c = (int)(e / nhp);
      const int2 ia = L.hp_orb[L.hp_off[q] + r];
      const int2 jb = L.hp_orb[L.hp_off[q] + c];
      const int2 sib = hp4_slot[(int64_t)ia.x * L.NP + (jb.y - L.A)];
      const int2 sja = hp4_slot[(int64_t)jb.x * L.NP + (ia.y - L.A)];
      S w = S(0.0);
      if (sib.x >= 0 && sja.x >= 0) {
        const int c4 = sib.x;
        const S v = cvt_in<S>(v4 + 2 * (v4_off[c4] + sib.y + (int64_t)n4[c4] * sja.y), flag);
        w = S(0.0) - v;
      }
      W[L.i4_off[q] + e] = w;
    }
  }
}
template <typename S>
void launch_build_w(const DevLayout &L, const int2 *hp4_slot, const int64_t *v4_off, const int *n4, const double *v4, S *W,
                    int *flag, cudaStream_t st) {
  if (L.nph) k_build_w<S><<<min(L.nph, 4096), 256, 0, st>>>(L, hp4_slot, v4_off, n4, v4, W, flag);
}

// V_ph(ia, bj) = V(ij, ab): the `amat` gather of ccm_t2_eqn.f90:694-716, done once
template <typename S>
__global__ void k_build_vph(DevLayout L, const S *__restrict__ Vhp, S *__restrict__ Vph) {
  for (int q = blockIdx.x; q < L.nph; q += gridDim.x) {
    const int nhp = L.n_hp[q], nph = L.n_ph[q];
    const int64_t n = (int64_t)nhp * nph;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
      const int r = (int)(e % nhp), c = (int)(e / nhp);
      const int2 ia = L.hp_orb[L.hp_off[q] + r];
      const int2 bj = L.ph_orb[L.ph_off[q] + c];
      const int2 sij = L.hh_slot[ia.x * L.A + bj.y];
      const int2 sab = L.pp_slot[(int64_t)(ia.y - L.A) * L.NP + (bj.x - L.A)];
      S v = S(0.0);
      if (sij.y && sab.y) {
        const int ch = sij.x;
        v = (ssign(sij.y) * ssign(sab.y)) * Vhp[L.t_off[ch] + (int64_t)sidx(sij.y) * L.P[ch] + sidx(sab.y)];
      }
      Vph[L.vph_off[q] + e] = v;
    }
  }
}
template <typename S> void launch_build_vph(const DevLayout &L, const S *Vhp, S *Vph, cudaStream_t st) {
  if (L.nph) k_build_vph<S><<<min(L.nph, 4096), 256, 0, st>>>(L, Vhp, Vph);
}

// ============================================================================
// Device potentials (generation of every block on the GPU)
// ============================================================================


// antisymmetrised element; with pair factors (complex engines, chiral-like kind) the
// relativity and regulator factors come from the per-pair table instead
template <typename S>
__device__ inline S gen_anti(const DevOrbits &O, const DevPotential &P, int p, int q, int r, int s, const double *fpq,
                             const double *frs) {
  if constexpr (ScalarOf<S>::complex) {
    if (fpq) return pot::chiral_anti_factored(O, P, p, q, r, s, *fpq, *frs);
  }
  return pot::vanti<S>(O, P, p, q, r, s);
}
// F(pq) (chiral_pair_factor) of every packed pp pair, every packed hh pair and every
// (hole, particle) pair, once per generation: pairf = [pp | hh | hp (A x NP)]
__global__ void k_pair_factors(DevLayout L, DevOrbits O, int npp, int nhh, double *pairf) {
  const int64_t nhp = (int64_t)L.A * L.NP, n = npp + nhh + nhp;
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    int p, q;
    if (x < npp) { p = L.pp_orb[x].x; q = L.pp_orb[x].y; }
    else if (x < npp + nhh) { p = L.hh_orb[x - npp].x; q = L.hh_orb[x - npp].y; }
    else { const int64_t y = x - npp - nhh; p = (int)(y / L.NP); q = L.A + (int)(y % L.NP); }
    pairf[x] = pot::chiral_pair_factor(O, p, q);
  }
}
template <typename S>
__global__ void k_gen_tblocks(DevLayout L, DevOrbits O, DevPotential P, const double *ppf, const double *hhf, S *Vhp) {
  const int2 tl = L.ttile[blockIdx.x];
  const int ch = tl.x, Pc = L.P[ch], H = L.H[ch];
  const int64_t n = (int64_t)Pc * H, end = min((int64_t)tl.y + kTileElems, n);
  for (int64_t e = tl.y + threadIdx.x; e < end; e += blockDim.x) {
    const int ij = (int)(e / Pc), ab = (int)(e % Pc);  // Vhp'(ij', ab') at ij'*P + ab'
    const int hi = L.hh_off[ch] + ij, pi = L.pp_off[ch] + ab;
    const int2 h = L.hh_orb[hi], p = L.pp_orb[pi];
    Vhp[L.t_off[ch] + e] = gen_anti<S>(O, P, h.x, h.y, p.x, p.y, hhf ? hhf + hi : nullptr, ppf ? ppf + pi : nullptr);
  }
}
// V_pppp' is Hermitian, <cd|V|ab> = conj(<ab|V|cd>): the elements on and above the
// diagonal are generated and mirrored, which halves the FP64 work of the largest block
// family.  The elements below the diagonal are written by the thread of their mirror.
template <typename S>
__global__ void k_gen_vpp(DevLayout L, DevOrbits O, DevPotential P, const double *ppf, S *Vpp) {
  const int2 tl = L.vtile[blockIdx.x];
  const int ch = tl.x, Pc = L.P[ch];
  const int64_t n = (int64_t)Pc * Pc, end = min((int64_t)tl.y + kTileElems, n);
  S *V = Vpp + L.vpp_off[ch];
  for (int64_t e = tl.y + threadIdx.x; e < end; e += blockDim.x) {
    const int r = (int)(e / Pc), c = (int)(e % Pc);
    if (r > c) continue;
    const int ri = L.pp_off[ch] + r, ci = L.pp_off[ch] + c;
    const int2 x = L.pp_orb[ri], y = L.pp_orb[ci];
    const S v = gen_anti<S>(O, P, x.x, x.y, y.x, y.y, ppf ? ppf + ri : nullptr, ppf ? ppf + ci : nullptr);
    V[e] = v;
    if (r != c) V[(int64_t)c * Pc + r] = conj_(v);
  }
}
template <typename S>
__global__ void k_gen_vhh(DevLayout L, DevOrbits O, DevPotential P, S *Vhh) {
  for (int ch = blockIdx.x; ch < L.nch; ch += gridDim.x) {
    const int H = L.H[ch];
    for (int e = threadIdx.x; e < H * H; e += blockDim.x) {
      const int r = e % H, c = e / H;
      const int2 x = L.hh_orb[L.hh_off[ch] + r], y = L.hh_orb[L.hh_off[ch] + c];
      Vhh[L.hh2_off[ch] + e] = pot::vanti<S>(O, P, x.x, x.y, y.x, y.y);
    }
  }
}
template <typename S>
__global__ void k_gen_w(DevLayout L, DevOrbits O, DevPotential P, const double *hpf, S *W) {
  for (int q = blockIdx.x; q < L.nph; q += gridDim.x) {
    const int nhp = L.n_hp[q];
    for (int64_t e = threadIdx.x; e < (int64_t)nhp * nhp; e += blockDim.x) {
      const int r = (int)(e % nhp), c = (int)(e / nhp);
      const int2 ia = L.hp_orb[L.hp_off[q] + r], jb = L.hp_orb[L.hp_off[q] + c];
      // -<ib|V|ja>_A; pair factors F(ib), F(ja) from the (hole, particle) table
      const double *fib = hpf ? hpf + (int64_t)ia.x * L.NP + (jb.y - L.A) : nullptr;
      const double *fja = hpf ? hpf + (int64_t)jb.x * L.NP + (ia.y - L.A) : nullptr;
      W[L.i4_off[q] + e] = S(0.0) - gen_anti<S>(O, P, ia.x, jb.y, jb.x, ia.y, fib, fja);
    }
  }
}
// Fock pieces: f(p,p), f(x, partner) for particles, f(partner, y) for holes;
// normal_ordered_hamiltonian, ccm_main.f90:1586-1657.  E0 :1661-1684.
template <typename S>
__global__ void k_gen_fock(DevLayout L, DevOrbits O, DevPotential P, S *fdiag, S *f6, S *f7) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= L.ns) return;
  S d = S(O.e[p]);
  for (int h = 0; h < L.A; ++h) d += pot::vanti<S>(O, P, h, p, h, p);
  fdiag[p] = d;
  const int pb = L.partner[p];
  if (p >= L.A) {
    S o = S(0.0);
    if (pb >= L.A)
      for (int h = 0; h < L.A; ++h) o += pot::vanti<S>(O, P, h, p, h, pb);
    f6[p - L.A] = o;
  } else {
    S o = S(0.0);
    if (pb >= 0 && pb < L.A)
      for (int h = 0; h < L.A; ++h) o += pot::vanti<S>(O, P, h, pb, h, p);
    f7[p] = o;
  }
}
template <typename S>
__global__ void k_gen_e0(DevLayout L, DevOrbits O, DevPotential P, double *e0) {
  double v[2] = {0.0, 0.0};
  for (int x = threadIdx.x; x < L.A * L.A; x += blockDim.x) {
    const int i = x / L.A, j = x % L.A;
    const S w = pot::vanti<S>(O, P, i, j, i, j);
    v[0] += 0.5 * real_(w);
    v[1] += 0.5 * imag_(w);
  }
  for (int i = threadIdx.x; i < L.A; i += blockDim.x) v[0] += O.e[i];
  block_partial<2>(v, e0);
}

template <typename S>
void launch_generate(const DevLayout &L, const DevOrbits &O, const DevPotential &pot, S *Vhp, S *Vpp, S *Vhh, S *W,
                     S *fdiag, S *f6, S *f7, double *e0, double *pairf, int npp, int nhh, cudaStream_t st) {
  const bool factored = ScalarOf<S>::complex && pot.kind == 1 && pairf;
  double *ppf = factored ? pairf : nullptr, *hhf = factored ? pairf + npp : nullptr;
  double *hpf = factored ? pairf + npp + nhh : nullptr;
  if (factored) k_pair_factors<<<1216, 256, 0, st>>>(L, O, npp, nhh, pairf);
  if (L.nttile) k_gen_tblocks<S><<<L.nttile, 256, 0, st>>>(L, O, pot, ppf, hhf, Vhp);
  if (L.nvtile) k_gen_vpp<S><<<L.nvtile, 256, 0, st>>>(L, O, pot, ppf, Vpp);
  if (L.nch) k_gen_vhh<S><<<min(L.nch, 4096), 128, 0, st>>>(L, O, pot, Vhh);
  if (L.nph) k_gen_w<S><<<min(L.nph, 4096), 128, 0, st>>>(L, O, pot, hpf, W);
  k_gen_fock<S><<<(L.ns + 127) / 128, 128, 0, st>>>(L, O, pot, fdiag, f6, f7);
  k_gen_e0<S><<<1, 256, 0, st>>>(L, O, pot, e0);
}

template <typename S>
__global__ void k_gen_ordered(DevOrbits O, DevPotential P, const int2 *__restrict__ rows, const int2 *__restrict__ cols,
                              int nr, int nc, int swap, double *__restrict__ out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)nr * nc; e += (int64_t)gridDim.x * blockDim.x) {
    const int2 x = rows[e % nr], y = cols[e / nr];
    const S v = swap ? pot::vanti<S>(O, P, y.x, y.y, x.x, x.y) : pot::vanti<S>(O, P, x.x, x.y, y.x, y.y);
    out[2 * e] = real_(v);
    out[2 * e + 1] = imag_(v);
  }
}
template <typename S>
void launch_gen_ordered(const DevOrbits &O, const DevPotential &pot, const int2 *rows, const int2 *cols, int nr, int nc,
                        int swap, double *out, cudaStream_t st) {
  if ((int64_t)nr * nc > 0) k_gen_ordered<S><<<1216, 256, 0, st>>>(O, pot, rows, cols, nr, nc, swap, out);
}

template <typename S>
__global__ void k_unpack_vblock(DevLayout L, int kind, int ch, int nr, int nc, const int *__restrict__ rs,
                                const int *__restrict__ cs, const S *__restrict__ src, double *__restrict__ out) {
  const int P = L.P[ch], H = L.H[ch];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)nr * nc; e += (int64_t)gridDim.x * blockDim.x) {
    const int r = rs[e % nr], c = cs[e / nr];
    S v = S(0.0);
    if (r && c) {
      const double sg = ssign(r) * ssign(c);
      if (kind == 3) v = sg * src[L.t_off[ch] + (int64_t)sidx(r) * P + sidx(c)];
      else if (kind == 6) v = sg * src[L.vpp_off[ch] + (int64_t)sidx(r) * P + sidx(c)];
      else v = sg * src[L.hh2_off[ch] + sidx(r) + (int64_t)H * sidx(c)];
    }
    out[2 * e] = real_(v);
    out[2 * e + 1] = imag_(v);
  }
}
template <typename S>
void launch_unpack_vblock(const DevLayout &L, int kind, int ch, int n_rows, int n_cols, const int *row_sgn,
                          const int *col_sgn, const S *src, double *out, cudaStream_t st) {
  if ((int64_t)n_rows * n_cols > 0)
    k_unpack_vblock<S><<<1216, 256, 0, st>>>(L, kind, ch, n_rows, n_cols, row_sgn, col_sgn, src, out);
}

template <typename S>
__global__ void k_axpy(int64_t n, const S *__restrict__ x, S *__restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) y[i] += x[i];
}
template <typename S> void launch_axpy(int64_t n, const S *x, S *y, cudaStream_t st) {
  if (n > 0) k_axpy<S><<<(int)std::min<int64_t>((n + 255) / 256, 2432), 256, 0, st>>>(n, x, y);
}

// register-only FMA chains; one store per thread
__global__ void k_fp64_probe(double *out, int iters) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-3 + k;
  for (int i = 0; i < iters; ++i)
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], 0.999, 1e-3);
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  out[(int64_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}
double measure_fp64_peak(int device) {
  int sm = 0;
  if (cudaSetDevice(device) != cudaSuccess || cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
    return -1.0;
  const int blocks = sm * 8, threads = 256, iters = 2048;
  double *out = nullptr;
  if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(double)) != cudaSuccess) return -1.0;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  k_fp64_probe<<<blocks, threads>>>(out, iters);
  cudaEventRecord(a);
  k_fp64_probe<<<blocks, threads>>>(out, iters);
  cudaEventRecord(b);
  cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess || ms <= 0.f) return -1.0;
  return 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
}

// MP2, setup_t_amplitudes (ccm_iter.f90:2355-2368): T = conj(V(ij,ab)) / (f_ii+f_jj-f_aa-f_bb)
template <typename S>
__global__ void k_mp2(DevLayout L, const S *__restrict__ Vhp, const S *__restrict__ fd, S *__restrict__ T) {
  const int2 tl = L.ttile[blockIdx.x];
  const int ch = tl.x, P = L.P[ch], H = L.H[ch];
  const int64_t n = (int64_t)P * H, end = min((int64_t)tl.y + kTileElems, n);
  for (int e = tl.y + threadIdx.x; e < end; e += blockDim.x) {
    const int ij = e / P, ab = e - ij * P;
    const int2 po = L.pp_orb[L.pp_off[ch] + ab], ho = L.hh_orb[L.hh_off[ch] + ij];
    const S den = ((S(0.0) - fd[po.x]) - fd[po.y] + fd[ho.x]) + fd[ho.y];
    const int64_t g = L.t_off[ch] + e;
    T[g] = (abs2(den) == 0.0) ? S(0.0) : conj_(Vhp[g]) / den;
  }
}
template <typename S> void launch_mp2(const DevLayout &L, const S *Vhp, const S *fdiag, S *T, cudaStream_t st) {
  if (L.nttile) k_mp2<S><<<L.nttile, 256, 0, st>>>(L, Vhp, fdiag, T);
}

// ordered (n_pp x n_hh) block <-> packed block
template <typename S>
__global__ void k_pack_t(DevLayout L, int ch, int n_pp, const double *__restrict__ stage, S *T, int *flag) {
  const int P = L.P[ch], H = L.H[ch];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)P * H; e += (int64_t)gridDim.x * blockDim.x) {
    const int ab = (int)(e % P), ij = (int)(e / P);
    const int64_t src = L.pp_row[L.pp_off[ch] + ab] + (int64_t)n_pp * L.hh_row[L.hh_off[ch] + ij];
    T[L.t_off[ch] + e] = cvt_in<S>(stage + 2 * src, flag);
  }
}
template <typename S> void launch_pack_t(const DevLayout &L, int ch, int n_pp, const double *stage, S *T, int *flag, cudaStream_t st) {
  k_pack_t<S><<<608, 256, 0, st>>>(L, ch, n_pp, stage, T, flag);
}
template <typename S>
__global__ void k_unpack_t(DevLayout L, int ch, int n_pp, const int *__restrict__ pp_signed, const int *__restrict__ hh_signed,
                            int n_hh, const S *__restrict__ T, double *stage) {
  const int P = L.P[ch];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)n_pp * n_hh; e += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(e % n_pp), c = (int)(e / n_pp);
    const int sp = pp_signed[r], sh = hh_signed[c];
    S v = S(0.0);
    if (sp && sh) v = (ssign(sp) * ssign(sh)) * T[L.t_off[ch] + sidx(sp) + (int64_t)P * sidx(sh)];
    stage[2 * e] = real_(v);
    stage[2 * e + 1] = imag_(v);
  }
}
template <typename S>
void launch_unpack_t(const DevLayout &L, int ch, int n_pp, const int *pp_signed, const int *hh_signed, int n_hh, const S *T,
                     double *stage, cudaStream_t st) {
  k_unpack_t<S><<<608, 256, 0, st>>>(L, ch, n_pp, pp_signed, hh_signed, n_hh, T, stage);
}

// ---- explicit instantiations -------------------------------------------------
#define CCX_INST(S)                                                                                                    \
  template void launch_gemm<S>(int, const GemmProb<S> *, const GemmTile *, int, cudaStream_t);                         \
  template void launch_splitk_reduce<S>(const GemmProb<S> *, const int *, int, cudaStream_t);                          \
  template void launch_gather_tph<S>(const DevLayout &, const S *, S *, cudaStream_t);                                 \
  template void launch_i7<S>(const DevLayout &, const S *, const S *, const S *, S *, S *, cudaStream_t);             \
  template void launch_i7_direct<S>(const DevLayout &, const S *, const S *, S *, const S *, const S *, S *, S *,      \
                                    cudaStream_t);                                                                  \
  template void launch_i9b<S>(int64_t, const S *, const S *, const S *, S *, cudaStream_t);                         \
  template void launch_i9<S>(const DevLayout &, int64_t, const S *, const S *, S *, cudaStream_t);                     \
  template void launch_xdot<S>(const DevLayout &, const int4 *, int, const int4 *, int, const S *, const S *, S *, S *, \
                              cudaStream_t);        \
  template void launch_i6<S>(const DevLayout &, const int2 *, int, S *, const S *, const S *, const S *, const S *,   \
                             S *, S *, cudaStream_t);                                                                  \
  template void launch_rinit<S>(const DevLayout &, const int4 *, const int4 *, const S *, const S *, const S *,      \
                               const S *, const S *, const S *, S *, S *, cudaStream_t);                                                         \
  template void launch_update<S>(const DevLayout &, int, S *, const S *, const S *, const S *, const S *, S *,         \
                                 typename StepOf<S>::type *,                                                            \
                                 double *, double *, cudaStream_t);                                                    \
  template void launch_dots<S>(int64_t, const S *, const S *const *, int, int, double *, double *, cudaStream_t);     \
  template void launch_update_std<S>(const DevLayout &, const S *, const S *, const S *, const S *, const S *, S *,    \
                                     typename StepOf<S>::type *, const typename StepOf<S>::type *const *, int, int,   \
                                     const int *, double *, double *, cudaStream_t);                                   \
  template void launch_diis_gram<S>(int64_t, const S *const *, int, double *, double *, cudaStream_t);                \
  template void launch_combine<S>(int64_t, const S *const *, const double *, int, S *, cudaStream_t);                 \
  template void launch_pack_vblock<S>(const DevLayout &, int, int, int, const double *, S *, int *, cudaStream_t);    \
  template void launch_pack_vblock_host<S>(const DevLayout &, int, int, int, int, int, const double *, S *, int *,      \
                                           cudaStream_t);                                                              \
  template void launch_build_w<S>(const DevLayout &, const int2 *, const int64_t *, const int *, const double *, S *,  \
                                  int *, cudaStream_t);                                                                \
  template void launch_build_vph<S>(const DevLayout &, const S *, S *, cudaStream_t);                                 \
  template void launch_generate<S>(const DevLayout &, const DevOrbits &, const DevPotential &, S *, S *, S *, S *,    \
                                   S *, S *, S *, double *, double *, int, int, cudaStream_t);                                             \
  template void launch_mp2<S>(const DevLayout &, const S *, const S *, S *, cudaStream_t);                            \
  template void launch_pack_t<S>(const DevLayout &, int, int, const double *, S *, int *, cudaStream_t);          \
  template void launch_axpy<S>(int64_t, const S *, S *, cudaStream_t);                                                 \
  template void launch_gen_ordered<S>(const DevOrbits &, const DevPotential &, const int2 *, const int2 *, int, int,  \
                                      int, double *, cudaStream_t);                                                    \
  template void launch_unpack_vblock<S>(const DevLayout &, int, int, int, int, const int *, const int *, const S *,  \
                                        double *, cudaStream_t);                                                       \
  template void launch_unpack_t<S>(const DevLayout &, int, int, const int *, const int *, int, const S *, double *,   \
                                   cudaStream_t);

CCX_INST(double)
CCX_INST(cplx)

}  // namespace ccx
