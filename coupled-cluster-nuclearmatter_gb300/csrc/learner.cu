// Learned warm start (see learner.hpp): feature extraction, FP32 training kernels
// (strided SIMT GEMM with fused bias/SiLU epilogues, split-K weight gradients reduced in a
// fixed order, Adam) and the fused BF16 tensor-core inference kernel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "common.cuh"
#include "engine.hpp"
#include "learner.hpp"
#include "tc_ptx.cuh"

namespace ccx {

namespace {

using namespace tcptx;

void lck(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw EngineError(2, std::string(what) + ": " + cudaGetErrorString(e));
}

struct LBuf {
  void *p = nullptr;
  size_t bytes = 0;
  LBuf() = default;
  LBuf(const LBuf &) = delete;
  LBuf &operator=(const LBuf &) = delete;
  LBuf(LBuf &&o) noexcept : p(o.p), bytes(o.bytes) { o.p = nullptr; o.bytes = 0; }
  ~LBuf() { if (p) cudaFree(p); }
  void alloc(size_t b) {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = std::max<size_t>(b, 16);
    lck(cudaMalloc(&p, bytes), "cudaMalloc (learner)");
  }
  template <typename T> T *as() const { return (T *)p; }
};

// ---------------------------------------------------------------- features
constexpr float kMlPriorUnit = 100.0f;  // the prior feature in units of 0.01, a typical correction
struct MLCtx {
  DevLayout L;
  DevOrbits O;
  const double *fd, *V;
  const float *prior;  // per packed amplitude, or null
  float rho, kF, eF, vol, th[3];
};

__device__ __forceinline__ float norm3(float x, float y, float z) { return sqrtf(x * x + y * y + z * z); }

// Features of packed amplitude e of hhpp channel ch (a<b particles, i<j holes), and
// its MP2 value V/D in FP64.  Momenta in units of kF and energies in units of eF make
// the features comparable across densities.
__device__ void ml_feat(const MLCtx &c, int ch, int e, float (&f)[kMlIn], double &tmp2) {
  const int P = c.L.P[ch];
  const int ij = e / P, ab = e - ij * P;
  const int2 po = c.L.pp_orb[c.L.pp_off[ch] + ab], ho = c.L.hh_orb[c.L.hh_off[ch] + ij];
  const int a = po.x, b = po.y, i = ho.x, j = ho.y;
  const double D = ((0.0 - c.fd[a]) - c.fd[b] + c.fd[i]) + c.fd[j];
  const double v = c.V[c.L.t_off[ch] + e];
  tmp2 = D == 0.0 ? 0.0 : v / D;
  const float ik = 1.0f / c.kF;
  const float ax = (float)c.O.kx[a] * ik, ay = (float)c.O.ky[a] * ik, az = (float)c.O.kz[a] * ik;
  const float bx = (float)c.O.kx[b] * ik, by = (float)c.O.ky[b] * ik, bz = (float)c.O.kz[b] * ik;
  const float ix = (float)c.O.kx[i] * ik, iy = (float)c.O.ky[i] * ik, iz = (float)c.O.kz[i] * ik;
  const float jx = (float)c.O.kx[j] * ik, jy = (float)c.O.ky[j] * ik, jz = (float)c.O.kz[j] * ik;
  f[0] = (c.rho - 0.12f) / 0.08f;
  f[1] = c.th[0];
  f[2] = c.th[1];
  f[3] = c.th[2];
  f[4] = (float)D / c.eF;
  f[5] = (float)v * c.vol / 500.0f;
  f[6] = (float)tmp2 * c.vol / 10.0f;
  f[7] = norm3(ax - ix, ay - iy, az - iz);
  f[8] = norm3(ax - jx, ay - jy, az - jz);
  f[9] = norm3(ax + bx, ay + by, az + bz);
  f[10] = (ax * ax + ay * ay + az * az) + (bx * bx + by * by + bz * bz) - 2.0f;
  f[11] = (ix * ix + iy * iy + iz * iz) + (jx * jx + jy * jy + jz * jz);
  f[12] = (float)(c.O.sz[a] * c.O.sz[b]);
  f[13] = (float)(c.O.sz[a] * c.O.sz[i]);
  f[14] = (float)(c.O.tz[a] * c.O.tz[b]);
  f[15] = (float)(c.O.tz[a] * c.O.tz[i]);
  // the prior: the correction interpolated from neighbouring converged solutions
  f[16] = c.prior ? c.prior[c.L.t_off[ch] + e] * kMlPriorUnit : 0.0f;
  f[17] = c.prior ? 1.0f : 0.0f;
}

// Target: the correction of the amplitude numerator, y = (T - T_MP2) D vol / kMlNum, with
// D the bare denominator.  The residual weights an amplitude error by D, so a uniform
// error in y is a uniform error in the residual of the start.
constexpr double kMlNum = 1000.0;  // MeV fm^3

// training samples of a converged solution, every stride-th packed amplitude g:
// X[g / stride] features, y[g / stride] the numerator correction
__global__ void k_ml_extract(MLCtx c, const double *__restrict__ T, int stride, float *__restrict__ X,
                             float *__restrict__ y) {
  const int2 tl = c.L.ttile[blockIdx.x];
  const int ch = tl.x;
  const int n = c.L.P[ch] * c.L.H[ch];
  const int end = min(tl.y + kTileElems, n);
  for (int e = tl.y + threadIdx.x; e < end; e += blockDim.x) {
    const int64_t g = c.L.t_off[ch] + e;
    if (g % stride) continue;
    float f[kMlIn];
    double tmp2;
    ml_feat(c, ch, e, f, tmp2);
    const int64_t o = g / stride;
#pragma unroll
    for (int q = 0; q < kMlIn; ++q) X[o * kMlIn + q] = f[q];
    const double D = (double)f[4] * (double)c.eF;
    // with a prior the network learns what the prior leaves over (a skip connection):
    // the BF16 inference then perturbs only that small remainder
    y[o] = (float)((T[g] - tmp2) * D * (double)c.vol / kMlNum) - (c.prior ? c.prior[g] : 0.0f);
  }
}
// A solution the prior is taken from (another density of the same lattice and twist)
struct PriorSrc {
  DevLayout L;
  const double *fd, *V, *T;
  const int *oof;
  double vol;
};
// prior += w * (the numerator correction of src's T), per packed amplitude g of the target
// layout Lt: the target's orbitals a, b, i, j are mapped to src's by quantum numbers
// (okey of the target, oof of src), and src's packed amplitude is read with the product of
// its two pair-slot signs.  The correction (T - V/D) D vol / 1000 is src's own, which
// makes it comparable across densities.
__global__ void k_ml_prior(DevLayout Lt, const int *__restrict__ okey, PriorSrc src, float w, int first,
                           float *__restrict__ prior) {
  const int2 tl = Lt.ttile[blockIdx.x];
  const int ch = tl.x;
  const int P = Lt.P[ch];
  const int end = min(tl.y + kTileElems, P * Lt.H[ch]);
  const DevLayout &L = src.L;
  for (int e = tl.y + threadIdx.x; e < end; e += blockDim.x) {
    const int ij = e / P, ab = e - ij * P;
    const int2 po = Lt.pp_orb[Lt.pp_off[ch] + ab], ho = Lt.hh_orb[Lt.hh_off[ch] + ij];
    const int a = src.oof[okey[po.x]], b = src.oof[okey[po.y]];
    const int i = src.oof[okey[ho.x]], j = src.oof[okey[ho.y]];
    float y = 0.0f;
    if (a >= L.A && b >= L.A && i >= 0 && i < L.A && j >= 0 && j < L.A) {
      const int2 sab = L.pp_slot[(int64_t)(a - L.A) * L.NP + (b - L.A)];
      const int2 sij = L.hh_slot[i * L.A + j];
      if (sab.y != 0 && sij.y != 0 && sab.x == sij.x) {
        const int64_t gs = L.t_off[sab.x] + sidx(sab.y) + (int64_t)L.P[sab.x] * sidx(sij.y);
        const double sg = ssign(sab.y) * ssign(sij.y);
        const double D = ((0.0 - src.fd[a]) - src.fd[b] + src.fd[i]) + src.fd[j];
        if (D != 0.0) y = (float)(sg * (src.T[gs] - src.V[gs] / D) * D * src.vol / kMlNum);
      }
    }
    const int64_t g = Lt.t_off[ch] + e;
    prior[g] = first ? w * y : fmaf(w, y, prior[g]);
  }
}

__global__ void k_ml_gather(const float *__restrict__ Xs, const float *__restrict__ ys, const int64_t *__restrict__ perm,
                            int64_t n, float *__restrict__ X, float *__restrict__ y) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = perm[r];
#pragma unroll
    for (int q = 0; q < kMlIn; ++q) X[r * kMlIn + q] = Xs[s * kMlIn + q];
    y[r] = ys[s];
  }
}

// ---------------------------------------------------------------- FP32 training
__device__ __forceinline__ float sigm(float z) { return 1.0f / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sigm(z); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = sigm(z);
  return s * (1.0f + z * (1.0f - s));
}

// C(m,n) = sum_k A(m,k) B(k,n) over strided operands, 64 x 64 tiles, 4 x 4 per thread,
// K split over blockIdx.z in chunks of kchunk (partials at C + z * M * N, dense).
// mode 0: C (+ bias[n]); 1: C = Z + bias[n] and H = silu(Z); 2: C *= silu'(Zp(m,n)).
struct SgArgs {
  const float *A, *B;
  int64_t sAm, sAk, sBk, sBn;
  int M, N, K;
  float *C;
  int64_t sCm, sCn;
  const float *bias;
  float *H;
  const float *Zp;
  int mode, kchunk;
};

__global__ void __launch_bounds__(256) k_sgemm(SgArgs g) {
  constexpr int BM = 64, BN = 64, BK = 16;
  __shared__ float As[BK][BM + 1];
  __shared__ float Bs[BK][BN + 1];
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int tid = threadIdx.x, tm = tid % 16, tn = tid / 16;
  int kb = 0, ke = g.K;
  if (g.kchunk > 0) {
    kb = blockIdx.z * g.kchunk;
    ke = min(g.K, kb + g.kchunk);
  }
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;
  for (int k0 = kb; k0 < ke; k0 += BK) {
    for (int x = tid; x < BM * BK; x += 256) {
      const int m = x % BM, k = x / BM;
      const int gm = m0 + m, gk = k0 + k;
      As[k][m] = (gm < g.M && gk < ke) ? g.A[(int64_t)gm * g.sAm + (int64_t)gk * g.sAk] : 0.0f;
    }
    for (int x = tid; x < BK * BN; x += 256) {
      const int n = x % BN, k = x / BN;
      const int gn = n0 + n, gk = k0 + k;
      Bs[k][n] = (gn < g.N && gk < ke) ? g.B[(int64_t)gk * g.sBk + (int64_t)gn * g.sBn] : 0.0f;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[k][tm * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[k][tn * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  float *C = g.C + (g.kchunk > 0 ? (int64_t)blockIdx.z * g.M * g.N : 0);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + tm * 4 + i;
    if (m >= g.M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tn * 4 + j;
      if (n >= g.N) continue;
      const int64_t o = (int64_t)m * g.sCm + (int64_t)n * g.sCn;
      float v = acc[i][j];
      if (g.bias) v += g.bias[n];
      if (g.mode == 1) {
        C[o] = v;
        g.H[o] = silu(v);
      } else if (g.mode == 2) {
        C[o] = v * dsilu(g.Zp[o]);
      } else {
        C[o] = v;
      }
    }
  }
}

// out[i] = sum_z part[z * len + i], fixed order
__global__ void k_ml_reduce(const float *__restrict__ part, int nz, int len, float *__restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < len; i += gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int z = 0; z < nz; ++z) s += part[(int64_t)z * len + i];
    out[i] = s;
  }
}

// dout = 2 (out - y) / n; loss partials per block
__global__ void k_ml_dloss(const float *__restrict__ out, const float *__restrict__ y, int n, float *__restrict__ dout,
                           double *__restrict__ part) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float d = out[i] - y[i];
    dout[i] = 2.0f * d / (float)n;
    s += (double)d * d;
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}
__global__ void k_ml_loss_finish(const double *__restrict__ part, int nb, int n, double *__restrict__ loss) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < nb; ++i) s += part[i];
    *loss = s / n;
  }
}

__global__ void k_ml_adam(float *__restrict__ p, float *__restrict__ m, float *__restrict__ v, const float *__restrict__ g,
                          int n, float lr, float b1t, float b2t) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / (1.0f - b1t)) / (sqrtf(vi / (1.0f - b2t)) + eps);
  }
}

__global__ void k_ml_scale(float *__restrict__ x, int64_t n, float s) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] *= s;
}
__global__ void k_ml_fill(float *__restrict__ x, int64_t n, float v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] = v;
}

// ---------------------------------------------------------------- BF16 tensor-core inference
// One persistent CTA of 128 threads per SM, one sample per thread and TMEM lane.  The
// three hidden layers are 128 x 128 x K tcgen05 MMAs with BF16 operands in shared
// memory (weights loaded once per CTA) and the FP32 accumulator in tensor memory; each
// thread turns its accumulator row into the next layer's BF16 operand row (bias, SiLU),
// and the 128 -> 1 output layer is a per-thread FP32 dot product.
constexpr uint32_t kWTile = 128u * 128u;           // one 128-row x 64-BF16 K tile
constexpr uint32_t kWBytes = 5u * kWTile;          // W1 (1 K tile), W2, W3 (2 each)
constexpr uint32_t kFeatOff = kWBytes;             // features: 1 K tile
constexpr uint32_t kActOff = kFeatOff + kWTile;    // activations: 2 K tiles
constexpr uint32_t kParOff = kActOff + 2 * kWTile; // b1, b2, b3, w4 (FP32) and b4
constexpr uint32_t kBarOff2 = kParOff + (4 * kMlW + 4) * 4;
constexpr size_t kInferSmem = kBarOff2 + 32;

struct InferArgs {
  MLCtx c;
  int use_view;
  double *T;                // view: T' written here
  const float *X;           // external features (n x 16)
  float *out;               // external outputs
  int n;
  const uint8_t *wt;        // BF16 weight tiles (kWBytes)
  const float *par;         // FP32 parameter vector
  int ntiles;
  int *err;
};

__device__ __forceinline__ uint32_t bf16_bits(float x) {
  // round to nearest even on the bit pattern (finite inputs)
  const uint32_t u = __float_as_uint(x);
  return (u + 0x7FFFu + ((u >> 16) & 1u)) >> 16;
}
// byte offset of element (row, k) inside a canonical no-swizzle K-major tile set
__device__ __forceinline__ uint32_t cm_off(int row, int k) {
  return (uint32_t)(k >> 6) * kWTile + (uint32_t)((((row >> 3) << 3) + ((k & 63) >> 3)) << 7) + (uint32_t)((row & 7) << 4) +
         (uint32_t)((k & 7) << 1);
}

__global__ void __launch_bounds__(128, 1) k_ml_infer(InferArgs g) {
  extern __shared__ __align__(1024) uint8_t smem[];
  const int tid = threadIdx.x, warp = tid >> 5;
  uint64_t *bar = (uint64_t *)(smem + kBarOff2);
  uint64_t *wbar = bar + 1;
  uint32_t *tslot = (uint32_t *)(bar + 2);
  volatile int *abort_flag = (volatile int *)(tslot + 1);
  float *sp = (float *)(smem + kParOff);
  if (warp == 0) {
    tmem_alloc(smem_u32(tslot), 128);
    tmem_relinquish();
  }
  if (tid == 0) {
    mbar_init(smem_u32(bar), 1);
    mbar_init(smem_u32(wbar), 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // biases and output weights; zero feature padding (K columns 32..63 are never rewritten)
  for (int x = tid; x < kMlW; x += 128) {
    sp[x] = g.par[kMlOffB1 + x];
    sp[kMlW + x] = g.par[kMlOffB2 + x];
    sp[2 * kMlW + x] = g.par[kMlOffB3 + x];
    sp[3 * kMlW + x] = g.par[kMlOffW4 + x];
  }
  if (tid == 0) sp[4 * kMlW] = g.par[kMlOffB4];
  for (int x = tid; x < (int)(kWTile / 16); x += 128) ((uint4 *)(smem + kFeatOff))[x] = make_uint4(0, 0, 0, 0);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  if (tid == 0) {
    mbar_expect_tx(smem_u32(wbar), kWBytes);
    bulk_g2s(smem_u32(smem), g.wt, kWBytes, smem_u32(wbar));
  }
  bool ok = mbar_wait(smem_u32(wbar), 0);
  if (!ok) *abort_flag = 1;
  __syncthreads();
  const uint32_t idesc16 = instr_desc<kTcBF16>(128, 128);
  const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
  uint32_t phase = 0;
  for (int t = blockIdx.x; t < g.ntiles && !*abort_flag; t += gridDim.x) {
    // ---- features of this thread's sample
    bool live = false;
    int ch = 0;
    int64_t gidx = 0;
    double tmp2 = 0.0;
    float f[kMlIn];
    if (g.use_view) {
      const int2 tt = g.c.L.ttile[t >> 3];
      ch = tt.x;
      const int e = tt.y + (t & 7) * 128 + tid;
      const int n = g.c.L.P[ch] * g.c.L.H[ch];
      live = e < min(tt.y + kTileElems, n);
      if (live) {
        ml_feat(g.c, ch, e, f, tmp2);
        gidx = g.c.L.t_off[ch] + e;
      }
    } else {
      const int r = t * 128 + tid;
      live = r < g.n;
      if (live)
        for (int q = 0; q < kMlIn; ++q) f[q] = g.X[(int64_t)r * kMlIn + q];
    }
    if (!live)
      for (int q = 0; q < kMlIn; ++q) f[q] = 0.0f;
    {  // features into K columns 0 .. kMlIn - 1 of the tile, zeros up to column 31
      uint32_t w[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const float lo = 2 * q < kMlIn ? f[2 * q] : 0.0f, hi = 2 * q + 1 < kMlIn ? f[2 * q + 1] : 0.0f;
        w[q] = bf16_bits(lo) | (bf16_bits(hi) << 16);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q)
        *(uint4 *)(smem + kFeatOff + cm_off(tid, 8 * q)) = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
    }
    float o = 0.0f;
    for (int layer = 0; layer < 3; ++layer) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      tc_fence_before();
      __syncthreads();
      if (tid == 0) {
        tc_fence_after();
        if (layer == 0) {  // K = 32: the features and their zero padding
#pragma unroll
          for (int ks = 0; ks < 2; ++ks)
            tc_mma<kTcBF16>(tmem, smem_desc(smem_u32(smem + kFeatOff) + ks * 256), smem_desc(smem_u32(smem) + ks * 256),
                            idesc16, ks ? 1u : 0u);
        } else {
          const uint32_t wb = smem_u32(smem + (layer == 1 ? kWTile : 3 * kWTile));
#pragma unroll
          for (int kt = 0; kt < 2; ++kt)
#pragma unroll
            for (int ks = 0; ks < 4; ++ks)
              tc_mma<kTcBF16>(tmem, smem_desc(smem_u32(smem + kActOff) + kt * kWTile + ks * 256),
                              smem_desc(wb + kt * kWTile + ks * 256), idesc16, (kt | ks) ? 1u : 0u);
        }
        tc_commit(smem_u32(bar));
      }
      const bool got = __all_sync(0xffffffffu, mbar_wait(smem_u32(bar), phase & 1u));
      ++phase;
      if (!got) {
        *abort_flag = 1;
        break;
      }
      tc_fence_after();
      const float *bias = sp + layer * kMlW;
      for (int c0 = 0; c0 < kMlW; c0 += 32) {
        uint32_t r[32];
        tmem_ld32(lane_base + (uint32_t)c0, r);
        tmem_ld_wait();
        if (layer < 2) {
#pragma unroll
          for (int q = 0; q < 32; q += 8) {
            uint32_t w[4];
#pragma unroll
            for (int h = 0; h < 4; ++h) {
              const float z0 = __uint_as_float(r[q + 2 * h]) + bias[c0 + q + 2 * h];
              const float z1 = __uint_as_float(r[q + 2 * h + 1]) + bias[c0 + q + 2 * h + 1];
              w[h] = bf16_bits(silu(z0)) | (bf16_bits(silu(z1)) << 16);
            }
            *(uint4 *)(smem + kActOff + cm_off(tid, c0 + q)) = make_uint4(w[0], w[1], w[2], w[3]);
          }
        } else {
#pragma unroll
          for (int q = 0; q < 32; ++q) o = fmaf(silu(__uint_as_float(r[q]) + bias[c0 + q]), sp[3 * kMlW + c0 + q], o);
        }
      }
    }
    if (*abort_flag) break;
    o += sp[4 * kMlW];
    if (live) {
      if (g.use_view) {
        if (g.c.prior) o += g.c.prior[gidx];  // the skip connection of the prior, in FP32
        const double D = (double)f[4] * (double)g.c.eF;
        g.T[gidx] = D == 0.0 ? tmp2 : tmp2 + (double)o * kMlNum / (D * (double)g.c.vol);
      }
      else g.out[t * 128 + tid] = o;
    }
  }
  if (*abort_flag && tid == 0) atomicExch(g.err, 1);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 128);
  }
}

// ---------------------------------------------------------------- host side
uint16_t host_bf16(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return (uint16_t)((u + 0x7FFFu + ((u >> 16) & 1u)) >> 16);
}
size_t host_cm_off(int row, int k) {
  return (size_t)(k >> 6) * kWTile + (size_t)((((row >> 3) << 3) + ((k & 63) >> 3)) << 7) + (size_t)((row & 7) << 4) +
         (size_t)((k & 7) << 1);
}

MLCtx make_ctx(const MLView &v) {
  MLCtx c{};
  c.L = v.L;
  c.O = v.O;
  c.fd = v.fdiag;
  c.V = v.Vhp;
  c.rho = (float)v.rho;
  c.kF = (float)v.kF;
  c.eF = (float)v.eF;
  c.vol = (float)v.vol;
  for (int q = 0; q < 3; ++q) c.th[q] = (float)(v.theta[q] / 3.14159265358979323846);
  return c;
}

class Learner final : public ILearner {
 public:
  Learner(int device, uint64_t seed) : device_(device) {
    lck(cudaSetDevice(device), "cudaSetDevice");
    lck(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking), "cudaStreamCreate");
    params_.alloc(kMlParams * 4);
    m_.alloc(kMlParams * 4);
    v_.alloc(kMlParams * 4);
    grad_.alloc(kMlParams * 4);
    wt_.alloc(kWBytes);
    err_.alloc(4);
    lck(cudaMemset(err_.p, 0, 4), "memset");
    // Kaiming-uniform initial weights from splitmix64, zero biases, small output layer
    std::vector<float> p(kMlParams, 0.0f);
    uint64_t s = seed;
    auto uni = [&]() {
      uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
      z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
      z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
      z ^= z >> 31;
      return (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
    };
    auto fill = [&](int off, int n, int fan_in, double gain) {
      const double a = gain * std::sqrt(6.0 / fan_in);
      for (int i = 0; i < n; ++i) p[off + i] = (float)(a * uni());
    };
    fill(kMlOffW1, kMlW * kMlIn, kMlIn, 1.0);
    fill(kMlOffW2, kMlW * kMlW, kMlW, 1.0);
    fill(kMlOffW3, kMlW * kMlW, kMlW, 1.0);
    fill(kMlOffW4, kMlW, kMlW, 0.1);
    set_params(p.data());
    folded_ = false;  // the initial output layer is in the standardised units of training
  }
  ~Learner() override {
    if (st_) cudaStreamDestroy(st_);
  }

  void add_solution(const MLView &v, int stride) override {
    lck(cudaSetDevice(device_), "cudaSetDevice");
    if (stride < 1) throw EngineError(1, "learner: sample stride must be >= 1");
    Chunk c;
    c.n = (v.n_t + stride - 1) / stride;
    c.X.alloc((size_t)c.n * kMlIn * 4);
    c.y.alloc((size_t)c.n * 4);
    const MLCtx ctx = ctx_of(v);
    if (v.L.nttile) k_ml_extract<<<v.L.nttile, 256, 0, v.st>>>(ctx, v.T, stride, c.X.as<float>(), c.y.as<float>());
    lck(cudaGetLastError(), "feature extraction");
    lck(cudaStreamSynchronize(v.st), "feature extraction");
    data_.push_back(std::move(c));
  }
  void set_prior(const MLView &target, const MLView *views, const double *w, int n) override {
    lck(cudaSetDevice(device_), "cudaSetDevice");
    has_prior_ = false;
    if (n <= 0) return;
    const int64_t nt = target.n_t;
    for (int i = 0; i < n; ++i)
      if (views[i].nkeys != target.nkeys || views[i].L.ns != target.L.ns || views[i].L.A != target.L.A)
        throw EngineError(1, "learner: the prior's engines are not the target's lattice at another density");
    if (prior_.bytes < (size_t)std::max<int64_t>(nt, 1) * 4) prior_.alloc((size_t)std::max<int64_t>(nt, 1) * 4);
    lck(cudaStreamSynchronize(target.st), "prior");
    for (int i = 0; i < n; ++i) {
      const MLView &v = views[i];
      lck(cudaStreamSynchronize(v.st), "prior");  // the source's amplitudes are final
      const PriorSrc src{v.L, v.fdiag, v.Vhp, v.T, v.oof, v.vol};
      if (target.L.nttile)
        k_ml_prior<<<target.L.nttile, 256, 0, target.st>>>(target.L, target.okey, src, (float)w[i], i == 0,
                                                            prior_.as<float>());
      lck(cudaGetLastError(), "prior");
    }
    lck(cudaStreamSynchronize(target.st), "prior");
    prior_n_ = nt;
    has_prior_ = true;
  }
  void clear() override { data_.clear(); }
  int64_t samples() const override {
    int64_t n = 0;
    for (const auto &c : data_) n += c.n;
    return n;
  }

  double train(int steps, int batch, double lr, uint64_t seed) override {
    lck(cudaSetDevice(device_), "cudaSetDevice");
    const int64_t N = samples();
    if (N < 1) throw EngineError(4, "learner: no training samples");
    if (batch < 1 || steps < 1) throw EngineError(1, "learner: steps and batch must be positive");
    batch = (int)std::min<int64_t>(batch, N);
    // one concatenated copy, shuffled once per pass with a host permutation
    LBuf Xa, ya, Xs, ys, perm;
    Xa.alloc((size_t)N * kMlIn * 4);
    ya.alloc((size_t)N * 4);
    int64_t o = 0;
    for (const auto &c : data_) {
      lck(cudaMemcpyAsync(Xa.as<float>() + o * kMlIn, c.X.p, (size_t)c.n * kMlIn * 4, cudaMemcpyDeviceToDevice, st_), "copy");
      lck(cudaMemcpyAsync(ya.as<float>() + o, c.y.p, (size_t)c.n * 4, cudaMemcpyDeviceToDevice, st_), "copy");
      o += c.n;
    }
    // The network trains on targets divided by their RMS (fixed at the first training)
    // and the output layer is scaled back afterwards, so that the loss is relative to the
    // size of what is learned (with a prior, a small remainder)
    if (yscale_ <= 0.0f) {
      std::vector<float> yh(N);
      lck(cudaMemcpyAsync(yh.data(), ya.p, (size_t)N * 4, cudaMemcpyDeviceToHost, st_), "targets");
      lck(cudaStreamSynchronize(st_), "targets");
      double ss = 0.0;
      for (float v : yh) ss += (double)v * v;
      yscale_ = (float)std::max(std::sqrt(ss / (double)N), 1e-12);
    }
    k_ml_scale<<<1216, 256, 0, st_>>>(ya.as<float>(), N, 1.0f / yscale_);
    if (folded_) k_ml_scale<<<1, 256, 0, st_>>>(params_.as<float>() + kMlOffW4, kMlW + 1, 1.0f / yscale_);
    Xs.alloc((size_t)N * kMlIn * 4);
    ys.alloc((size_t)N * 4);
    perm.alloc((size_t)N * 8);
    std::vector<int64_t> pv(N);
    std::mt19937_64 rng(seed);
    const int64_t passes_steps = std::max<int64_t>(1, N / batch);
    std::vector<double> losses(steps);
    LBuf lossd;
    lossd.alloc((size_t)steps * 8);
    ensure_batch(batch);
    for (int s = 0; s < steps; ++s) {
      if (s % passes_steps == 0) {
        for (int64_t i = 0; i < N; ++i) pv[i] = i;
        std::shuffle(pv.begin(), pv.end(), rng);
        lck(cudaMemcpyAsync(perm.p, pv.data(), (size_t)N * 8, cudaMemcpyHostToDevice, st_), "perm");
        k_ml_gather<<<1216, 256, 0, st_>>>(Xa.as<float>(), ya.as<float>(), perm.as<int64_t>(), N, Xs.as<float>(),
                                           ys.as<float>());
        lck(cudaStreamSynchronize(st_), "shuffle");
      }
      const int64_t off = (int64_t)(s % passes_steps) * batch;
      forward_backward(Xs.as<float>() + off * kMlIn, ys.as<float>() + off, batch, lossd.as<double>() + s);
      ++t_;
      const float b1t = (float)std::pow(0.9, (double)t_), b2t = (float)std::pow(0.999, (double)t_);
      k_ml_adam<<<(kMlParams + 255) / 256, 256, 0, st_>>>(params_.as<float>(), m_.as<float>(), v_.as<float>(),
                                                           grad_.as<float>(), kMlParams, (float)lr, b1t, b2t);
    }
    // the output layer back in the targets' units (the Adam moments stay with the
    // standardised units of the next training)
    k_ml_scale<<<1, 256, 0, st_>>>(params_.as<float>() + kMlOffW4, kMlW + 1, yscale_);
    folded_ = true;
    lck(cudaGetLastError(), "training");
    lck(cudaMemcpyAsync(losses.data(), lossd.p, (size_t)steps * 8, cudaMemcpyDeviceToHost, st_), "loss");
    lck(cudaStreamSynchronize(st_), "training");
    double tail = 0.0;
    const int k0 = std::max(0, steps - 10);
    for (int s = k0; s < steps; ++s) tail += losses[s];
    weights_dirty_ = true;
    return tail / (steps - k0) * (double)yscale_ * (double)yscale_;
  }

  void warm_start(const MLView &v) override {
    lck(cudaSetDevice(device_), "cudaSetDevice");
    upload_weight_tiles();
    InferArgs a{};
    a.c = ctx_of(v);
    a.use_view = 1;
    a.T = v.T;
    a.wt = wt_.as<uint8_t>();
    a.par = params_.as<float>();
    a.ntiles = v.L.nttile * 8;
    a.err = err_.as<int>();
    run_infer(a, v.st);
  }

  void get_params(float *p) const override {
    lck(cudaMemcpy(p, params_.p, kMlParams * 4, cudaMemcpyDeviceToHost), "params");
  }
  void set_params(const float *p) override {
    lck(cudaMemcpy(params_.p, p, kMlParams * 4, cudaMemcpyHostToDevice), "params");
    folded_ = true;  // parameters from get_params: output layer in the targets' units
    lck(cudaMemset(m_.p, 0, kMlParams * 4), "adam");
    lck(cudaMemset(v_.p, 0, kMlParams * 4), "adam");
    t_ = 0;
    weights_dirty_ = true;
  }

  void loss_grad(const float *X, const float *y, int n, double *loss, float *grad) override {
    lck(cudaSetDevice(device_), "cudaSetDevice");
    if (n < 1) throw EngineError(1, "learner: empty batch");
    LBuf dX, dy, dl;
    dX.alloc((size_t)n * kMlIn * 4);
    dy.alloc((size_t)n * 4);
    dl.alloc(8);
    lck(cudaMemcpy(dX.p, X, (size_t)n * kMlIn * 4, cudaMemcpyHostToDevice), "copy");
    lck(cudaMemcpy(dy.p, y, (size_t)n * 4, cudaMemcpyHostToDevice), "copy");
    ensure_batch(n);
    forward_backward(dX.as<float>(), dy.as<float>(), n, dl.as<double>());
    lck(cudaStreamSynchronize(st_), "loss_grad");
    lck(cudaMemcpy(loss, dl.p, 8, cudaMemcpyDeviceToHost), "copy");
    lck(cudaMemcpy(grad, grad_.p, kMlParams * 4, cudaMemcpyDeviceToHost), "copy");
  }

  void infer(const float *X, int n, float *out, int tensor_cores) override {
    lck(cudaSetDevice(device_), "cudaSetDevice");
    if (n < 1) return;
    LBuf dX, dout;
    dX.alloc((size_t)n * kMlIn * 4);
    dout.alloc((size_t)n * 4);
    lck(cudaMemcpy(dX.p, X, (size_t)n * kMlIn * 4, cudaMemcpyHostToDevice), "copy");
    if (tensor_cores) {
      upload_weight_tiles();
      InferArgs a{};
      a.use_view = 0;
      a.X = dX.as<float>();
      a.out = dout.as<float>();
      a.n = n;
      a.wt = wt_.as<uint8_t>();
      a.par = params_.as<float>();
      a.ntiles = (n + 127) / 128;
      a.err = err_.as<int>();
      run_infer(a, st_);
    } else {
      ensure_batch(n);
      forward(dX.as<float>(), n);
      lck(cudaMemcpyAsync(dout.p, out_.p, (size_t)n * 4, cudaMemcpyDeviceToDevice, st_), "copy");
    }
    lck(cudaStreamSynchronize(st_), "infer");
    lck(cudaMemcpy(out, dout.p, (size_t)n * 4, cudaMemcpyDeviceToHost), "copy");
  }

 private:
  struct Chunk {
    LBuf X, y;
    int64_t n = 0;
  };

  // the feature context of a view, with the prior when one is set
  MLCtx ctx_of(const MLView &v) const {
    MLCtx c = make_ctx(v);
    if (has_prior_) {
      if (v.n_t != prior_n_) throw EngineError(1, "learner: the prior was set for another layout");
      c.prior = prior_.as<float>();
    }
    return c;
  }

  void ensure_batch(int b) {
    if (b <= cap_) return;
    cap_ = b;
    for (LBuf *x : {&Z1_, &H1_, &Z2_, &H2_, &Z3_, &H3_, &dZ_, &dZb_}) x->alloc((size_t)b * kMlW * 4);
    out_.alloc((size_t)b * 4);
    dout_.alloc((size_t)b * 4);
    ones_.alloc((size_t)b * 4);
    k_ml_fill<<<256, 256, 0, st_>>>(ones_.as<float>(), b, 1.0f);
    nsplit_max_ = (b + kSplitK - 1) / kSplitK;
    part_.alloc((size_t)nsplit_max_ * kMlW * kMlW * 4);
    lpart_.alloc(256 * 8);
    lck(cudaGetLastError(), "learner buffers");
  }

  void sgemm(const float *A, int64_t sAm, int64_t sAk, const float *B, int64_t sBk, int64_t sBn, int M, int N, int K,
             float *C, int64_t sCm, int64_t sCn, const float *bias, float *H, const float *Zp, int mode) {
    SgArgs g{A, B, sAm, sAk, sBk, sBn, M, N, K, C, sCm, sCn, bias, H, Zp, mode, 0};
    dim3 grid((M + 63) / 64, (N + 63) / 64, 1);
    k_sgemm<<<grid, 256, 0, st_>>>(g);
  }
  // C (dense M x N, row-major) = sum over a long K with split-K partials
  void sgemm_long(const float *A, int64_t sAm, int64_t sAk, const float *B, int64_t sBk, int64_t sBn, int M, int N, int K,
                  float *C) {
    const int nz = (K + kSplitK - 1) / kSplitK;
    SgArgs g{A, B, sAm, sAk, sBk, sBn, M, N, K, part_.as<float>(), N, 1, nullptr, nullptr, nullptr, 0, kSplitK};
    dim3 grid((M + 63) / 64, (N + 63) / 64, nz);
    k_sgemm<<<grid, 256, 0, st_>>>(g);
    k_ml_reduce<<<(M * N + 255) / 256, 256, 0, st_>>>(part_.as<float>(), nz, M * N, C);
  }

  void forward(const float *X, int n) {
    const float *p = params_.as<float>();
    sgemm(X, kMlIn, 1, p + kMlOffW1, 1, kMlIn, n, kMlW, kMlIn, Z1_.as<float>(), kMlW, 1, p + kMlOffB1, H1_.as<float>(),
          nullptr, 1);
    sgemm(H1_.as<float>(), kMlW, 1, p + kMlOffW2, 1, kMlW, n, kMlW, kMlW, Z2_.as<float>(), kMlW, 1, p + kMlOffB2,
          H2_.as<float>(), nullptr, 1);
    sgemm(H2_.as<float>(), kMlW, 1, p + kMlOffW3, 1, kMlW, n, kMlW, kMlW, Z3_.as<float>(), kMlW, 1, p + kMlOffB3,
          H3_.as<float>(), nullptr, 1);
    sgemm(H3_.as<float>(), kMlW, 1, p + kMlOffW4, 1, 0, n, 1, kMlW, out_.as<float>(), 1, 1, p + kMlOffB4, nullptr,
          nullptr, 0);
  }

  void forward_backward(const float *X, const float *y, int n, double *loss) {
    const float *p = params_.as<float>();
    float *gr = grad_.as<float>();
    forward(X, n);
    const int nb = std::min(256, (n + 255) / 256);
    k_ml_dloss<<<nb, 256, 0, st_>>>(out_.as<float>(), y, n, dout_.as<float>(), lpart_.as<double>());
    k_ml_loss_finish<<<1, 32, 0, st_>>>(lpart_.as<double>(), nb, n, loss);
    // output layer: dw4 = H3^T dout, db4 = sum dout, dZ3 = (dout w4^T) * silu'(Z3)
    sgemm_long(H3_.as<float>(), 1, kMlW, dout_.as<float>(), 1, 1, kMlW, 1, n, gr + kMlOffW4);
    sgemm_long(dout_.as<float>(), 0, 1, ones_.as<float>(), 1, 1, 1, 1, n, gr + kMlOffB4);
    sgemm(dout_.as<float>(), 1, 0, p + kMlOffW4, 0, 1, n, kMlW, 1, dZ_.as<float>(), kMlW, 1, nullptr, nullptr,
          Z3_.as<float>(), 2);
    // layer 3: dW3 = dZ3^T H2, db3, dZ2 = (dZ3 W3) * silu'(Z2)
    sgemm_long(dZ_.as<float>(), 1, kMlW, H2_.as<float>(), kMlW, 1, kMlW, kMlW, n, gr + kMlOffW3);
    sgemm_long(dZ_.as<float>(), 1, kMlW, ones_.as<float>(), 1, 1, kMlW, 1, n, gr + kMlOffB3);
    sgemm(dZ_.as<float>(), kMlW, 1, p + kMlOffW3, kMlW, 1, n, kMlW, kMlW, dZb_.as<float>(), kMlW, 1, nullptr, nullptr,
          Z2_.as<float>(), 2);
    // layer 2
    sgemm_long(dZb_.as<float>(), 1, kMlW, H1_.as<float>(), kMlW, 1, kMlW, kMlW, n, gr + kMlOffW2);
    sgemm_long(dZb_.as<float>(), 1, kMlW, ones_.as<float>(), 1, 1, kMlW, 1, n, gr + kMlOffB2);
    sgemm(dZb_.as<float>(), kMlW, 1, p + kMlOffW2, kMlW, 1, n, kMlW, kMlW, dZ_.as<float>(), kMlW, 1, nullptr, nullptr,
          Z1_.as<float>(), 2);
    // layer 1
    sgemm_long(dZ_.as<float>(), 1, kMlW, X, kMlIn, 1, kMlW, kMlIn, n, gr + kMlOffW1);
    sgemm_long(dZ_.as<float>(), 1, kMlW, ones_.as<float>(), 1, 1, kMlW, 1, n, gr + kMlOffB1);
  }

  void upload_weight_tiles() {
    if (!weights_dirty_) return;
    std::vector<float> p(kMlParams);
    get_params(p.data());
    std::vector<uint8_t> w(kWBytes, 0);
    auto put = [&](size_t base, int o, int k, float x) {
      const uint16_t b = host_bf16(x);
      std::memcpy(&w[base + host_cm_off(o, k)], &b, 2);
    };
    for (int o = 0; o < kMlW; ++o) {
      for (int k = 0; k < kMlIn; ++k) put(0, o, k, p[kMlOffW1 + o * kMlIn + k]);
      for (int k = 0; k < kMlW; ++k) {
        put(kWTile, o, k, p[kMlOffW2 + o * kMlW + k]);
        put(3 * kWTile, o, k, p[kMlOffW3 + o * kMlW + k]);
      }
    }
    lck(cudaMemcpy(wt_.p, w.data(), kWBytes, cudaMemcpyHostToDevice), "weight tiles");
    weights_dirty_ = false;
  }

  void run_infer(const InferArgs &a, cudaStream_t st) {
    if (a.ntiles <= 0) return;
    int sms = 0;
    lck(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_), "attribute");
    lck(cudaFuncSetAttribute(k_ml_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem), "attribute");
    k_ml_infer<<<std::min(a.ntiles, std::max(sms, 1)), 128, kInferSmem, st>>>(a);
    lck(cudaGetLastError(), "inference launch");
    int err = 0;
    lck(cudaMemcpyAsync(&err, err_.p, 4, cudaMemcpyDeviceToHost, st), "copy");
    lck(cudaStreamSynchronize(st), "inference");
    if (err) {
      cudaMemset(err_.p, 0, 4);
      throw EngineError(2, "tensor-core inference timed out on an mbarrier wait");
    }
  }

  static constexpr int kSplitK = 512;
  int device_ = 0;
  cudaStream_t st_ = nullptr;
  LBuf params_, m_, v_, grad_, wt_, err_;
  LBuf Z1_, H1_, Z2_, H2_, Z3_, H3_, dZ_, dZb_, out_, dout_, ones_, part_, lpart_;
  int cap_ = 0, nsplit_max_ = 0;
  int64_t t_ = 0;
  bool weights_dirty_ = true;
  std::vector<Chunk> data_;
  LBuf prior_;
  int64_t prior_n_ = 0;
  bool has_prior_ = false;
  float yscale_ = 0.0f;  // RMS of the training targets (0: not measured yet)
  bool folded_ = false;  // the output layer is in the targets' units
};

}  // namespace

std::unique_ptr<ILearner> make_learner(int device, uint64_t seed) { return std::make_unique<Learner>(device, seed); }

}  // namespace ccx
