// Perturbative triples (T): pert_triples2 (ccm_triples.f90:528-735) with its two
// helpers three_body_oneparticle_1 (:174-232) and three_body_onehole_1 (:238-294),
// over the triple channels of setup_t3_channel_structures
// (ccm_t3full_channels.f90:4-284).  One thread per (abc, ijk) pair; the FP64 sum of
// conj(W) W / D is reduced per block and finished in a fixed order.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <stdexcept>
#include <thread>
#include <utility>
#include <vector>

#include "common.cuh"
#include "engine.hpp"
#include "potential.cuh"
#include "triples.hpp"

namespace ccx {

namespace {

void tck(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw EngineError(2, std::string(what) + ": " + cudaGetErrorString(e));
}

struct TriplesDev {
  int ns, A, NP, nk0, nk1, nk2;
  const int *orbit_of;                 // (nx, ny, nz, spin, isospin) -> orbital or -1
  // quantum numbers of each orbital one per byte, biased by kQBias: nx, ny, nz, tz.  A
  // momentum sum q_i + q_j - q_a stays bytewise (no carries, no borrows).
  const unsigned *qn;
  unsigned qlo, qspan;                 // per byte: smallest allowed value, allowed span
  int tzlo;                            // the isospin of the smallest allowed byte-3 value
  const int2 *hp5_slot, *pp5_slot;     // hppp blocks: (channel, row) / (channel, column)
  const int64_t *v5_off;
  const int *n5;                       // rows of each hppp block
  const int2 *hh2_slot, *hp2_slot;     // hhhp blocks: (channel, row) / (channel, column)
  const int64_t *v2_off;
  const int *n2;
  int nt3;
  const int64_t *elem_off;             // prefix of n_hhh * n_ppp over triple channels
  const int *nbra;                     // n_hhh per channel
  const int64_t *hhh_off, *ppp_off;
  const int3 *hhh, *ppp;
};

constexpr int kQBias = 64;

// Bytewise q_i + q_j - q_a of packed quantum numbers: the momentum and isospin of the
// orbital that closes a pair (each byte stays in 0 .. 255 for |n| <= 21 per axis).
__device__ __forceinline__ unsigned qsum(unsigned qi, unsigned qj, unsigned qa) { return __vsub4(__vadd4(qi, qj), qa); }

// Index into orbit_of of packed quantum numbers q with spin -1 (spin +1 is two entries
// further on), or -1 when q lies outside the lattice or the isospin range.
__device__ __forceinline__ int64_t t_orbit_base(const TriplesDev &D, unsigned q) {
  const unsigned d = __vsub4(q, D.qlo);  // per byte: n + nk, and tz - tzlo
  if (__vcmpgtu4(d, D.qspan)) return -1;
  const int x = (int)(d & 0xffu), y = (int)((d >> 8) & 0xffu), z = (int)((d >> 16) & 0xffu);
  const int t = (int)(d >> 24) + D.tzlo;
  const int ey = 2 * D.nk1 + 1, ez = 2 * D.nk2 + 1;
  return ((((int64_t)x * ey + y) * ez + z) * 2) * 2 + (t > 0);
}

// The 18 gather-contractions of a pair run in the contraction type W: the engine's
// scalar S (FP64), or its FP32 counterpart (float, or cplxf for complex engines) on
// FP32 copies of T, V_hppp and V_hhhp.  GB300's FP64 pipe retires 2 FMA per clock per SM
// against 128 for FP32, so the FP32 form takes the contractions off the narrow pipe; the
// |W|^2 / D accumulation stays FP64 in both.
template <typename S> struct LowOf;
template <> struct LowOf<double> { using type = float; };
template <> struct LowOf<cplx> { using type = cplxf; };

template <typename W> __device__ __forceinline__ W wzero();
template <> __device__ __forceinline__ double wzero<double>() { return 0.0; }
template <> __device__ __forceinline__ float wzero<float>() { return 0.0f; }
template <> __device__ __forceinline__ cplx wzero<cplx>() { return cplx(0.0, 0.0); }
template <> __device__ __forceinline__ cplxf wzero<cplxf>() { return cplxf{0.0f, 0.0f}; }

// x with its sign flipped when s is 1: a sign-bit flip on the integer pipe
__device__ __forceinline__ double flip(double x, unsigned s) {
  return __longlong_as_double((long long)((unsigned long long)__double_as_longlong(x) ^ ((unsigned long long)s << 63)));
}
__device__ __forceinline__ float flip(float x, unsigned s) { return __int_as_float(__float_as_int(x) ^ (int)(s << 31)); }
__device__ __forceinline__ cplx flip(cplx x, unsigned s) { return cplx(flip(x.re, s), flip(x.im, s)); }
__device__ __forceinline__ cplxf flip(cplxf x, unsigned s) { return cplxf{flip(x.re, s), flip(x.im, s)}; }

// T(ab, ij) from the two pair slots, with the extra sign m
template <typename W>
__device__ __forceinline__ W t2_slots(const DevLayout &L, const W *T, int2 sab, int2 sij, unsigned m) {
  if (sab.y == 0 || sij.y == 0) return wzero<W>();
  if ((sab.y < 0) != (sij.y < 0)) m ^= 1u;
  return flip(T[L.t_off[sab.x] + sidx(sab.y) + (int64_t)L.P[sab.x] * sidx(sij.y)], m);
}
__device__ __forceinline__ double madd_conj(double v, double t, double acc) { return fma(v, t, acc); }
__device__ __forceinline__ cplx madd_conj(cplx v, cplx t, cplx acc) { return acc + conj_(v) * t; }
__device__ __forceinline__ float madd_conj(float v, float t, float acc) { return fmaf(v, t, acc); }
__device__ __forceinline__ cplxf madd_conj(cplxf v, cplxf t, cplxf acc) {
  return cplxf{fmaf(v.re, t.re, fmaf(v.im, t.im, acc.re)), fmaf(v.re, t.im, fmaf(-v.im, t.re, acc.im))};
}
// |W|^2 in FP64 as the engine's scalar
__device__ __forceinline__ double wnorm2(double w) { return w * w; }
__device__ __forceinline__ double wnorm2(cplx w) { return w.re * w.re + w.im * w.im; }

// acc + sign * sum_d conj(<cb|V|kd>) T(ad, ij), the sign as a bit
template <typename W>
__device__ __forceinline__ W one_particle(const TriplesDev &D, const DevLayout &L, const W *T, const W *V5, int a, int b,
                                       int c, int i, int j, int k, unsigned m, W acc) {
  const int64_t ob = t_orbit_base(D, qsum(D.qn[i], D.qn[j], D.qn[a]));  // d = i + j - a
  if (ob < 0) return acc;
  const int2 cl = D.pp5_slot[(int64_t)(c - D.A) * D.NP + (b - D.A)];
  if (cl.x < 0) return acc;
  const int2 sij = L.hh_slot[i * L.A + j];  // the same for both spins of d
  if (sij.y == 0) return acc;
  for (int sd = 0; sd < 4; sd += 2) {
    const int d = D.orbit_of[ob + sd];
    if (d < D.A) continue;
    const int2 r = D.hp5_slot[(int64_t)k * D.NP + (d - D.A)];
    if (r.x < 0) continue;
    const W t = t2_slots<W>(L, T, L.pp_slot[(int64_t)(a - L.A) * L.NP + (d - L.A)], sij, m);
    acc = madd_conj(V5[D.v5_off[r.x] + r.y + (int64_t)D.n5[r.x] * cl.y], t, acc);
  }
  return acc;
}

// acc + sign * sum_l conj(<jk|V|lc>) T(ab, il)
template <typename W>
__device__ __forceinline__ W one_hole(const TriplesDev &D, const DevLayout &L, const W *T, const W *V2, int a, int b,
                                   int c, int i, int j, int k, unsigned m, W acc) {
  const int64_t ob = t_orbit_base(D, qsum(D.qn[k], D.qn[j], D.qn[c]));  // l = k + j - c
  if (ob < 0) return acc;
  const int2 r = D.hh2_slot[j * D.A + k];
  if (r.x < 0) return acc;
  // the same for both spins of l: the particle pair, its T column base and the V row
  const int2 sab = L.pp_slot[(int64_t)(a - L.A) * L.NP + (b - L.A)];
  if (sab.y == 0) return acc;
  const W *Tc = T + L.t_off[sab.x] + sidx(sab.y);
  const int64_t Pc = L.P[sab.x];
  const W *Vr = V2 + D.v2_off[r.x] + r.y;
  const int64_t nr = D.n2[r.x];
  for (int sl = 0; sl < 4; sl += 2) {
    const int l = D.orbit_of[ob + sl];
    if (l < 0 || l >= D.A) continue;
    const int2 cl = D.hp2_slot[(int64_t)l * D.NP + (c - D.A)];
    if (cl.x < 0) continue;
    const int2 sil = L.hh_slot[i * L.A + l];
    if (sil.y == 0) continue;
    const W t = flip(Tc[Pc * sidx(sil.y)], m ^ (unsigned)((sab.y < 0) != (sil.y < 0)));
    acc = madd_conj(Vr[nr * cl.y], t, acc);
  }
  return acc;
}

// acc += |W|^2 / D.  With FP64 contractions in FP64; with FP32 contractions the ratio is
// formed in FP32 as well (its rounding, 6e-8 of the term, is far below the FP32
// contractions' own) and only the sum is FP64: this GPU's FP64 pipe is 64 times
// narrower, and a complex FP64 division per pair kept it a third busy.
__device__ __forceinline__ void add_term(double w, double d, double (&acc)[2]) { acc[0] += wnorm2(w) / d; }
__device__ __forceinline__ void add_term(cplx w, cplx d, double (&acc)[2]) {
  const cplx t = cplx(wnorm2(w), 0.0) / d;
  acc[0] += t.re;
  acc[1] += t.im;
}
__device__ __forceinline__ void add_term(float w, double d, double (&acc)[2]) {
  acc[0] += (double)((w * w) / (float)d);
}
__device__ __forceinline__ void add_term(cplxf w, cplx d, double (&acc)[2]) {
  const float n = w.re * w.re + w.im * w.im;  // |W|^2
  const float dr = (float)d.re, di = (float)d.im;
  const float s = n / (dr * dr + di * di);     // |W|^2 / D = |W|^2 conj(D) / |D|^2
  acc[0] += (double)(s * dr);
  acc[1] += (double)(-s * di);
}

// FP32 copy of an FP64 array
__device__ __forceinline__ float to_low(double x) { return __double2float_rn(x); }
__device__ __forceinline__ cplxf to_low(cplx x) { return cplxf{__double2float_rn(x.re), __double2float_rn(x.im)}; }
template <typename S>
__global__ void k_to_low(const S *__restrict__ src, int64_t n, typename LowOf<S>::type *__restrict__ dst) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    dst[e] = to_low(src[e]);
}

template <int NV>
__device__ void block_sum(double (&v)[NV], double *partial) {
  __shared__ double red[NV][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = 0; k < NV; ++k) {
    double x = warp_sum(v[k]);
    if (lane == 0) red[k][wid] = x;
  }
  __syncthreads();
  if (wid == 0)
    for (int k = 0; k < NV; ++k) {
      double x = lane < nw ? red[k][lane] : 0.0;
      x = warp_sum(x);
      if (lane == 0) partial[(int64_t)blockIdx.x * NV + k] = x;
    }
}

// Fock sums of every hole triple (f_ii + f_jj + f_kk) and particle triple, once per (T)
template <typename S>
__global__ void k_triple_fock(const int3 *__restrict__ t, int64_t n, const S *__restrict__ fd, S *__restrict__ e) {
  for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
    const int3 q = t[x];
    e[x] = fd[q.x] + fd[q.y] + fd[q.z];
  }
}

// (permutation of the particles, permutation of the holes) of the nine terms of each
// kind, 2 + 2 bits per term: (0,0) (1,0) (2,0) (0,1) (0,2) (2,2) (2,1) (1,2) (1,1)
constexpr unsigned long long kTermOrder = 0x596A84210ull;

template <typename S, typename W>
__global__ void __launch_bounds__(256) k_triples(TriplesDev D, DevLayout L, const W *__restrict__ T,
                                                 const W *__restrict__ V5, const W *__restrict__ V2,
                                                 const S *__restrict__ eh, const S *__restrict__ ep, int64_t total,
                                                 double *partial) {
  double acc[2] = {0.0, 0.0};
  int ch = 0;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
    while (g >= D.elem_off[ch + 1]) ++ch;
    const int64_t loc = g - D.elem_off[ch];
    const int nb = D.nbra[ch];
    const int ket = (int)(loc / nb), bra = (int)(loc % nb);
    const int3 abc = D.ppp[D.ppp_off[ch] + ket];
    const int3 ijk = D.hhh[D.hhh_off[ch] + bra];
    const int a = abc.x, b = abc.y, c = abc.z, i = ijk.x, j = ijk.y, k = ijk.z;
    const S spen = eh[D.hhh_off[ch] + bra] - ep[D.ppp_off[ch] + ket];
    // W = the 9 particle terms minus the 9 hole terms, accumulated in one sum with the
    // permutation signs applied as sign-bit flips.  Each term is one permutation of
    // (a, b, c) and one of (i, j, k), taken in pert_triples2's order (kTermOrder: 2 bits
    // each); the orbitals of a term are picked by selects, so one copy of each term body
    // serves all nine (eighteen inlined bodies outgrow the instruction cache).
    W tc = wzero<W>();
#pragma unroll 3
    for (int t = 0; t < 9; ++t) {
      const int pp = (int)(kTermOrder >> (4 * t)) & 3, hp = (int)(kTermOrder >> (4 * t + 2)) & 3;
      // particle term: (a, b, c) as is, (b, a, c) or (c, b, a); (i, j, k) as is, (k, j, i) or (i, k, j)
      const int A1 = pp == 1 ? b : pp == 2 ? c : a, B1 = pp == 1 ? a : b, C1 = pp == 2 ? a : c;
      const int I1 = hp == 1 ? k : i, J1 = hp == 2 ? k : j, K1 = hp == 1 ? i : hp == 2 ? j : k;
      tc = one_particle<W>(D, L, T, V5, A1, B1, C1, I1, J1, K1, (unsigned)((pp != 0) != (hp != 0)), tc);
    }
#pragma unroll 3
    for (int t = 0; t < 9; ++t) {
      const int pp = (int)(kTermOrder >> (4 * t)) & 3, hp = (int)(kTermOrder >> (4 * t + 2)) & 3;
      // hole term: (a, b, c) as is, (a, c, b) or (c, b, a); (i, j, k) as is, (k, j, i) or (j, i, k)
      const int A1 = pp == 2 ? c : a, B1 = pp == 1 ? c : b, C1 = pp == 1 ? b : pp == 2 ? a : c;
      const int I1 = hp == 1 ? k : hp == 2 ? j : i, J1 = hp == 2 ? i : j, K1 = hp == 1 ? i : k;
      tc = one_hole<W>(D, L, T, V2, A1, B1, C1, I1, J1, K1, (unsigned)((pp != 0) == (hp != 0)), tc);
    }
    add_term(tc, spen, acc);
  }
  block_sum<2>(acc, partial);
}

__global__ void k_finish2(const double *partial, int nb, double *out) {
  const int k = blockIdx.x;
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) s += partial[(int64_t)b * 2 + k];
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

// generation of the V_hppp / V_hhhp blocks (setup_vnn_hppp_block NN part, ccm_iter.f90:1720-1760;
// V_hhhp as ccm_iter.f90:885-930): vnn_hppp(kl, ij) = <ij|V|kl>, vnn_hhhp(ij, kd) = <ij|V|kd>
template <typename S>
__global__ void k_gen_block(DevOrbits O, DevPotential P, const int2 *__restrict__ rows, const int2 *__restrict__ cols,
                            const int64_t *__restrict__ off, const int *__restrict__ nr, const int *__restrict__ nc,
                            const int *__restrict__ roff, const int *__restrict__ coff, int nchan, int rows_are_ket,
                            S *__restrict__ V) {
  for (int ch = blockIdx.x; ch < nchan; ch += gridDim.x) {
    const int r = nr[ch], c = nc[ch];
    for (int64_t e = threadIdx.x; e < (int64_t)r * c; e += blockDim.x) {
      const int ri = (int)(e % r), ci = (int)(e / r);
      const int2 x = rows[roff[ch] + ri], y = cols[coff[ch] + ci];
      V[off[ch] + e] = rows_are_ket ? pot::vanti<S>(O, P, y.x, y.y, x.x, x.y) : pot::vanti<S>(O, P, x.x, x.y, y.x, y.y);
    }
  }
}

template <typename S> __device__ inline S in_cvt(const double *p);
template <> __device__ inline double in_cvt<double>(const double *p) { return p[0]; }
template <> __device__ inline cplx in_cvt<cplx>(const double *p) { return cplx(p[0], p[1]); }
template <typename S>
__global__ void k_copy_in(const double *__restrict__ src, int64_t n, S *__restrict__ dst) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    dst[e] = in_cvt<S>(src + 2 * e);
}

struct DB {
  void *p = nullptr;
  size_t n = 0;
  ~DB() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  template <typename T> void put(const std::vector<T> &h) {
    n = std::max<size_t>(h.size(), 1) * sizeof(T);
    tck(cudaMalloc(&p, n), "cudaMalloc (T)");
    if (!h.empty()) tck(cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice), "upload (T)");
  }
  void zeros(size_t bytes) {
    n = std::max<size_t>(bytes, 1);
    tck(cudaMalloc(&p, n), "cudaMalloc (T)");
    tck(cudaMemset(p, 0, n), "memset (T)");
  }
  template <typename T> T *as() const { return (T *)p; }
};

}  // namespace

template <typename S>
class Triples final : public ITriples<S> {
 public:
  Triples(const Layout &L, const DevLayout &D, const DevOrbits &O, int device) : D_(D), O_(O) {
    tck(cudaSetDevice(device), "cudaSetDevice");
    const Basis &B = L.b;
    const int ns = B.ns, A = B.A, NP = ns - A;
    TD_.ns = ns; TD_.A = A; TD_.NP = NP;
    TD_.nk0 = B.nkmax[0]; TD_.nk1 = B.nkmax[1]; TD_.nk2 = B.nkmax[2];
    orbit_of_.put(B.orbit_of);
    TD_.orbit_of = orbit_of_.as<int>();
    {
      const int nkm = std::max(B.nkmax[0], std::max(B.nkmax[1], B.nkmax[2]));
      if (nkm > 21) throw EngineError(1, "(T): momentum range too large for packed quantum numbers");
      std::vector<unsigned> q(ns);
      for (int p = 0; p < ns; ++p)
        q[p] = (unsigned)(B.nx[p] + kQBias) | (unsigned)(B.ny[p] + kQBias) << 8 | (unsigned)(B.nz[p] + kQBias) << 16 |
               (unsigned)(B.tz[p] + kQBias) << 24;
      qn_.put(q);
      TD_.qn = qn_.as<unsigned>();
      // allowed: |n| <= nk per axis, and the closing orbital's isospin in [tzmin, tzmax]
      // and in [-1, 1]
      const int tzlo = std::max(-1, B.tzmin), tzhi = std::min(1, B.tzmax);
      TD_.tzlo = tzlo;
      TD_.qlo = (unsigned)(kQBias - B.nkmax[0]) | (unsigned)(kQBias - B.nkmax[1]) << 8 |
                (unsigned)(kQBias - B.nkmax[2]) << 16 | (unsigned)(kQBias + tzlo) << 24;
      TD_.qspan = (unsigned)(2 * B.nkmax[0]) | (unsigned)(2 * B.nkmax[1]) << 8 | (unsigned)(2 * B.nkmax[2]) << 16 |
                  (unsigned)std::max(0, tzhi - tzlo) << 24;
    }
    // hppp (kind 5) and hhhp (kind 2) blocks in the reference's ordered layout
    auto blocks = [&](int kind, std::vector<int2> &s1slot, std::vector<int2> &s2slot, bool s1_is_hh, DB &off, DB &nrow,
                      std::vector<int64_t> &offh, std::vector<int2> &rows, std::vector<int2> &cols, std::vector<int> &nr,
                      std::vector<int> &nc, std::vector<int> &roff, std::vector<int> &coff) {
      const ChannelFamily &F = L.fam[kind];
      int64_t acc = 0;
      for (int c = 0; c < F.count(); ++c) {
        const PairList &a = F.side1[c], &b = F.side2[c];
        offh.push_back(acc);
        nr.push_back(a.size());
        nc.push_back(b.size());
        roff.push_back((int)rows.size());
        coff.push_back((int)cols.size());
        acc += (int64_t)a.size() * b.size();
        for (int r = 0; r < a.size(); ++r) {
          rows.push_back(make_int2(a.p[r], a.q[r]));
          if (s1_is_hh) s1slot[(size_t)a.p[r] * A + a.q[r]] = make_int2(c, r);
          else s1slot[(size_t)a.p[r] * NP + (a.q[r] - A)] = make_int2(c, r);
        }
        for (int r = 0; r < b.size(); ++r) {
          cols.push_back(make_int2(b.p[r], b.q[r]));
          if (kind == 5) s2slot[(size_t)(b.p[r] - A) * NP + (b.q[r] - A)] = make_int2(c, r);
          else s2slot[(size_t)b.p[r] * NP + (b.q[r] - A)] = make_int2(c, r);
        }
      }
      off.put(offh);
      nrow.put(nr);
      return acc;
    };
    std::vector<int2> hp5((size_t)A * NP, make_int2(-1, 0)), pp5((size_t)NP * NP, make_int2(-1, 0));
    std::vector<int2> hh2((size_t)A * A, make_int2(-1, 0)), hp2((size_t)A * NP, make_int2(-1, 0));
    std::vector<int64_t> o5, o2;
    std::vector<int2> r5, c5, r2, c2;
    std::vector<int> nr5, nc5, ro5, co5, nr2, nc2, ro2, co2;
    n_v5_ = blocks(5, hp5, pp5, false, v5_off_, n5_, o5, r5, c5, nr5, nc5, ro5, co5);
    n_v2_ = blocks(2, hh2, hp2, true, v2_off_, n2_, o2, r2, c2, nr2, nc2, ro2, co2);
    off5_h_ = o5; off2_h_ = o2; nr5_h_ = nr5; nc5_h_ = nc5; nr2_h_ = nr2; nc2_h_ = nc2;
    hp5_slot_.put(hp5); pp5_slot_.put(pp5); hh2_slot_.put(hh2); hp2_slot_.put(hp2);
    rows5_.put(r5); cols5_.put(c5); rows2_.put(r2); cols2_.put(c2);
    nc5_.put(nc5); ro5_.put(ro5); co5_.put(co5); nc2_.put(nc2); ro2_.put(ro2); co2_.put(co2);
    TD_.hp5_slot = hp5_slot_.as<int2>(); TD_.pp5_slot = pp5_slot_.as<int2>();
    TD_.v5_off = v5_off_.as<int64_t>(); TD_.n5 = n5_.as<int>();
    TD_.hh2_slot = hh2_slot_.as<int2>(); TD_.hp2_slot = hp2_slot_.as<int2>();
    TD_.v2_off = v2_off_.as<int64_t>(); TD_.n2 = n2_.as<int>();
    V5_.zeros((size_t)n_v5_ * sizeof(S));
    V2_.zeros((size_t)n_v2_ * sizeof(S));
    build_t3(L);
    partial_.zeros(kBlocks * 2 * sizeof(double));
    res_.zeros(4 * sizeof(double));
  }

  bool has_v() const override { return have5_ && have2_; }
  int64_t launches() const override { return launches_; }
  int64_t count() const override { return total_; }

  void set_hhhp(int ch, const double *v, cudaStream_t st) override {
    if (ch < 0 || ch >= (int)off2_h_.size()) throw EngineError(1, "hhhp channel out of range");
    stage(v, (int64_t)nr2_h_[ch] * nc2_h_[ch], V2_.as<S>() + off2_h_[ch], st);
    have2_ = true;
    low_ready_ = false;
  }
  void set_hppp(int ch, const double *v, cudaStream_t st) override {
    if (ch < 0 || ch >= (int)off5_h_.size()) throw EngineError(1, "hppp channel out of range");
    stage(v, (int64_t)nr5_h_[ch] * nc5_h_[ch], V5_.as<S>() + off5_h_[ch], st);
    have5_ = true;
    low_ready_ = false;
  }
  void generate_v(const DevPotential &pot, cudaStream_t st) override {
    const int n5 = (int)off5_h_.size(), n2 = (int)off2_h_.size();
    if (n5) k_gen_block<S><<<std::min(n5, 8192), 256, 0, st>>>(O_, pot, rows5_.as<int2>(), cols5_.as<int2>(), v5_off_.as<int64_t>(),
                                                    n5_.as<int>(), nc5_.as<int>(), ro5_.as<int>(), co5_.as<int>(), n5, 1,
                                                    V5_.as<S>());
    if (n2) k_gen_block<S><<<std::min(n2, 8192), 256, 0, st>>>(O_, pot, rows2_.as<int2>(), cols2_.as<int2>(), v2_off_.as<int64_t>(),
                                                    n2_.as<int>(), nc2_.as<int>(), ro2_.as<int>(), co2_.as<int>(), n2, 0,
                                                    V2_.as<S>());
    launches_ += 2;
    tck(cudaGetLastError(), "V_hppp/V_hhhp generation");
    have5_ = have2_ = true;
    low_ready_ = false;
  }
  void energy(const S *T, int64_t n_t, const S *fdiag, double et[2], cudaStream_t st, bool fp32) override {
    if (!has_v()) throw EngineError(4, "(T): V_hppp and V_hhhp blocks are not set");
    if (total_ > 0) {
      k_triple_fock<S><<<1024, 256, 0, st>>>(hhh_.as<int3>(), n_hhh_, fdiag, eh_.as<S>());
      k_triple_fock<S><<<1024, 256, 0, st>>>(ppp_.as<int3>(), n_ppp_, fdiag, ep_.as<S>());
      if (fp32) {
        using Wt = typename LowOf<S>::type;
        if (!low_ready_) {  // FP32 copies of the interaction, once per interaction
          if (!V5l_.p) V5l_.zeros((size_t)std::max<int64_t>(n_v5_, 1) * sizeof(Wt));
          if (!V2l_.p) V2l_.zeros((size_t)std::max<int64_t>(n_v2_, 1) * sizeof(Wt));
          k_to_low<S><<<1216, 256, 0, st>>>(V5_.as<S>(), n_v5_, V5l_.as<Wt>());
          k_to_low<S><<<1216, 256, 0, st>>>(V2_.as<S>(), n_v2_, V2l_.as<Wt>());
          launches_ += 2;
          low_ready_ = true;
        }
        if (Tl_.n < (size_t)std::max<int64_t>(n_t, 1) * sizeof(Wt)) {
          Tl_.release();
          Tl_.zeros((size_t)std::max<int64_t>(n_t, 1) * sizeof(Wt));
        }
        k_to_low<S><<<1216, 256, 0, st>>>(T, n_t, Tl_.as<Wt>());
        k_triples<S, Wt><<<kBlocks, 256, 0, st>>>(TD_, D_, Tl_.as<Wt>(), V5l_.as<Wt>(), V2l_.as<Wt>(), eh_.as<S>(),
                                                  ep_.as<S>(), total_, partial_.as<double>());
        ++launches_;
      } else {
        k_triples<S, S><<<kBlocks, 256, 0, st>>>(TD_, D_, T, V5_.as<S>(), V2_.as<S>(), eh_.as<S>(), ep_.as<S>(), total_,
                                                 partial_.as<double>());
      }
      k_finish2<<<2, 256, 0, st>>>(partial_.as<double>(), kBlocks, res_.as<double>());
      launches_ += 4;
      tck(cudaGetLastError(), "(T) kernel");
      double h[2];
      tck(cudaMemcpyAsync(h, res_.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, st), "(T) result");
      tck(cudaStreamSynchronize(st), "(T) sync");
      et[0] = h[0];
      et[1] = h[1];
    } else {
      et[0] = et[1] = 0.0;
    }
  }

 private:
  static constexpr int kBlocks = 152 * 8;

  void stage(const double *v, int64_t n, S *dst, cudaStream_t st) {
    if (!v) throw EngineError(1, "null V block");
    DB tmp;
    tmp.zeros((size_t)n * 2 * sizeof(double));
    tck(cudaMemcpyAsync(tmp.p, v, (size_t)n * 2 * sizeof(double), cudaMemcpyHostToDevice, st), "V block upload");
    k_copy_in<S><<<608, 256, 0, st>>>(tmp.as<double>(), n, dst);
    ++launches_;
    tck(cudaStreamSynchronize(st), "V block sync");
    if (!ScalarOf<S>::complex) {
      std::vector<double> h((size_t)n * 2);
      std::copy(v, v + 2 * n, h.begin());
      for (int64_t e = 0; e < n; ++e)
        if (h[2 * e + 1] != 0.0) throw EngineError(1, "complex V block given to a real engine");
    }
  }

  // triple channels keyed by (Tz, N), hhh (i<j<k) bras and ppp (a<b<c) kets, in the
  // enumeration order of setup_t3_channel_structures; only keys with both kinds.
  void build_t3(const Layout &L) {
    const Basis &B = L.b;
    const int ns = B.ns, A = B.A;
    int mn[3] = {1 << 30, 1 << 30, 1 << 30}, mx[3] = {-(1 << 30), -(1 << 30), -(1 << 30)};
    for (int p = 0; p < ns; ++p) {
      const int v[3] = {B.nx[p], B.ny[p], B.nz[p]};
      for (int d = 0; d < 3; ++d) { mn[d] = std::min(mn[d], v[d]); mx[d] = std::max(mx[d], v[d]); }
    }
    const int lo[3] = {3 * mn[0], 3 * mn[1], 3 * mn[2]}, hi[3] = {3 * mx[0], 3 * mx[1], 3 * mx[2]};
    const int tlo = 3 * B.tzmin, thi = 3 * B.tzmax;
    const int ex[3] = {hi[0] - lo[0] + 1, hi[1] - lo[1] + 1, hi[2] - lo[2] + 1};
    const int et = thi - tlo + 1;
    auto key = [&](int t, int x, int y, int z) {
      return (((size_t)(t - tlo) * ex[0] + (x - lo[0])) * ex[1] + (y - lo[1])) * ex[2] + (z - lo[2]);
    };
    const size_t nkeys = (size_t)et * ex[0] * ex[1] * ex[2];
    std::vector<std::vector<int3>> hhh(nkeys);
    for (int a = 0; a < A; ++a)
      for (int b = a + 1; b < A; ++b)
        for (int c = b + 1; c < A; ++c)
          hhh[key(B.tz[a] + B.tz[b] + B.tz[c], B.nx[a] + B.nx[b] + B.nx[c], B.ny[a] + B.ny[b] + B.ny[c],
                  B.nz[a] + B.nz[b] + B.nz[c])].push_back(make_int3(a, b, c));
    // particle triples a < b < c of every key that has hole triples, enumerated by host
    // threads over slices of the a range in two passes (count, then fill), laid out key
    // by key in ascending key order and, within a key, in the serial (a, b, c) order
    std::vector<int> live(nkeys, -1);
    int nlive = 0;
    for (size_t k = 0; k < nkeys; ++k)
      if (!hhh[k].empty()) live[k] = nlive++;
    const int nthr = std::max(1, std::min<int>(64, (int)std::thread::hardware_concurrency()));
    const int nsl = std::max(1, std::min(ns - A, 4 * nthr));
    auto bound = [&](int q) {  // slices of about equal work: a costs about (ns - a)^2 / 2
      if (q >= nsl) return ns;
      return A + (int)std::lround((1.0 - std::cbrt(1.0 - (double)q / nsl)) * (ns - A));
    };
    auto sweep = [&](int sl, auto &&emit) {
      for (int a = bound(sl); a < bound(sl + 1); ++a)
        for (int b = a + 1; b < ns; ++b) {
          const int t2 = B.tz[a] + B.tz[b], x2 = B.nx[a] + B.nx[b], y2 = B.ny[a] + B.ny[b], z2 = B.nz[a] + B.nz[b];
          for (int c = b + 1; c < ns; ++c) {
            const int id = live[key(t2 + B.tz[c], x2 + B.nx[c], y2 + B.ny[c], z2 + B.nz[c])];
            if (id >= 0) emit(id, a, b, c);
          }
        }
    };
    auto parallel = [&](auto &&fn) {
      std::atomic<int> next{0};
      auto loop = [&]() {
        for (int sl = next++; sl < nsl; sl = next++) fn(sl);
      };
      std::vector<std::thread> pool;
      for (int t = 1; t < nthr; ++t) pool.emplace_back(loop);
      loop();
      for (auto &t : pool) t.join();
    };
    std::vector<int64_t> cnt((size_t)nsl * nlive, 0);
    parallel([&](int sl) {
      int64_t *c = &cnt[(size_t)sl * nlive];
      sweep(sl, [&](int id, int, int, int) { ++c[id]; });
    });
    std::vector<int64_t> kcount(nlive, 0), kstart(nlive + 1, 0);
    for (int sl = 0; sl < nsl; ++sl)
      for (int id = 0; id < nlive; ++id) kcount[id] += cnt[(size_t)sl * nlive + id];
    for (int id = 0; id < nlive; ++id) kstart[id + 1] = kstart[id] + kcount[id];
    // cnt becomes each slice's write position per key
    for (int id = 0; id < nlive; ++id) {
      int64_t pos = kstart[id];
      for (int sl = 0; sl < nsl; ++sl) {
        const int64_t n = cnt[(size_t)sl * nlive + id];
        cnt[(size_t)sl * nlive + id] = pos;
        pos += n;
      }
    }
    std::vector<int3> pflat(kstart[nlive]);
    parallel([&](int sl) {
      int64_t *w = &cnt[(size_t)sl * nlive];
      sweep(sl, [&](int id, int a, int b, int c) { pflat[w[id]++] = make_int3(a, b, c); });
    });
    std::vector<int64_t> eoff(1, 0), hoff, poff;
    std::vector<int> nbra;
    std::vector<int3> hl;
    for (int t = tlo; t <= thi; t += 2)
      for (int x = lo[0]; x <= hi[0]; ++x)
        for (int y = lo[1]; y <= hi[1]; ++y)
          for (int z = lo[2]; z <= hi[2]; ++z) {
            const size_t k = key(t, x, y, z);
            if (live[k] < 0 || kcount[live[k]] == 0) continue;
            const int id = live[k];
            hoff.push_back((int64_t)hl.size());
            poff.push_back(kstart[id]);  // the key's particle triples, in place in pflat
            nbra.push_back((int)hhh[k].size());
            hl.insert(hl.end(), hhh[k].begin(), hhh[k].end());
            eoff.push_back(eoff.back() + (int64_t)hhh[k].size() * kcount[id]);
          }
    TD_.nt3 = (int)nbra.size();
    total_ = eoff.back();
    eoff.push_back(eoff.back());  // sentinel so the channel walk never reads past the end
    elem_off_.put(eoff); nbra_.put(nbra); hhh_off_.put(hoff); ppp_off_.put(poff); hhh_.put(hl); ppp_.put(pflat);
    n_hhh_ = (int64_t)hl.size();
    n_ppp_ = (int64_t)pflat.size();
    eh_.zeros((size_t)std::max<int64_t>(n_hhh_, 1) * sizeof(S));
    ep_.zeros((size_t)std::max<int64_t>(n_ppp_, 1) * sizeof(S));
    TD_.elem_off = elem_off_.as<int64_t>(); TD_.nbra = nbra_.as<int>();
    TD_.hhh_off = hhh_off_.as<int64_t>(); TD_.ppp_off = ppp_off_.as<int64_t>();
    TD_.hhh = hhh_.as<int3>(); TD_.ppp = ppp_.as<int3>();
  }

  DevLayout D_;
  DevOrbits O_;
  TriplesDev TD_{};
  DB orbit_of_, qn_, hp5_slot_, pp5_slot_, hh2_slot_, hp2_slot_, v5_off_, n5_, v2_off_, n2_;
  DB rows5_, cols5_, rows2_, cols2_, nc5_, ro5_, co5_, nc2_, ro2_, co2_;
  DB V5l_, V2l_, Tl_;  // FP32 copies for the FP32 contractions
  bool low_ready_ = false;
  DB V5_, V2_, elem_off_, nbra_, hhh_off_, ppp_off_, hhh_, ppp_, partial_, res_, eh_, ep_;
  int64_t n_hhh_ = 0, n_ppp_ = 0;
  std::vector<int64_t> off5_h_, off2_h_;
  std::vector<int> nr5_h_, nc5_h_, nr2_h_, nc2_h_;
  int64_t n_v5_ = 0, n_v2_ = 0, total_ = 0, launches_ = 0;
  bool have5_ = false, have2_ = false;
};

template <typename S>
std::unique_ptr<ITriples<S>> make_triples(const Layout &L, const DevLayout &D, const DevOrbits &O, int device) {
  return std::unique_ptr<ITriples<S>>(new Triples<S>(L, D, O, device));
}

template std::unique_ptr<ITriples<double>> make_triples<double>(const Layout &, const DevLayout &, const DevOrbits &, int);
template std::unique_ptr<ITriples<cplx>> make_triples<cplx>(const Layout &, const DevLayout &, const DevOrbits &, int);

}  // namespace ccx
