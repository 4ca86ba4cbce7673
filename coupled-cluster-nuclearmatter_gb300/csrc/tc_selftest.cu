// Self-test of the tensor-core split GEMM: grouped random problems against an FP64
// host product.  Exposed through ccx_selftest_tc_gemm.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "engine.hpp"
#include "ozaki.cuh"
#include "tcgemm.cuh"

namespace ccx {

namespace {
void sck(cudaError_t e, const char *w) {
  if (e != cudaSuccess) throw EngineError(2, std::string(w) + ": " + cudaGetErrorString(e));
}
struct Dev {
  void *p = nullptr;
  size_t bytes = 0;
  explicit Dev(size_t b) : bytes(std::max<size_t>(b, 16)) { sck(cudaMalloc(&p, bytes), "cudaMalloc"); }
  ~Dev() { cudaFree(p); }
};
}  // namespace

// Ozaki digit-product GEMM on the same kind of problems; reference in long double.
static void oz_selftest(int nprob, const int *Ms, const int *Ns, const int *Ks, uint64_t seed, double *max_rel, double *ms) {
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  struct Host {
    int M, N, K, nk, npad, mpad;
    std::vector<double> A, B, C;
  };
  std::vector<Host> h(nprob);
  size_t fa = 0, fb = 0, fc = 0, pa = 0, pb = 0;
  for (int i = 0; i < nprob; ++i) {
    Host &x = h[i];
    x.M = Ms[i]; x.N = Ns[i]; x.K = Ks[i];
    if (x.M <= 0 || x.N <= 0 || x.N > 2048 || x.K <= 0) throw EngineError(1, "selftest: bad problem shape");
    x.nk = (x.K + 63) / 64;
    x.npad = (x.N + 15) / 16 * 16;
    x.mpad = (x.M + 127) / 128 * 128;
    x.A.resize((size_t)x.M * x.K);
    x.B.resize((size_t)x.K * x.N);
    x.C.resize((size_t)x.M * x.N);
    for (double &v : x.A) v = U(rng) * std::pow(10.0, -3.0 * std::fabs(U(rng)));
    for (double &v : x.B) v = U(rng) * std::pow(10.0, -3.0 * std::fabs(U(rng)));
    for (double &v : x.C) v = U(rng);
    fa += x.A.size(); fb += x.B.size(); fc += x.C.size();
    pa += (size_t)x.mpad * x.nk * 64;
    pb += (size_t)x.npad * x.nk * 64;
  }
  Dev dA(fa * 8), dB(fb * 8), dC(fc * 8), plA(pa * kOzSlices * 2), plB(pb * kOzSlices * 2);
  size_t ra = 0, rb = 0;
  for (auto &x : h) { ra += x.M; rb += x.npad; }
  Dev eA(ra * 4), eB(rb * 4), dE(4);
  std::vector<OzSplitJob> jobs;
  std::vector<OzProb> probs;
  std::vector<OzTile> tiles;
  size_t oa = 0, ob = 0, oc = 0, qa = 0, qb = 0, xa = 0, xb = 0;
  for (int i = 0; i < nprob; ++i) {
    Host &x = h[i];
    sck(cudaMemcpy((double *)dA.p + oa, x.A.data(), x.A.size() * 8, cudaMemcpyHostToDevice), "copy A");
    sck(cudaMemcpy((double *)dB.p + ob, x.B.data(), x.B.size() * 8, cudaMemcpyHostToDevice), "copy B");
    sck(cudaMemcpy((double *)dC.p + oc, x.C.data(), x.C.size() * 8, cudaMemcpyHostToDevice), "copy C");
    OzSplitJob ja{};
    ja.src = (double *)dA.p + oa; ja.sr = x.K; ja.sk = 1; ja.rows = x.M; ja.cols = x.K; ja.tile_rows = 128;
    ja.nk = x.nk; ja.rows_pad = x.mpad; ja.planes = (uint16_t *)plA.p + qa; ja.plane_elems = (int64_t)pa;
    ja.exps = (int *)eA.p + xa;
    OzSplitJob jb{};
    jb.src = (double *)dB.p + ob; jb.sr = x.K; jb.sk = 1; jb.rows = x.N; jb.cols = x.K; jb.tile_rows = x.npad;
    jb.nk = x.nk; jb.rows_pad = x.npad; jb.planes = (uint16_t *)plB.p + qb; jb.plane_elems = (int64_t)pb;
    jb.exps = (int *)eB.p + xb;
    jobs.push_back(ja);
    jobs.push_back(jb);
    OzProb p{};
    p.A = ja.planes; p.eA = ja.exps; p.B = jb.planes; p.eB = jb.exps; p.a_plane = (int64_t)pa; p.b_plane = (int64_t)pb;
    p.M = x.M; p.N = x.N; p.nk = x.nk; p.npad = x.npad;
    p.C = (double *)dC.p + oc; p.sCm = 1; p.sCn = x.M; p.alpha = 0.5;
    for (int mt = 0; mt < x.mpad / 128; ++mt)
      for (int n0 = 0; n0 < x.npad; n0 += kOzN) tiles.push_back(OzTile{i, mt, n0});
    probs.push_back(p);
    oa += x.A.size(); ob += x.B.size(); oc += x.C.size();
    qa += (size_t)x.mpad * x.nk * 64; qb += (size_t)x.npad * x.nk * 64;
    xa += x.M; xb += x.npad;
  }
  const std::vector<int2> rows = oz_row_table(jobs);
  const std::vector<int4> chunks = oz_split_chunks(jobs);
  Dev dJ(jobs.size() * sizeof(OzSplitJob)), dR(rows.size() * sizeof(int2)), dK(chunks.size() * sizeof(int4));
  Dev dP(probs.size() * sizeof(OzProb)), dT(tiles.size() * sizeof(OzTile));
  sck(cudaMemcpy(dJ.p, jobs.data(), jobs.size() * sizeof(OzSplitJob), cudaMemcpyHostToDevice), "copy jobs");
  sck(cudaMemcpy(dR.p, rows.data(), rows.size() * sizeof(int2), cudaMemcpyHostToDevice), "copy rows");
  sck(cudaMemcpy(dK.p, chunks.data(), chunks.size() * sizeof(int4), cudaMemcpyHostToDevice), "copy chunks");
  sck(cudaMemcpy(dP.p, probs.data(), probs.size() * sizeof(OzProb), cudaMemcpyHostToDevice), "copy probs");
  sck(cudaMemset(plA.p, 0, pa * kOzSlices * 2), "memset planes");
  sck(cudaMemset(plB.p, 0, pb * kOzSlices * 2), "memset planes");
  sck(cudaMemcpy(dT.p, tiles.data(), tiles.size() * sizeof(OzTile), cudaMemcpyHostToDevice), "copy tiles");
  sck(cudaMemset(dE.p, 0, 4), "memset");
  launch_oz_split((const OzSplitJob *)dJ.p, (const int2 *)dR.p, (int)rows.size(), (const int4 *)dK.p,
                  (int)chunks.size(), 0);
  sck(cudaGetLastError(), "oz split launch");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0);
  launch_oz_gemm((const OzProb *)dP.p, (const OzTile *)dT.p, (int)tiles.size(), (int *)dE.p, 0);
  cudaEventRecord(e1);
  sck(cudaGetLastError(), "oz gemm launch");
  sck(cudaEventSynchronize(e1), "oz gemm");
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = t;
  int err = 0;
  sck(cudaMemcpy(&err, dE.p, 4, cudaMemcpyDeviceToHost), "copy err");
  if (err) throw EngineError(2, "Ozaki GEMM reported error code " + std::to_string(err));
  double worst = 0.0;
  oc = 0;
  for (auto &x : h) {
    std::vector<double> c(x.C.size());
    sck(cudaMemcpy(c.data(), (double *)dC.p + oc, c.size() * 8, cudaMemcpyDeviceToHost), "copy C back");
    long double scale = 0.0L, diff = 0.0L;
    for (int n = 0; n < x.N; ++n)
      for (int m = 0; m < x.M; ++m) {
        long double ref = 0.0L;
        for (int k = 0; k < x.K; ++k) ref += (long double)x.A[(size_t)m * x.K + k] * x.B[(size_t)k + (size_t)x.K * n];
        const long double prod = 0.5L * ref;
        scale = std::max(scale, std::fabs(prod));
        const long double exact = (long double)x.C[m + (size_t)x.M * n] + prod;
        diff = std::max(diff, std::fabs((long double)c[m + (size_t)x.M * n] - exact));
      }
    worst = std::max(worst, (double)(diff / std::max(scale, 1e-300L)));
    oc += x.C.size();
  }
  *max_rel = worst;
}

// problems: M_i, N_i, K_i for i < nprob.  Returns max |C - C_ref| / max |C_ref| over all
// problems and the kernel time (ms).  kind 2: the Ozaki digit-product GEMM.
// wait_budget > 0: the clock-cycle budget of the kernel's pipeline waits; kernel_err
// non-null: the kernel's error word is returned there instead of raised, and the product
// is checked only when it is 0.
void tc_selftest(int device, int kind, int nprob, const int *Ms, const int *Ns, const int *Ks, int use_alo, uint64_t seed,
                 double *max_rel, double *ms, long long wait_budget, int *kernel_err) {
  sck(cudaSetDevice(device), "cudaSetDevice");
  if (kind == 2) {
    oz_selftest(nprob, Ms, Ns, Ks, seed, max_rel, ms);
    return;
  }
  const int tk = kind == kTcBF16 ? 64 : 32;
  const int es = kind == kTcBF16 ? 2 : 4;
  // use_alo bit 1: K cut into up to three separately tiled segments accumulated into one
  // tile, with a C0 term; even problems C = C0 + 1/2 A B, odd ones C += C0 + 1/2 A B
  const bool segmented = (use_alo & 2) != 0;
  use_alo &= 1;
  std::mt19937_64 rng(seed);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  struct Host {
    int M, N, K, nk, npad, mpad;
    std::vector<double> A, B, C, C0;
    std::vector<int> kseg;  // segment boundaries in K (multiples of the K tile)
    size_t a_el, b_el;
  };
  std::vector<Host> h(nprob);
  size_t a_tot = 0, b_tot = 0, c_tot = 0;
  int npad_max = 16;
  for (int i = 0; i < nprob; ++i) {
    Host &x = h[i];
    x.M = Ms[i];
    x.N = Ns[i];
    x.K = Ks[i];
    if (x.M <= 0 || x.N <= 0 || x.N > 2048 || x.K <= 0) throw EngineError(1, "selftest: bad problem shape");
    x.nk = (x.K + tk - 1) / tk;
    x.npad = (x.N + 15) / 16 * 16;
    x.mpad = (x.M + 127) / 128 * 128;
    x.A.resize((size_t)x.M * x.K);
    x.B.resize((size_t)x.K * x.N);
    x.C.resize((size_t)x.M * x.N);
    // entries spanning a few decades, as CCD operands do
    for (double &v : x.A) v = U(rng) * std::pow(10.0, -3.0 * std::fabs(U(rng)));
    for (double &v : x.B) v = U(rng) * std::pow(10.0, -3.0 * std::fabs(U(rng)));
    for (double &v : x.C) v = U(rng);
    x.kseg = {0};
    const int nseg = segmented ? std::min(3, x.nk) : 1;
    for (int g = 1; g < nseg; ++g) x.kseg.push_back(x.nk * g / nseg * tk);
    x.kseg.push_back(x.K);
    if (segmented) {
      x.C0.resize(x.C.size());
      for (double &v : x.C0) v = U(rng);
    }
    int nk_all = 0;
    for (size_t g = 0; g + 1 < x.kseg.size(); ++g) nk_all += (x.kseg[g + 1] - x.kseg[g] + tk - 1) / tk;
    x.a_el = (size_t)x.mpad * nk_all * tk;
    x.b_el = (size_t)x.npad * nk_all * tk;
    a_tot += x.a_el;
    b_tot += x.b_el;
    c_tot += x.C.size();
  }
  // FP64 device copies of the inputs (A row-major M x K, B column-major K x N, C col-major)
  size_t fa = 0, fb = 0;
  for (auto &x : h) { fa += x.A.size(); fb += x.B.size(); }
  Dev dA(fa * 8), dB(fb * 8), dC(c_tot * 8), dC0(segmented ? c_tot * 8 : 8), tAh(a_tot * es), tAl(a_tot * es),
      tBh(b_tot * es), tBl(b_tot * es);
  std::vector<TcSplitJob> jobs;
  std::vector<TcProb> probs;
  std::vector<TcTile> tiles;
  size_t oa = 0, ob = 0, oc = 0, ta = 0, tb = 0;
  for (int i = 0; i < nprob; ++i) {
    Host &x = h[i];
    sck(cudaMemcpy((double *)dA.p + oa, x.A.data(), x.A.size() * 8, cudaMemcpyHostToDevice), "copy A");
    sck(cudaMemcpy((double *)dB.p + ob, x.B.data(), x.B.size() * 8, cudaMemcpyHostToDevice), "copy B");
    sck(cudaMemcpy((double *)dC.p + oc, x.C.data(), x.C.size() * 8, cudaMemcpyHostToDevice), "copy C");
    if (segmented)
      sck(cudaMemcpy((double *)dC0.p + oc, x.C0.data(), x.C0.size() * 8, cudaMemcpyHostToDevice), "copy C0");
    std::vector<TcSeg> segs;
    size_t sa = ta, sb = tb;
    for (size_t g = 0; g + 1 < x.kseg.size(); ++g) {
      const int k0 = x.kseg[g], kg = x.kseg[g + 1] - k0, nkg = (kg + tk - 1) / tk;
      TcSplitJob ja{};
      ja.src = (double *)dA.p + oa + k0; ja.sub = nullptr; ja.sr = x.K; ja.sk = 1;
      ja.rows = x.M; ja.cols = kg; ja.tile_rows = 128; ja.nk = nkg; ja.rows_pad = x.mpad;
      ja.hi = (char *)tAh.p + sa * es; ja.lo = (char *)tAl.p + sa * es;
      TcSplitJob jb{};
      jb.src = (double *)dB.p + ob + k0; jb.sub = nullptr; jb.sr = x.K; jb.sk = 1;  // B(n, k) = B_colmajor[k + K n]
      jb.rows = x.N; jb.cols = kg; jb.tile_rows = x.npad; jb.nk = nkg; jb.rows_pad = x.npad;
      jb.hi = (char *)tBh.p + sb * es; jb.lo = (char *)tBl.p + sb * es;
      jobs.push_back(ja);
      jobs.push_back(jb);
      segs.push_back(TcSeg{ja.hi, use_alo ? ja.lo : nullptr, jb.hi, jb.lo, nkg, 0});
      sa += (size_t)x.mpad * nkg * tk;
      sb += (size_t)x.npad * nkg * tk;
    }
    // N beyond one accumulator: column blocks of <= 256 stepping through the whole B
    for (int n0 = 0; n0 < x.N; n0 += 256) {
      const int nb = std::min(256, x.N - n0);
      const int64_t bst = x.npad > 256 ? (int64_t)x.npad * 128 : 0;
      TcProb p{};
      p.Ahi = segs[0].Ahi; p.Alo = segs[0].Alo;
      p.Bhi = (const char *)segs[0].Bhi + (size_t)n0 * 128; p.Blo = (const char *)segs[0].Blo + (size_t)n0 * 128;
      p.M = x.M; p.N = nb; p.nk = segs[0].nk; p.npad = (nb + 15) / 16 * 16;
      p.bstride = bst;
      for (size_t g = 1; g < segs.size(); ++g) {
        TcSeg e = segs[g];
        e.Bhi = (const char *)e.Bhi + (size_t)n0 * 128;
        e.Blo = (const char *)e.Blo + (size_t)n0 * 128;
        e.bstride = bst;
        p.ext[g - 1] = e;
      }
      p.next = (int)segs.size() - 1;
      if (segmented) {
        p.C0 = (const double *)dC0.p + oc + (size_t)n0 * x.M;
        p.overwrite = (&x - h.data()) % 2 == 0 ? 1 : 0;
      }
      p.C = (double *)dC.p + oc + (size_t)n0 * x.M; p.sCm = 1; p.sCn = x.M; p.alpha = 0.5;
      for (int mt = 0; mt < x.mpad / 128; ++mt) tiles.push_back(TcTile{(int)probs.size(), mt});
      probs.push_back(p);
      npad_max = std::max(npad_max, p.npad);
    }
    oa += x.A.size(); ob += x.B.size(); oc += x.C.size(); ta += x.a_el; tb += x.b_el;
  }
  Dev dJ(jobs.size() * sizeof(TcSplitJob)), dP(probs.size() * sizeof(TcProb)), dT(tiles.size() * sizeof(TcTile)), dE(4);
  sck(cudaMemcpy(dJ.p, jobs.data(), jobs.size() * sizeof(TcSplitJob), cudaMemcpyHostToDevice), "copy jobs");
  sck(cudaMemcpy(dP.p, probs.data(), probs.size() * sizeof(TcProb), cudaMemcpyHostToDevice), "copy probs");
  sck(cudaMemcpy(dT.p, tiles.data(), tiles.size() * sizeof(TcTile), cudaMemcpyHostToDevice), "copy tiles");
  sck(cudaMemset(dE.p, 0, 4), "memset");
  const std::vector<int4> chunks = tc_split_chunks(jobs);
  Dev dK(chunks.size() * sizeof(int4));
  sck(cudaMemcpy(dK.p, chunks.data(), chunks.size() * sizeof(int4), cudaMemcpyHostToDevice), "copy chunks");
  for (Dev *b : {&tAh, &tAl, &tBh, &tBl}) sck(cudaMemset(b->p, 0, b->bytes), "memset tiles");
  launch_tc_split(kind, (const TcSplitJob *)dJ.p, (const int4 *)dK.p, (int)chunks.size(), 0);
  sck(cudaGetLastError(), "split launch");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0);
  int max_nk = 1;  // K tiles of all segments
  for (const auto &x : h) max_nk = std::max<int>(max_nk, (int)(x.a_el / ((size_t)x.mpad * tk)));
  launch_tc_gemm(kind, (const TcProb *)dP.p, (const TcTile *)dT.p, (int)tiles.size(), npad_max, max_nk, (int *)dE.p, 0,
                 wait_budget);
  cudaEventRecord(e1);
  sck(cudaGetLastError(), "tc gemm launch");
  sck(cudaEventSynchronize(e1), "tc gemm");
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = t;
  int err = 0;
  sck(cudaMemcpy(&err, dE.p, 4, cudaMemcpyDeviceToHost), "copy err");
  if (kernel_err) *kernel_err = err;
  if (err && kernel_err) {
    *max_rel = -1.0;
    return;
  }
  if (err) throw EngineError(2, "tensor-core GEMM reported error code " + std::to_string(err));
  double worst = 0.0;
  oc = 0;
  for (auto &x : h) {
    std::vector<double> c(x.C.size());
    sck(cudaMemcpy(c.data(), (double *)dC.p + oc, c.size() * 8, cudaMemcpyDeviceToHost), "copy C back");
    double scale = 0.0, diff = 0.0;
    for (int n = 0; n < x.N; ++n)
      for (int m = 0; m < x.M; ++m) {
        double ref = 0.0;
        for (int k = 0; k < x.K; ++k) ref += x.A[(size_t)m * x.K + k] * x.B[(size_t)k + (size_t)x.K * n];
        const double prod = 0.5 * ref;
        scale = std::max(scale, std::fabs(prod));
        const size_t e = m + (size_t)x.M * n;
        double want = x.C[e] + prod;
        if (segmented) want = ((&x - h.data()) % 2 == 0 ? 0.0 : x.C[e]) + x.C0[e] + prod;
        diff = std::max(diff, std::fabs(c[e] - want));
      }
    worst = std::max(worst, diff / std::max(scale, 1e-300));
    oc += x.C.size();
  }
  *max_rel = worst;
}

}  // namespace ccx
