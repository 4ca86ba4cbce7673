// CCD engine: device image of the layout and the iteration driver
// (ccd_iter, ccm_iter.f90:1-133, with t2_intermediate, diis_t1t2 and
// ccd_energy_save as its per-iteration steps).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "devlayout.hpp"
#include "engine.hpp"
#include "kernels.hpp"
#include "ozaki.cuh"
#include "tcgemm.cuh"
#include "triples.hpp"

namespace ccx {

namespace {

void ck(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw EngineError(2, std::string(what) + ": " + cudaGetErrorString(e));
}
#define CK(x) ck((x), #x)

// Device address of host memory that the current device can read and write in place
// (allocated or registered pinned with CUDA, hence mapped), else null: such blocks are
// read by the packing kernels directly instead of through staging copies.
double *device_view(const void *p) {
  if (!p) return nullptr;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // an unknown pointer is not an error here
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
  return (double *)a.devicePointer;
}

// RAII device buffer
struct DBuf {
  void *p = nullptr;
  size_t bytes = 0;  // requested size
  size_t cap = 0;    // allocated size: a later request that fits reuses the allocation
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  ~DBuf() { if (p) cudaFree(p); }
  void alloc(size_t b, int64_t *counter) {
    if (p && b <= cap) {
      bytes = b;
      return;
    }
    if (p) { cudaFree(p); if (counter) *counter -= (int64_t)cap; p = nullptr; }
    bytes = b;
    cap = 0;
    if (b == 0) return;
    cudaError_t e = cudaMalloc(&p, b);
    if (e != cudaSuccess) {
      p = nullptr;
      throw EngineError(3, std::string("cudaMalloc of ") + std::to_string(b) + " bytes: " + cudaGetErrorString(e));
    }
    cap = b;
    if (counter) *counter += (int64_t)b;
  }
  template <typename T> T *as() const { return (T *)p; }
};

// Two timing events, destroyed on every path out of the scope that made them.
struct EventPair {
  cudaEvent_t a = nullptr, b = nullptr;
  EventPair() {
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
  }
  EventPair(const EventPair &) = delete;
  EventPair &operator=(const EventPair &) = delete;
  ~EventPair() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
  // device time of f() on stream s, in ms
  template <class F>
  float time(cudaStream_t s, F &&f) {
    CK(cudaEventRecord(a, s));
    f();
    CK(cudaEventRecord(b, s));
    CK(cudaEventSynchronize(b));
    float x = 0.f;
    CK(cudaEventElapsedTime(&x, a, b));
    return x;
  }
};

template <typename T>
void upload(DBuf &d, const std::vector<T> &h, int64_t *counter) {
  d.alloc(std::max<size_t>(h.size(), 1) * sizeof(T), counter);
  if (!h.empty()) CK(cudaMemcpy(d.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
}

uint64_t splitmix(uint64_t &st) {
  uint64_t z = (st += 0x9e3779b97f4a7c15ULL);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

// complex LU solve with partial pivoting on |re|+|im| (the pivot rule of ZGESV)
bool zsolve(int n, std::vector<std::complex<double>> &a, std::vector<std::complex<double>> &b) {
  std::vector<int> piv(n);
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = -1.0;
    for (int i = k; i < n; ++i) {
      const auto v = a[i + n * k];
      const double m = std::fabs(v.real()) + std::fabs(v.imag());
      if (m > best) { best = m; p = i; }
    }
    piv[k] = p;
    if (best == 0.0) return false;
    if (p != k)
      for (int j = 0; j < n; ++j) std::swap(a[k + n * j], a[p + n * j]);
    for (int i = k + 1; i < n; ++i) {
      a[i + n * k] /= a[k + n * k];
      for (int j = k + 1; j < n; ++j) a[i + n * j] -= a[i + n * k] * a[k + n * j];
    }
  }
  for (int k = 0; k < n; ++k)
    if (piv[k] != k) std::swap(b[k], b[piv[k]]);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < i; ++j) b[i] -= a[i + n * j] * b[j];
  for (int i = n - 1; i >= 0; --i) {
    for (int j = i + 1; j < n; ++j) b[i] -= a[i + n * j] * b[j];
    b[i] /= a[i + n * i];
  }
  return true;
}

bool dsolve(int n, std::vector<double> a, std::vector<double> &b) {
  for (int k = 0; k < n; ++k) {
    int p = k;
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(a[i + n * k]) > std::fabs(a[p + n * k])) p = i;
    if (a[p + n * k] == 0.0) return false;
    if (p != k) {
      for (int j = 0; j < n; ++j) std::swap(a[k + n * j], a[p + n * j]);
      std::swap(b[k], b[p]);
    }
    for (int i = k + 1; i < n; ++i) {
      const double f = a[i + n * k] / a[k + n * k];
      for (int j = k; j < n; ++j) a[i + n * j] -= f * a[k + n * j];
      b[i] -= f * b[k];
    }
  }
  for (int i = n - 1; i >= 0; --i) {
    for (int j = i + 1; j < n; ++j) b[i] -= a[i + n * j] * b[j];
    b[i] /= a[i + n * i];
  }
  return true;
}

}  // namespace

void draw_lecs(uint64_t seed, double out[9]) {
  // centres: CS, CT in 10^4 GeV^-2, C1..C7 in 10^4 GeV^-4, each drawn uniformly in +/-50%
  // from a splitmix64 stream; units converted to MeV (x1e-2, x1e-8) as the reference does
  // (chiral_module_andreas_with_delta.f90:586-596) and divided by 16 pi, the normalisation
  // of its operator LECs (CS = (c1s0+3 c3s1)/16/pi, :599-600; cnlo, :604-614)
  const double centre[9] = {-0.1, 0.01, 0.1, 0.1, 0.1, 0.1, 0.1, 0.1, 0.1};
  const double pi = 3.14159265358979;
  uint64_t st = seed;
  for (int i = 0; i < 9; ++i) {
    const double u = (double)(splitmix(st) >> 11) * 0x1.0p-53;
    out[i] = centre[i] * (0.5 + u) * (i < 2 ? 1.0e-2 : 1.0e-8) / (16.0 * pi);
  }
}

template <typename S>
class Engine final : public IEngine {
  using E = typename StepOf<S>::type;  // DIIS step vectors of the standard mode

 public:
  Engine(std::shared_ptr<const Layout> L, int device) : L_(std::move(L)) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) throw EngineError(6, "no CUDA device available");
    if (device < 0 || device >= ndev) throw EngineError(1, "device ordinal out of range");
    device_ = device;
    CK(cudaSetDevice(device_));
    check_memory_plan();
    // the residual's X chain runs on a lower-priority side stream beside the main one
    int prio_low = 0, prio_high = 0;
    CK(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high));
    CK(cudaStreamCreateWithPriority(&st_, cudaStreamNonBlocking, prio_high));
    CK(cudaStreamCreateWithPriority(&xs_, cudaStreamNonBlocking, prio_low));
    for (auto &e : xev_) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (auto &e : ev_) CK(cudaEventCreate(&e));
    for (auto &e : kev_) CK(cudaEventCreate(&e));
    build_tables();
    alloc_state();
    // where each packed amplitude's one-body and ring terms come from (layout only)
    omap_.alloc(std::max<int64_t>(n_t_, 1) * sizeof(int4), &bytes_);
    rmap_.alloc(std::max<int64_t>(n_t_, 1) * sizeof(int4), &bytes_);
    launch_rinit_maps(D_, omap_.as<int4>(), rmap_.as<int4>(), st_);
    CK(cudaStreamSynchronize(st_));
  }
  ~Engine() override {
    cudaSetDevice(device_);
    if (st_) cudaStreamSynchronize(st_);
    for (auto &e : ev_) if (e) cudaEventDestroy(e);
    for (auto &e : kev_) if (e) cudaEventDestroy(e);
    if (xs_) cudaStreamSynchronize(xs_);
    if (st_) cudaStreamDestroy(st_);
    if (xs_) cudaStreamDestroy(xs_);
    for (auto &e : xev_) if (e) cudaEventDestroy(e);
    if (cs_) cudaStreamDestroy(cs_);
    for (auto &e : sev_) if (e) cudaEventDestroy(e);
    for (auto &r : replay_) if (r.exec) cudaGraphExecDestroy(r.exec);
    if (host_res_) cudaFreeHost(host_res_);
  }

  bool is_complex() const override { return ScalarOf<S>::complex; }
  int64_t device_bytes() const override { return bytes_; }
  int64_t launches() const override { return launches_; }
  int64_t diis_fallbacks() const override { return diis_fallbacks_; }
  void set_triples_precision(int p) override {
    if (p != 0 && p != 1) throw EngineError(1, "unknown (T) precision");
    triples_fp32_ = p == 1;
  }
  void timers(double ms[10]) const override { for (int i = 0; i < 10; ++i) ms[i] = timers_[i]; }
  void kernel_timers(double ms[kKernelSlots], int64_t n[kKernelSlots]) const override {
    for (int i = 0; i < kKernelSlots; ++i) { ms[i] = ktimers_[i]; n[i] = kcount_[i]; }
  }
  const std::vector<IterRecord> &iter_log() const override { return ilog_; }

  // ---------------------------------------------------------------- interaction
  void set_fock(const double *fock, const double e0[2]) override {
    const Layout &L = *L_;
    const int ns = L.b.ns, A = L.b.A;
    std::vector<S> fd(ns), f6(std::max(ns - A, 1)), f7(std::max(A, 1));
    auto F = [&](int p, int q) {
      const size_t o = 2 * ((size_t)p + (size_t)ns * q);
      return check_real(fock[o], fock[o + 1]);
    };
    for (int p = 0; p < ns; ++p) {
      fd[p] = F(p, p);
      const int pb = partner_[p];
      if (p >= A) f6[p - A] = (pb >= A) ? F(p, pb) : S(0.0);
      else f7[p] = (pb >= 0 && pb < A) ? F(pb, p) : S(0.0);
    }
    CK(cudaMemcpy(fdiag_.p, fd.data(), ns * sizeof(S), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(f6_.p, f6.data(), f6.size() * sizeof(S), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(f7_.p, f7.data(), f7.size() * sizeof(S), cudaMemcpyHostToDevice));
    e0_[0] = e0 ? e0[0] : 0.0;
    e0_[1] = e0 ? e0[1] : 0.0;
    have_fock_ = true;
  }

  // one block; the host buffer is read before the call returns
  void set_vblock(int kind, int ch, const double *v) override {
    if (double *dv = (kind == 1 || kind == 3 || kind == 6) ? device_view(v) : nullptr) set_vblock_direct(kind, ch, dv);
    else set_vblock_async(kind, ch, v, 0);
    finish_vblocks();
  }
  // a block in device-addressable host memory, packed in place on the compute stream
  void set_vblock_direct(int kind, int ch, const double *src) {
    const Layout &L = *L_;
    int rows = 0, target = -1, rp = 0, cp = 0;
    if (kind == 3 || kind == 6) {
      check_ch(ch, L.fam[3].count());
      const auto &pk = L.pk[ch];
      target = ch;
      rows = kind == 3 ? pk.n_hh : pk.n_pp;
      rp = kind == 3 ? pk.H : pk.P;
      cp = pk.P;
    } else {
      check_ch(ch, L.fam[1].count());
      rows = L.fam[1].side1[ch].size();
      target = hhhh_to_hhpp_[ch];
      if (target < 0) return;  // an hhhh channel without an hhpp partner is not used by CCD
      rp = cp = L.pk[target].H;
    }
    S *dst = kind == 3 ? Vhp_.as<S>() : kind == 6 ? Vpp_.as<S>() : Vhh_.as<S>();
    launch_pack_vblock_host<S>(D_, kind, target, rows, rp, cp, src, dst, flag_.as<int>(), st_);
    ++launches_;
    dirty_ = true;
    user_set_ |= 1u << kind;
    ++v_version_;
  }
  // HPHP blocks in device-addressable host memory: one batched copy launch
  void set_v4_direct(int n, const int *chs, double *const *src) {
    const Layout &L = *L_;
    adopt_hphp();
    std::vector<CopyJob> jobs(n);
    for (int i = 0; i < n; ++i) {
      check_ch(chs[i], L.fam[4].count());
      const int64_t m = L.fam[4].side1[chs[i]].size();
      jobs[i] = CopyJob{src[i], v4_.as<double>() + 2 * v4_off_h_[chs[i]], m * m * 2};
    }
    copyjobs_.alloc(std::max<size_t>(jobs.size(), 1) * sizeof(CopyJob), &bytes_);
    CK(cudaMemcpyAsync(copyjobs_.p, jobs.data(), jobs.size() * sizeof(CopyJob), cudaMemcpyHostToDevice, st_));
    launch_copy_jobs((const CopyJob *)copyjobs_.p, n, st_);
    CK(cudaStreamSynchronize(st_));  // the job table on the host goes out of scope
    ++launches_;
    dirty_ = true;
    user_set_ |= 1u << 4;
    ++v_version_;
  }
  // Many blocks of one kind with one synchronisation at the end.  Staged blocks
  // alternate between two staging buffers: the host-to-device copies run back to back
  // on a copy stream while the compute stream packs the previous block.
  void set_vblocks(int kind, int n, const int *chs, const double *const *vs) override {
    const bool staged = kind == 1 || kind == 3 || kind == 6;
    if (n > 0 && (staged || kind == 4)) {
      // blocks in device-addressable host memory are read in place: no staging copies,
      // and only the cache lines that hold unique pairs cross the link.  V_pppp' is read
      // a column at a time; another family larger than kDirectMaxBytes goes through the
      // copy engines instead (its tile transposes spread over too many host pages).
      std::vector<double *> dv(n);
      bool direct = kind == 6 || family_bytes(kind, n, chs) <= kDirectMaxBytes;
      for (int i = 0; i < n && direct; ++i) direct = (dv[i] = device_view(vs[i])) != nullptr;
      if (direct) {
        if (kind == 4) set_v4_direct(n, chs, dv.data());
        else for (int i = 0; i < n; ++i) set_vblock_direct(kind, chs[i], dv[i]);
        finish_vblocks();
        return;
      }
    }
    if (staged && n > 1) {
      if (!cs_) {
        CK(cudaStreamCreateWithFlags(&cs_, cudaStreamNonBlocking));
        for (auto &e : sev_) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      }
      if (stage2_.bytes < stage_.bytes) stage2_.alloc(stage_.bytes, &bytes_);
      // earlier work on the compute stream may still read the staging buffers
      CK(cudaEventRecord(sev_[4], st_));
      CK(cudaStreamWaitEvent(cs_, sev_[4], 0));
    }
    for (int i = 0; i < n; ++i) set_vblock_async(kind, chs[i], vs[i], staged && n > 1 ? 1 + (i & 1) : 0, i >= 2);
    if (staged && n > 1) CK(cudaStreamSynchronize(cs_));
    finish_vblocks();
  }
  static constexpr double kDirectMaxBytes = 16e9;
  // bytes of n reference-layout blocks of one family
  double family_bytes(int kind, int n, const int *chs) const {
    const Layout &L = *L_;
    double b = 0.0;
    for (int i = 0; i < n; ++i) {
      const int ch = chs[i];
      double r = 0, c = 0;
      if ((kind == 3 || kind == 6) && ch >= 0 && ch < L.fam[3].count()) {
        r = kind == 3 ? L.pk[ch].n_hh : L.pk[ch].n_pp;
        c = L.pk[ch].n_pp;
      } else if ((kind == 1 || kind == 4) && ch >= 0 && ch < L.fam[kind].count()) {
        r = c = L.fam[kind].side1[ch].size();
      }
      b += 16.0 * r * c;
    }
    return b;
  }
  // the copies have been read once this returns; reports here whether any block it
  // packed held a NaN or Inf, or (real engine) a non-zero imaginary part
  void finish_vblocks() { check_flag("V block has a non-zero imaginary part but the engine is real"); }
  // slot 0: stage through stage_ on the compute stream; slots 1, 2: stage_ / stage2_
  // with the copy on the copy stream (reuse waits for the slot's previous pack)
  void set_vblock_async(int kind, int ch, const double *v, int slot, bool reuse = false) {
    const Layout &L = *L_;
    if (!v) throw EngineError(1, "null V block");
    int rows = 0;
    int64_t elems = 0;
    int target = -1;
    switch (kind) {
      case 3:
        check_ch(ch, L.fam[3].count());
        rows = L.pk[ch].n_hh;
        elems = (int64_t)rows * L.pk[ch].n_pp;
        target = ch;
        break;
      case 6:
        check_ch(ch, L.fam[3].count());
        rows = L.pk[ch].n_pp;
        elems = (int64_t)rows * rows;
        target = ch;
        break;
      case 1: {
        check_ch(ch, L.fam[1].count());
        rows = L.fam[1].side1[ch].size();
        elems = (int64_t)rows * rows;
        target = hhhh_to_hhpp_[ch];
        break;
      }
      case 4: {
        check_ch(ch, L.fam[4].count());
        adopt_hphp();
        const int n = L.fam[4].side1[ch].size();
        CK(cudaMemcpyAsync(v4_.as<double>() + 2 * v4_off_h_[ch], v, (size_t)n * n * 2 * sizeof(double),
                           cudaMemcpyHostToDevice, st_));
        user_set_ |= 1u << 4;
        dirty_ = true;
        ++v_version_;
        return;
      }
      case 2:
        check_ch(ch, L.fam[2].count());
        if (!tr_) tr_ = make_triples<S>(*L_, D_, O_, device_);
        tr_->set_hhhp(ch, v, st_);
        return;
      case 5:
        check_ch(ch, L.fam[5].count());
        if (!tr_) tr_ = make_triples<S>(*L_, D_, O_, device_);
        tr_->set_hppp(ch, v, st_);
        return;
      default:
        throw EngineError(1, "unknown V block kind");
    }
    if (target < 0) return;  // an hhhh channel without an hhpp partner is not used by CCD
    S *dst = kind == 3 ? Vhp_.as<S>() : kind == 6 ? Vpp_.as<S>() : Vhh_.as<S>();
    const size_t bytes = (size_t)elems * 2 * sizeof(double);
    if (slot == 0) {
      CK(cudaMemcpyAsync(stage_.p, v, bytes, cudaMemcpyHostToDevice, st_));
      launch_pack_vblock<S>(D_, kind, target, rows, stage_.as<double>(), dst, flag_.as<int>(), st_);
    } else {
      const int b = slot - 1;
      double *buf = (b ? stage2_ : stage_).as<double>();
      if (reuse) CK(cudaStreamWaitEvent(cs_, sev_[2 + b], 0));  // the slot's previous pack is done
      CK(cudaMemcpyAsync(buf, v, bytes, cudaMemcpyHostToDevice, cs_));
      CK(cudaEventRecord(sev_[b], cs_));
      CK(cudaStreamWaitEvent(st_, sev_[b], 0));
      launch_pack_vblock<S>(D_, kind, target, rows, buf, dst, flag_.as<int>(), st_);
      CK(cudaEventRecord(sev_[2 + b], st_));
    }
    ++launches_;
    dirty_ = true;
    user_set_ |= 1u << kind;
    ++v_version_;
  }

  void generate(const PotentialSpec &p) override {
    if (!ScalarOf<S>::complex && p.kind != 0) throw EngineError(1, "the chiral-like potential needs a complex engine");
    DevPotential pot{};
    pot.kind = p.kind;
    pot.f32_literals = p.f32_literals;
    draw_lecs(p.lec_seed, pot.lec);
    const int npp = npp_total_, nhh = nhh_total_;
    if (ScalarOf<S>::complex && p.kind == 1)
      pairf_.alloc(((size_t)npp + nhh + (size_t)D_.A * D_.NP) * sizeof(double) + 8, &bytes_);
    launch_generate<S>(D_, O_, pot, Vhp_.as<S>(), Vpp_.as<S>(), Vhh_.as<S>(), W_.as<S>(), fdiag_.as<S>(), f6_.as<S>(),
                       f7_.as<S>(), res_.as<double>(), pairf_.as<double>(), npp, nhh, st_);
    launches_ += 6;
    CK(cudaMemcpyAsync(host_res_, res_.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, st_));
    CK(cudaStreamSynchronize(st_));
    e0_[0] = host_res_[0];
    e0_[1] = host_res_[1];
    have_fock_ = true;
    generated_ = true;
    w_generated_ = true;
    user_set_ = 0;
    pot_ = pot;
    dirty_ = true;
    ++v_version_;
    vph_ready_ = false;
    commit();
  }
  // The first caller HPHP block on a generated engine: W is rebuilt from the stored
  // reference-layout blocks from now on, so every HPHP block of the generated
  // interaction is written there first (channels the caller does not set keep it).
  void adopt_hphp() {
    if (!w_generated_) return;
    const Layout &L = *L_;
    const ChannelFamily &F = L.fam[4];
    std::vector<int2> pairs;
    std::vector<int64_t> first(F.count());
    for (int ch = 0; ch < F.count(); ++ch) {
      first[ch] = (int64_t)pairs.size();
      const PairList &pl = F.side1[ch];
      for (int i = 0; i < pl.size(); ++i) pairs.push_back(make_int2(pl.p[i], pl.q[i]));
    }
    DBuf dp;
    upload(dp, pairs, nullptr);
    for (int ch = 0; ch < F.count(); ++ch) {
      const int n = F.side1[ch].size();
      if (n <= 0) continue;
      const int2 *pr = dp.as<int2>() + first[ch];
      launch_gen_ordered<S>(O_, pot_, pr, pr, n, n, 0, v4_.as<double>() + 2 * v4_off_h_[ch], st_);
      ++launches_;
    }
    CK(cudaStreamSynchronize(st_));  // the pair table goes out of scope
    w_generated_ = false;
  }
  void get_e0(double e0[2]) override { e0[0] = e0_[0]; e0[1] = e0_[1]; }
  void *stream() const override { return (void *)st_; }

  void get_vblock(int kind, int ch, double *v) override {
    const Layout &L = *L_;
    if (!v) throw EngineError(1, "null output block");
    const ChannelFamily *F = nullptr;
    switch (kind) {
      case 1: F = &L.fam[1]; break;
      case 2: F = &L.fam[2]; break;
      case 3: F = &L.fam[3]; break;
      case 4: F = &L.fam[4]; break;
      case 5: F = &L.fam[5]; break;
      case 6: F = &L.fam[3]; break;
      default: throw EngineError(1, "unknown V block kind");
    }
    check_ch(ch, F->count());
    const PairList &rows = kind == 6 ? F->side2[ch] : F->side1[ch];
    const PairList &cols = (kind == 1 || kind == 4) ? F->side1[ch] : F->side2[ch];
    const int nr = rows.size(), nc = cols.size();
    const size_t bytes = (size_t)nr * nc * 2 * sizeof(double);
    if (bytes > stage_.bytes) stage_.alloc(bytes, &bytes_);
    if (kind == 4 && !w_generated_ && (user_set_ >> 4 & 1u)) {  // the caller's HPHP block, as stored
      CK(cudaMemcpyAsync(v, v4_.as<double>() + 2 * v4_off_h_[ch], bytes, cudaMemcpyDeviceToHost, st_));
      CK(cudaStreamSynchronize(st_));
      return;
    }
    if (generated_ && !(user_set_ >> kind & 1u)) {
      std::vector<int2> r(nr), c(nc);
      for (int i = 0; i < nr; ++i) r[i] = make_int2(rows.p[i], rows.q[i]);
      for (int i = 0; i < nc; ++i) c[i] = make_int2(cols.p[i], cols.q[i]);
      DBuf dr, dc;
      upload(dr, r, nullptr);
      upload(dc, c, nullptr);
      launch_gen_ordered<S>(O_, pot_, dr.as<int2>(), dc.as<int2>(), nr, nc, kind == 5 ? 1 : 0, stage_.as<double>(), st_);
      ++launches_;
      CK(cudaMemcpyAsync(v, stage_.p, bytes, cudaMemcpyDeviceToHost, st_));
      CK(cudaStreamSynchronize(st_));
      return;
    }
    int target = ch;
    if (kind == 1) target = hhhh_to_hhpp_[ch];
    if (!(kind == 3 || kind == 6 || (kind == 1 && target >= 0)))
      throw EngineError(4, "this V block is not stored by the engine (it was not generated on the device)");
    const int *rs = (kind == 3 || kind == 1) ? hh_sgn_.as<int>() + hhsgn_off_[target] : pp_sgn_.as<int>() + ppsgn_off_[target];
    const int *cs = (kind == 1) ? hh_sgn_.as<int>() + hhsgn_off_[target] : pp_sgn_.as<int>() + ppsgn_off_[target];
    const S *src = kind == 3 ? Vhp_.as<S>() : kind == 6 ? Vpp_.as<S>() : Vhh_.as<S>();
    launch_unpack_vblock<S>(D_, kind, target, nr, nc, rs, cs, src, stage_.as<double>(), st_);
    ++launches_;
    CK(cudaMemcpyAsync(v, stage_.p, bytes, cudaMemcpyDeviceToHost, st_));
    CK(cudaStreamSynchronize(st_));
  }

  void get_fock(double *f) override {
    const Layout &L = *L_;
    const int ns = L.b.ns, A = L.b.A;
    std::vector<S> fd(ns), f6(std::max(ns - A, 1)), f7(std::max(A, 1));
    CK(cudaStreamSynchronize(st_));
    CK(cudaMemcpy(fd.data(), fdiag_.p, ns * sizeof(S), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(f6.data(), f6_.p, f6.size() * sizeof(S), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(f7.data(), f7_.p, f7.size() * sizeof(S), cudaMemcpyDeviceToHost));
    std::fill(f, f + 2 * (size_t)ns * ns, 0.0);
    auto put = [&](int p, int q, S v, bool conj) {
      const size_t o = 2 * ((size_t)p + (size_t)ns * q);
      f[o] = real_(v);
      f[o + 1] = conj ? -imag_(v) : imag_(v);
    };
    for (int p = 0; p < ns; ++p) {
      put(p, p, fd[p], false);
      const int pb = partner_[p];
      if (p >= A && pb >= A) {
        put(p, pb, f6[p - A], false);
        put(pb, p, f6[p - A], true);
      } else if (p < A && pb >= 0 && pb < A) {
        put(pb, p, f7[p], false);
        put(p, pb, f7[p], true);
      }
    }
  }

  // ---------------------------------------------------------------- amplitudes
  void mp2() override {
    commit();
    launch_mp2<S>(D_, Vhp_.as<S>(), fdiag_.as<S>(), T_.as<S>(), st_);
    ++launches_;
    have_t_ = true;
    CK(cudaStreamSynchronize(st_));
  }
  void set_t2(int ch, const double *t) override {
    const Layout &L = *L_;
    check_ch(ch, L.fam[3].count());
    const auto &P = L.pk[ch];
    CK(cudaMemcpyAsync(stage_.p, t, (size_t)P.n_pp * P.n_hh * 2 * sizeof(double), cudaMemcpyHostToDevice, st_));
    launch_pack_t<S>(D_, ch, P.n_pp, stage_.as<double>(), T_.as<S>(), flag_.as<int>(), st_);
    ++launches_;
    check_flag("T2 has a non-zero imaginary part but the engine is real");
    have_t_ = true;
  }
  void get_block(int ch, const S *src, double *out) {
    const Layout &L = *L_;
    check_ch(ch, L.fam[3].count());
    const auto &P = L.pk[ch];
    launch_unpack_t<S>(D_, ch, P.n_pp, pp_sgn_.as<int>() + ppsgn_off_[ch], hh_sgn_.as<int>() + hhsgn_off_[ch], P.n_hh,
                       src, stage_.as<double>(), st_);
    ++launches_;
    CK(cudaMemcpyAsync(out, stage_.p, (size_t)P.n_pp * P.n_hh * 2 * sizeof(double), cudaMemcpyDeviceToHost, st_));
    CK(cudaStreamSynchronize(st_));
  }
  void get_t2(int ch, double *t) override { get_block(ch, T_.as<S>(), t); }
  void get_r2(int ch, double *r) override { get_block(ch, R_.as<S>(), r); }
  void set_t2_all(const double *t) override {
    const Layout &L = *L_;
    for (int c = 0; c < L.fam[3].count(); ++c) set_t2(c, t + 2 * L.pk[c].amp_off);
  }
  void get_t2_all(double *t) override {
    const Layout &L = *L_;
    if (double *dt = device_view(t)) {
      // device-addressable host memory: every channel unpacked in place, one sync
      for (int c = 0; c < L.fam[3].count(); ++c) {
        const auto &P = L.pk[c];
        launch_unpack_t<S>(D_, c, P.n_pp, pp_sgn_.as<int>() + ppsgn_off_[c], hh_sgn_.as<int>() + hhsgn_off_[c], P.n_hh,
                           T_.as<S>(), dt + 2 * P.amp_off, st_);
        ++launches_;
      }
      CK(cudaStreamSynchronize(st_));
      return;
    }
    for (int c = 0; c < L.fam[3].count(); ++c) get_t2(c, t + 2 * L.pk[c].amp_off);
  }
  void get_denominators(double *d2ij, double *d2ab) override {
    const Layout &L = *L_;
    const int A = L.b.A, NP = L.b.ns - A;
    std::vector<S> a(A), b(NP);
    CK(cudaStreamSynchronize(st_));
    CK(cudaMemcpy(a.data(), d2ij_.p, A * sizeof(S), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(b.data(), d2ab_.p, NP * sizeof(S), cudaMemcpyDeviceToHost));
    for (int i = 0; i < A; ++i) { d2ij[2 * i] = real_(a[i]); d2ij[2 * i + 1] = imag_(a[i]); }
    for (int i = 0; i < NP; ++i) { d2ab[2 * i] = real_(b[i]); d2ab[2 * i + 1] = imag_(b[i]); }
  }

  // ---------------------------------------------------------------- hot path
  void t2_intermediate() override {
    require_ready();
    residual(false);
    CK(cudaStreamSynchronize(st_));
  }
  void diis_setup(int subspace, int step) override {
    if (subspace < 2 || subspace > 6 || step < 1) throw EngineError(1, "diis subspace must be 2..6, step >= 1");
    subspace_ = subspace;
    diis_step_ = step;
    nstep_ = 0;
    hist_.alloc((size_t)(subspace + 1) * n_t_ * sizeof(S), &bytes_);
    phys_.resize(subspace + 1);
    for (int i = 0; i <= subspace; ++i) phys_[i] = i;
  }
  void diis_t1t2(int *count) override {
    if (subspace_ == 0) diis_setup(6, 6);
    ++nstep_;
    reference_update(*count);
    if (*count == diis_step_) *count = 0;
    CK(cudaStreamSynchronize(st_));
  }
  void energy(double e[2]) override {
    require_ready();
    launch_update<S>(D_, 2, T_.as<S>(), R_.as<S>(), Vhp_.as<S>(), d2ij_.as<S>(), d2ab_.as<S>(), nullptr, nullptr,
                     partial_.as<double>(), res_.as<double>(), st_);
    launches_ += 2;
    fetch_res(3);
    e[0] = host_res_[0];
    e[1] = host_res_[1];
  }
  double residual_norm() override {
    launch_update<S>(D_, 3, T_.as<S>(), R_.as<S>(), Vhp_.as<S>(), d2ij_.as<S>(), d2ab_.as<S>(), nullptr, nullptr,
                     partial_.as<double>(), res_.as<double>(), st_);
    launches_ += 2;
    fetch_res(3);
    return 2.0 * std::sqrt(host_res_[2]);
  }

  void ccd_iter(const IterOpts &o, IterResult &r) override {
    require_ready();
    if (o.precision < 0 || o.precision > 2) throw EngineError(1, "unknown precision");
    if (o.rebase < 0 || o.rebase > 1) throw EngineError(1, "unknown re-base product kind");
    if (o.precision != 0 && o.mode != 1) throw EngineError(1, "mixed precision runs with the standard (DIIS) mode");
    r = IterResult();
    if (o.mode == 0) {
      double e[2];
      energy(e);
      r.e_mbpt2[0] = e[0];
      r.e_mbpt2[1] = e[1];
    }
    for (double &t : timers_) t = 0.0;
    for (double &t : ktimers_) t = 0.0;
    for (int64_t &c : kcount_) c = 0;
    kn_ = 0;
    timing_ = profiling_;
    CK(cudaEventRecord(ev_[10], st_));
    if (o.mode == 0) iterate_reference(o, r);
    else iterate_standard(o, r);
    CK(cudaEventRecord(ev_[11], st_));
    CK(cudaEventSynchronize(ev_[11]));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ev_[10], ev_[11]));
    r.seconds = ms * 1e-3;
    timers_[9] = ms;
    timing_ = false;
  }

  void triples(double et[2]) override {
    require_ready();
    if (!tr_) tr_ = make_triples<S>(*L_, D_, O_, device_);
    if (!tr_->has_v()) {
      if (!generated_) throw EngineError(4, "(T) needs V_hhhp and V_hppp: set every HHHP and HPPP block, or generate the interaction");
      tr_->generate_v(pot_, st_);
    }
    tr_->energy(T_.as<S>(), n_t_, fdiag_.as<S>(), et, st_, triples_fp32_);
    launches_ += tr_->launches();
  }

 private:
  // ================================================================== setup
  void check_ch(int ch, int n) const {
    if (ch < 0 || ch >= n) throw EngineError(1, "channel index out of range");
  }
  S check_real(double re, double im) {
    if (!ScalarOf<S>::complex && im != 0.0) throw EngineError(1, "complex input given to a real engine");
    return make_scalar<S>(re, im);
  }
  // Input checks of the packing kernels (cvt_in): a NaN or Inf is CCX_ENUMERIC, a
  // complex value given to a real engine CCX_EINVAL with msg.  The flag is cleared
  // either way, so the engine stays usable once the caller hands over a valid block.
  void check_flag(const char *msg) {
    int f = 0;
    CK(cudaMemcpyAsync(&host_flag_, flag_.p, sizeof(int), cudaMemcpyDeviceToHost, st_));
    CK(cudaStreamSynchronize(st_));
    f = host_flag_;
    if (f) {
      CK(cudaMemsetAsync(flag_.p, 0, sizeof(int), st_));
      CK(cudaStreamSynchronize(st_));
      if (f & 2) throw EngineError(5, "input holds NaN or Inf");
      throw EngineError(1, msg);
    }
  }
  bool ml_view(MLView &v, bool need_t) override {
    if constexpr (!std::is_same<S, double>::value) {
      return false;
    } else {
      if (!have_fock_) throw EngineError(4, "no Fock matrix / interaction set");
      if (need_t && !have_t_) throw EngineError(4, "no T2 amplitudes");
      commit();
      const Basis &b = L_->b;
      v.L = D_;
      v.O = O_;
      v.fdiag = fdiag_.as<double>();
      v.Vhp = Vhp_.as<double>();
      v.T = T_.as<double>();
      v.n_t = n_t_;
      v.okey = okey_.as<int>();
      v.oof = oof_.as<int>();
      v.nkeys = nkeys_;
      v.vol = b.L * b.L * b.L;
      v.rho = b.A / v.vol;
      const bool snm = b.tzmin != b.tzmax;
      const double pi = 3.14159265358979323846;
      v.kF = std::cbrt(3.0 * pi * pi * v.rho / (snm ? 2.0 : 1.0));
      v.eF = (197.3269788 * v.kF) * (197.3269788 * v.kF) / (2.0 * 939.565);
      if (b.ns > 0) {
        v.theta[0] = b.kx[0] * b.L - 2.0 * pi * b.nx[0];
        v.theta[1] = b.ky[0] * b.L - 2.0 * pi * b.ny[0];
        v.theta[2] = b.kz[0] * b.L - 2.0 * pi * b.nz[0];
      }
      v.st = st_;
      return true;
    }
  }
  void mark_t_set() override { have_t_ = true; }

  void require_ready() {
    if (!have_fock_) throw EngineError(4, "no Fock matrix / interaction set");
    if (!have_t_) throw EngineError(4, "no T2 amplitudes (call setup_t_amplitudes or set_t2)");
    commit();
  }
  void commit() {
    if (!dirty_ && vph_ready_) return;
    launch_build_vph<S>(D_, Vhp_.as<S>(), Vph_.as<S>(), st_);
    ++launches_;
    if (!w_generated_) {
      launch_build_w<S>(D_, hp4_slot_.as<int2>(), v4_off_.as<int64_t>(), n4_.as<int>(), v4_.as<double>(), W_.as<S>(),
                        flag_.as<int>(), st_);
      ++launches_;
      check_flag("V_hphp has a non-zero imaginary part but the engine is real");
    }
    dirty_ = false;
    vph_ready_ = true;
  }

  // Device bytes of the resident state (amplitudes, residual, interaction blocks, ring
  // blocks, per-amplitude maps and pair slots), from the layout alone.  A layout that
  // does not fit in the device's free memory is rejected with CCX_ENOMEM before the
  // engine allocates anything.
  void check_memory_plan() const {
    const Layout &L = *L_;
    const int64_t ns = L.b.ns, A = L.b.A, NP = ns - A;
    int64_t vpp = 0, hh2 = 0, ph = 0, i4 = 0;
    for (int c = 0; c < L.fam[3].count(); ++c) {
      vpp += (int64_t)L.pk[c].P * L.pk[c].P;
      hh2 += (int64_t)L.pk[c].H * L.pk[c].H;
    }
    for (int q = 0; q < L.ph[1].count(); ++q) {
      const int64_t a = L.ph[1].side1[q].size(), b = L.ph[1].side2[q].size();
      ph += a * b;
      i4 += b * b;
    }
    const double need = (double)sizeof(S) * (3.0 * L.n_tpacked + vpp + 3.0 * hh2 + 3.0 * ph + 2.0 * i4) +
                        2.0 * 16.0 * L.n_tpacked + 8.0 * (NP * NP + A * A);
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    if (need > (double)free_b) {
      char msg[256];
      std::snprintf(msg, sizeof msg,
                    "layout needs %.1f GB of device memory for its resident state (V_pppp' alone %.1f GB); "
                    "the device has %.1f GB free",
                    need / 1e9, (double)sizeof(S) * vpp / 1e9, (double)free_b / 1e9);
      throw EngineError(3, msg);
    }
  }

  void build_tables() {
    const Layout &L = *L_;
    const int ns = L.b.ns, A = L.b.A, NP = ns - A;
    const int nc = L.fam[3].count();
    std::vector<int> P(nc), H(nc), pp_off(nc), hh_off(nc);
    std::vector<int64_t> t_off(nc), vpp_off(nc), hh2_off(nc);
    std::vector<int2> pp_orb, hh_orb, ttile, vtile;
    std::vector<int> pp_row, hh_row, pp_sgn, hh_sgn;
    int64_t vacc = 0, hacc = 0;
    hhhh_to_hhpp_.assign(L.fam[1].count(), -1);
    for (int c = 0; c < nc; ++c) {
      const PackedChannel &pk = L.pk[c];
      P[c] = pk.P;
      H[c] = pk.H;
      t_off[c] = pk.t_off;
      vpp_off[c] = vacc;
      hh2_off[c] = hacc;
      vacc += (int64_t)pk.P * pk.P;
      hacc += (int64_t)pk.H * pk.H;
      pp_off[c] = (int)pp_orb.size();
      hh_off[c] = (int)hh_orb.size();
      const PairList &pl = L.fam[3].side2[c], &hl = L.fam[3].side1[c];
      for (int r : pk.pp_of_packed) { pp_orb.push_back(make_int2(pl.p[r], pl.q[r])); pp_row.push_back(r); }
      for (int r : pk.hh_of_packed) { hh_orb.push_back(make_int2(hl.p[r], hl.q[r])); hh_row.push_back(r); }
      ppsgn_off_.push_back((int64_t)pp_sgn.size());
      hhsgn_off_.push_back((int64_t)hh_sgn.size());
      pp_sgn.insert(pp_sgn.end(), pk.pp_packed.begin(), pk.pp_packed.end());
      hh_sgn.insert(hh_sgn.end(), pk.hh_packed.begin(), pk.hh_packed.end());
      for (int64_t s = 0; s < (int64_t)pk.P * pk.H; s += kTileElems) ttile.push_back(make_int2(c, (int)s));
      for (int64_t s = 0; s < (int64_t)pk.P * pk.P; s += kTileElems) vtile.push_back(make_int2(c, (int)s));
      if (pk.hhhh >= 0) hhhh_to_hhpp_[pk.hhhh] = c;
      max_stage_ = std::max<int64_t>(max_stage_, (int64_t)pk.n_pp * std::max(pk.n_pp, pk.n_hh));
    }
    n_t_ = L.n_tpacked;
    n_vpp_ = vacc;
    n_hh2_ = hacc;
    // slots
    std::vector<int2> pp_slot((size_t)NP * NP, make_int2(-1, 0)), hh_slot((size_t)A * A, make_int2(-1, 0));
    for (int a = A; a < ns; ++a)
      for (int b = A; b < ns; ++b) {
        const int pos = L.pp_hhpp[(size_t)a * ns + b];
        if (!pos) continue;
        const int c = L.chan3_of_pair(a, b);
        pp_slot[(size_t)(a - A) * NP + (b - A)] = make_int2(c, L.pk[c].pp_packed[pos - 1]);
      }
    for (int i = 0; i < A; ++i)
      for (int j = 0; j < A; ++j) {
        const int pos = L.hh_hhpp[(size_t)i * ns + j];
        if (!pos) continue;
        const int c = L.chan3_of_pair(i, j);
        hh_slot[(size_t)i * A + j] = make_int2(c, L.pk[c].hh_packed[pos - 1]);
      }
    partner_.assign(ns, -1);
    for (int p = 0; p < ns; ++p) partner_[p] = L.b.orbitof(L.b.nx[p], L.b.ny[p], L.b.nz[p], -L.b.sz[p], L.b.tz[p]);
    // ring channels
    const int nq = L.ph[1].count();
    std::vector<int> nph(nq), nhp(nq), ph_off(nq), hp_off(nq);
    std::vector<int64_t> tph_off(nq), i4_off(nq), vph_off(nq);
    std::vector<int2> ph_orb, hp_orb, phtile;
    int64_t tacc = 0, iacc = 0;
    for (int q = 0; q < nq; ++q) {
      const PairList &s1 = L.ph[1].side1[q], &s2 = L.ph[1].side2[q];
      nph[q] = s1.size();
      nhp[q] = s2.size();
      tph_off[q] = tacc;
      vph_off[q] = tacc;
      i4_off[q] = iacc;
      tacc += (int64_t)nph[q] * nhp[q];
      iacc += (int64_t)nhp[q] * nhp[q];
      ph_off[q] = (int)ph_orb.size();
      hp_off[q] = (int)hp_orb.size();
      for (int r = 0; r < s1.size(); ++r) ph_orb.push_back(make_int2(s1.p[r], s1.q[r]));
      for (int r = 0; r < s2.size(); ++r) hp_orb.push_back(make_int2(s2.p[r], s2.q[r]));
      for (int64_t s = 0; s < (int64_t)nph[q] * nhp[q]; s += kTileElems) phtile.push_back(make_int2(q, (int)s));
    }
    n_ph_ = tacc;
    n_i4_ = iacc;
    std::vector<int2> ph_slot((size_t)NP * A, make_int2(-1, 0)), hp_slot((size_t)A * NP, make_int2(-1, 0));
    for (int a = A; a < ns; ++a)
      for (int i = 0; i < A; ++i) {
        const int pos = L.ph_ph_phhp[(size_t)a * ns + i];
        if (!pos) continue;
        const int q = L.phgrid[1].get((L.b.tz[a] - L.b.tz[i]) / 2, L.b.nx[a] - L.b.nx[i], L.b.ny[a] - L.b.ny[i],
                                      L.b.nz[a] - L.b.nz[i]) - 1;
        ph_slot[(size_t)(a - A) * A + i] = make_int2(q, pos - 1);
      }
    for (int j = 0; j < A; ++j)
      for (int b = A; b < ns; ++b) {
        const int pos = L.hp_ph_phhp[(size_t)j * ns + b];
        if (!pos) continue;
        const int q = L.phgrid[1].get((L.b.tz[j] - L.b.tz[b]) / 2, L.b.nx[j] - L.b.nx[b], L.b.ny[j] - L.b.ny[b],
                                      L.b.nz[j] - L.b.nz[b]) - 1;
        hp_slot[(size_t)j * NP + (b - A)] = make_int2(q, pos - 1);
      }
    // kind-4 (hphp pair-sum) blocks for W
    const int n4c = L.fam[4].count();
    std::vector<int> n4(std::max(n4c, 1));
    std::vector<int2> hp4_slot((size_t)A * NP, make_int2(-1, 0));
    int64_t v4acc = 0;
    v4_off_h_.resize(std::max(n4c, 1));
    for (int c = 0; c < n4c; ++c) {
      n4[c] = L.fam[4].side1[c].size();
      v4_off_h_[c] = v4acc;
      v4acc += (int64_t)n4[c] * n4[c];
      const PairList &pl = L.fam[4].side1[c];
      for (int r = 0; r < pl.size(); ++r) hp4_slot[(size_t)pl.p[r] * NP + (pl.q[r] - A)] = make_int2(c, r);
    }
    // uploads
    upload(dP_, P, &bytes_); upload(dH_, H, &bytes_);
    upload(dt_off_, t_off, &bytes_); upload(dvpp_off_, vpp_off, &bytes_); upload(dhh2_off_, hh2_off, &bytes_);
    upload(dpp_off_, pp_off, &bytes_); upload(dhh_off_, hh_off, &bytes_);
    upload(dpp_orb_, pp_orb, &bytes_); upload(dhh_orb_, hh_orb, &bytes_);
    npp_total_ = (int)pp_orb.size();
    nhh_total_ = (int)hh_orb.size();
    {  // orbitals by quantum numbers (the learned start's prior maps lattices through them)
      const Basis &B = L.b;
      std::vector<int> okey(std::max(B.ns, 1), -1);
      for (size_t k = 0; k < B.orbit_of.size(); ++k)
        if (B.orbit_of[k] >= 0) okey[B.orbit_of[k]] = (int)k;
      upload(okey_, okey, &bytes_);
      upload(oof_, B.orbit_of, &bytes_);
      nkeys_ = (int)B.orbit_of.size();
    }
    upload(dpp_row_, pp_row, &bytes_); upload(dhh_row_, hh_row, &bytes_);
    upload(dpp_slot_, pp_slot, &bytes_); upload(dhh_slot_, hh_slot, &bytes_);
    upload(dpartner_, partner_, &bytes_);
    upload(dn_ph_, nph, &bytes_); upload(dn_hp_, nhp, &bytes_);
    upload(dtph_off_, tph_off, &bytes_); upload(di4_off_, i4_off, &bytes_); upload(dvph_off_, vph_off, &bytes_);
    upload(dph_off_, ph_off, &bytes_); upload(dhp_off_, hp_off, &bytes_);
    upload(dph_orb_, ph_orb, &bytes_); upload(dhp_orb_, hp_orb, &bytes_);
    upload(dph_slot_, ph_slot, &bytes_); upload(dhp_slot_, hp_slot, &bytes_);
    upload(dttile_, ttile, &bytes_); upload(dphtile_, phtile, &bytes_); upload(dvtile_, vtile, &bytes_);
    upload(pp_sgn_, pp_sgn, &bytes_); upload(hh_sgn_, hh_sgn, &bytes_);
    upload(n4_, n4, &bytes_); upload(hp4_slot_, hp4_slot, &bytes_);
    std::vector<int64_t> v4off(v4_off_h_.begin(), v4_off_h_.end());
    upload(v4_off_, v4off, &bytes_);
    v4_.alloc((size_t)std::max<int64_t>(v4acc, 1) * 2 * sizeof(double), &bytes_);
    CK(cudaMemset(v4_.p, 0, v4_.bytes));
    // orbits
    upload(onx_, L.b.nx, &bytes_); upload(ony_, L.b.ny, &bytes_); upload(onz_, L.b.nz, &bytes_);
    upload(osz_, L.b.sz, &bytes_); upload(otz_, L.b.tz, &bytes_);
    upload(okx_, L.b.kx, &bytes_); upload(oky_, L.b.ky, &bytes_); upload(okz_, L.b.kz, &bytes_);
    upload(oe_, L.b.e, &bytes_);
    O_.ns = ns;
    O_.nx = onx_.as<int>(); O_.ny = ony_.as<int>(); O_.nz = onz_.as<int>();
    O_.sz = osz_.as<int>(); O_.tz = otz_.as<int>();
    O_.kx = okx_.as<double>(); O_.ky = oky_.as<double>(); O_.kz = okz_.as<double>(); O_.e = oe_.as<double>();
    O_.volume = L.b.L * L.b.L * L.b.L;

    DevLayout &D = D_;
    D.ns = ns; D.A = A; D.NP = NP; D.nch = nc;
    D.P = dP_.as<int>(); D.H = dH_.as<int>();
    D.t_off = dt_off_.as<int64_t>(); D.vpp_off = dvpp_off_.as<int64_t>(); D.hh2_off = dhh2_off_.as<int64_t>();
    D.pp_off = dpp_off_.as<int>(); D.hh_off = dhh_off_.as<int>();
    D.pp_orb = dpp_orb_.as<int2>(); D.hh_orb = dhh_orb_.as<int2>();
    D.pp_row = dpp_row_.as<int>(); D.hh_row = dhh_row_.as<int>();
    D.pp_slot = dpp_slot_.as<int2>(); D.hh_slot = dhh_slot_.as<int2>();
    D.partner = dpartner_.as<int>();
    D.nph = nq;
    D.n_ph = dn_ph_.as<int>(); D.n_hp = dn_hp_.as<int>();
    D.tph_off = dtph_off_.as<int64_t>(); D.i4_off = di4_off_.as<int64_t>(); D.vph_off = dvph_off_.as<int64_t>();
    D.ph_off = dph_off_.as<int>(); D.hp_off = dhp_off_.as<int>();
    D.ph_orb = dph_orb_.as<int2>(); D.hp_orb = dhp_orb_.as<int2>();
    D.ph_slot = dph_slot_.as<int2>(); D.hp_slot = dhp_slot_.as<int2>();
    D.ttile = dttile_.as<int2>(); D.nttile = (int)ttile.size();
    D.phtile = dphtile_.as<int2>(); D.nphtile = (int)phtile.size();
    D.vtile = dvtile_.as<int2>(); D.nvtile = (int)vtile.size();
    n_ttile_ = D.nttile;
  }

  void alloc_state() {
    const Layout &L = *L_;
    const int ns = L.b.ns, A = L.b.A, NP = ns - A;
    const size_t s = sizeof(S);
    T_.alloc(std::max<int64_t>(n_t_, 1) * s, &bytes_);
    R_.alloc(std::max<int64_t>(n_t_, 1) * s, &bytes_);
    Vhp_.alloc(std::max<int64_t>(n_t_, 1) * s, &bytes_);
    Vpp_.alloc(std::max<int64_t>(n_vpp_, 1) * s, &bytes_);
    Vhh_.alloc(std::max<int64_t>(n_hh2_, 1) * s, &bytes_);
    X_.alloc(std::max<int64_t>(n_hh2_, 1) * s, &bytes_);
    I9_.alloc(std::max<int64_t>(n_hh2_, 1) * s, &bytes_);
    Tph_.alloc(std::max<int64_t>(n_ph_, 1) * s, &bytes_);
    Rph_.alloc(std::max<int64_t>(n_ph_, 1) * s, &bytes_);
    Vph_.alloc(std::max<int64_t>(n_ph_, 1) * s, &bytes_);
    W_.alloc(std::max<int64_t>(n_i4_, 1) * s, &bytes_);
    I4_.alloc(std::max<int64_t>(n_i4_, 1) * s, &bytes_);
    fdiag_.alloc(ns * s, &bytes_);
    f6_.alloc(std::max(NP, 1) * s, &bytes_);
    f7_.alloc(std::max(A, 1) * s, &bytes_);
    d2ij_.alloc(std::max(A, 1) * s, &bytes_);
    d2ab_.alloc(std::max(NP, 1) * s, &bytes_);
    i6off_.alloc(std::max(NP, 1) * s, &bytes_);
    i7off_.alloc(std::max(A, 1) * s, &bytes_);
    for (DBuf *b : {&T_, &R_, &Vhp_, &Vpp_, &Vhh_, &X_, &I9_, &Tph_, &Rph_, &Vph_, &W_, &I4_, &fdiag_, &f6_, &f7_, &d2ij_,
                    &d2ab_, &i6off_, &i7off_})
      CK(cudaMemset(b->p, 0, b->bytes));
    const size_t npart = std::max<size_t>({(size_t)n_ttile_ * 3, (size_t)608 * 32, 64});
    partial_.alloc(npart * sizeof(double), &bytes_);
    res_.alloc(64 * sizeof(double), &bytes_);
    flag_.alloc(sizeof(int), &bytes_);
    CK(cudaMemset(flag_.p, 0, sizeof(int)));
    stage_.alloc((size_t)std::max<int64_t>(max_stage_, 1) * 2 * sizeof(double), &bytes_);
    CK(cudaMallocHost(&host_res_, 64 * sizeof(double)));
    build_gemm_plans();
  }

  // A grouped GEMM launch plan: problems, tile lists per tile shape, split-K problems.
  struct Plan {
    DBuf probs, tiles[2], splits;
    int ntiles[2] = {0, 0}, nsplit = 0;
  };
  // N buckets of the tile-shape choice: N <= 16, <= 32, <= 64, > 64
  static int n_bucket(int N) { return N <= 16 ? 0 : N <= 32 ? 1 : N <= 64 ? 2 : 3; }
  struct PlanBuilder {
    const int *shape_of = nullptr;  // tile shape per N bucket
    int only_bucket = -1;           // >= 0: keep only the problems of this bucket
    std::vector<GemmProb<S>> probs;
    std::vector<GemmTile> tiles[2];
    std::vector<int> splits;
    std::vector<int64_t> work;
    void add(GemmProb<S> p, int64_t w) {
      if (only_bucket >= 0 && n_bucket(p.N) != only_bucket) return;
      const int shape = shape_of ? shape_of[n_bucket(p.N)] : (p.N <= 32 ? kShape128x32 : kShape64x64);
      const int bm = gemm_bm(shape), bn = gemm_bn(shape);
      const int id = (int)probs.size();
      const int nsl = p.kchunk > 0 ? (p.seg[0].K + p.kchunk - 1) / p.kchunk : 1;
      for (int ks = 0; ks < nsl; ++ks)
        for (int m0 = 0; m0 < p.M; m0 += bm)
          for (int n0 = 0; n0 < p.N; n0 += bn) tiles[shape].push_back(GemmTile{id, m0, n0, ks});
      if (p.kchunk > 0) splits.push_back(id);
      probs.push_back(p);
      work.push_back(p.kchunk > 0 ? w / nsl : w);
    }
  };
  void finalize_plan(Plan &pl, PlanBuilder &b) {
    // largest problems first for load balance across the SMs
    for (int sh = 0; sh < 2; ++sh) {
      std::stable_sort(b.tiles[sh].begin(), b.tiles[sh].end(),
                       [&](const GemmTile &x, const GemmTile &y) { return b.work[x.prob] > b.work[y.prob]; });
      upload(pl.tiles[sh], b.tiles[sh], &bytes_);
      pl.ntiles[sh] = (int)b.tiles[sh].size();
    }
    upload(pl.probs, b.probs, &bytes_);
    upload(pl.splits, b.splits, &bytes_);
    pl.nsplit = (int)b.splits.size();
  }
  void run_plan(const Plan &pl, cudaStream_t s = nullptr) {
    if (!s) s = st_;
    const GemmProb<S> *pr = (const GemmProb<S> *)pl.probs.p;
    for (int sh = 0; sh < 2; ++sh)
      if (pl.ntiles[sh]) {
        launch_gemm<S>(sh, pr, (const GemmTile *)pl.tiles[sh].p, pl.ntiles[sh], s);
        ++launches_;
      }
    if (pl.nsplit) {
      launch_splitk_reduce<S>(pr, (const int *)pl.splits.p, pl.nsplit, s);
      ++launches_;
    }
  }
  void run_x(cudaStream_t s = nullptr) {
    launch_xdot<S>(D_, (const int4 *)xwork_.p, nxwork_, (const int4 *)xgroups_.p, nxgroups_, Vhp_.as<S>(), T_.as<S>(),
                   xpart_.as<S>(), X_.as<S>(), s ? s : st_);
    launches_ += 2;
  }
  void build_gemm_plans() {
    const Layout &L = *L_;
    const int nc = L.fam[3].count();
    {  // I6 row tiles and the per-row dot buffer
      std::vector<int2> rt;
      for (int c = 0; c < nc; ++c)
        for (int r0 = 0; r0 < L.pk[c].P; r0 += kI6Rows)
          if (L.pk[c].H > 0) rt.push_back(make_int2(c, r0));
      upload(i6rows_, rt, &bytes_);
      ni6rows_ = (int)rt.size();
      i6dots_.alloc((size_t)std::max<int64_t>(3 * n_t_, 1) * sizeof(S), &bytes_);
    }
    {  // X = V_hhpp' T'  (H x H, K = P): column-dot items of at most kXSlice K each,
       // longest first; their partial tiles are summed per X tile in slice order
      std::vector<int4> w, gr;
      std::vector<int> klen;
      int slot = 0;
      for (int c = 0; c < nc; ++c) {
        const auto &pk = L.pk[c];
        if (pk.H <= 0 || pk.P <= 0) continue;
        const int nsl = (pk.P + kXSlice - 1) / kXSlice;
        for (int m0 = 0; m0 < pk.H; m0 += kXM)
          for (int j0 = 0; j0 < pk.H; j0 += kXJ) {
            gr.push_back(make_int4(c, m0 | (j0 << 16), slot, nsl));
            for (int ks = 0; ks < nsl; ++ks) {
              w.push_back(make_int4(c, m0 | (j0 << 16), ks, slot++));
              klen.push_back(std::min(pk.P, (ks + 1) * kXSlice) - ks * kXSlice);
            }
          }
      }
      std::vector<int> ord(w.size());
      for (size_t i = 0; i < ord.size(); ++i) ord[i] = (int)i;
      std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return klen[x] > klen[y]; });
      std::vector<int4> ws(w.size());
      for (size_t i = 0; i < ord.size(); ++i) ws[i] = w[ord[i]];
      upload(xwork_, ws, &bytes_);
      upload(xgroups_, gr, &bytes_);
      nxwork_ = (int)ws.size();
      nxgroups_ = (int)gr.size();
      xpart_.alloc((size_t)std::max(slot, 1) * kXM * kXJ * sizeof(S), &bytes_);
    }
    build_fp64_plans(planLadder_, planI4_, planRing_, -1, nullptr);
  }
  // The grouped FP64 GEMM plans of the residual; bucket >= 0 keeps only the problems of
  // that N bucket, shapes overrides the engine's tile shape per bucket.
  void build_fp64_plans(Plan &ladder, Plan &i4, Plan &ring, int bucket, const int *shapes) {
    ++plan_epoch_;
    const Layout &L = *L_;
    const int nc = L.fam[3].count();
    {  // R' += V_pppp' T' + T' I9'
      PlanBuilder b;
      b.shape_of = shapes ? shapes : gemm_shape_;
      b.only_bucket = bucket;
      int64_t hoff = 0, voff = 0;
      for (int c = 0; c < nc; ++c) {
        const auto &pk = L.pk[c];
        if (pk.H > 0 && pk.P > 0) {
          GemmProb<S> p{};
          p.nseg = 2;
          p.M = pk.P; p.N = pk.H;
          p.seg[0] = GemmSeg<S>{Vpp_.as<S>() + voff, T_.as<S>() + pk.t_off, pk.P, 1, 1, pk.P, pk.P, 1.0};
          p.seg[1] = GemmSeg<S>{T_.as<S>() + pk.t_off, I9_.as<S>() + hoff, 1, pk.P, 1, pk.H, pk.H, 1.0};
          p.C = R_.as<S>() + pk.t_off; p.C0 = nullptr; p.sCm = 1; p.sCn = pk.P; p.accumulate = 1;
          b.add(p, (int64_t)pk.P * pk.H * (pk.P + pk.H));
        }
        hoff += (int64_t)pk.H * pk.H;
        voff += (int64_t)pk.P * pk.P;
      }
      finalize_plan(ladder, b);
    }
    {  // I4 = W + 1/2 V_ph T_ph ; R_ph = T_ph I4
      PlanBuilder b4, br;
      b4.shape_of = br.shape_of = shapes ? shapes : gemm_shape_;
      b4.only_bucket = br.only_bucket = bucket;
      int64_t toff = 0, ioff = 0;
      for (int q = 0; q < L.ph[1].count(); ++q) {
        const int nph = L.ph[1].side1[q].size(), nhp = L.ph[1].side2[q].size();
        if (nph > 0 && nhp > 0) {
          GemmProb<S> a{};
          a.nseg = 1;
          a.M = nhp; a.N = nhp;
          a.seg[0] = GemmSeg<S>{Vph_.as<S>() + toff, Tph_.as<S>() + toff, 1, nhp, 1, nph, nph, 0.5};
          a.C = I4_.as<S>() + ioff; a.C0 = W_.as<S>() + ioff; a.sCm = 1; a.sCn = nhp; a.accumulate = 0;
          b4.add(a, (int64_t)nhp * nhp * nph);
          GemmProb<S> r{};
          r.nseg = 1;
          r.M = nph; r.N = nhp;
          r.seg[0] = GemmSeg<S>{Tph_.as<S>() + toff, I4_.as<S>() + ioff, 1, nph, 1, nhp, nhp, 1.0};
          r.C = Rph_.as<S>() + toff; r.C0 = nullptr; r.sCm = 1; r.sCn = nph; r.accumulate = 0;
          br.add(r, (int64_t)nph * nhp * nhp);
        }
        toff += (int64_t)nph * nhp;
        ioff += (int64_t)nhp * nhp;
      }
      finalize_plan(i4, b4);
      finalize_plan(ring, br);
    }
  }

  // Autotuner of the grouped FP64 GEMM: for each N bucket, time the residual's ladder,
  // I4 and ring problems of that bucket with each tile shape (best of 3 launches, CUDA
  // events on the engine stream), keep the faster shape and rebuild every plan.  The
  // timed launches only write buffers that each residual evaluation rewrites.
  void autotune(int shapes[4], double ms[8]) override {
    require_ready();
    EventPair ev;
    const int64_t held = bytes_;  // the trial plans are freed again below
    for (int k = 0; k < 4; ++k) {
      double best = 1e300;
      int pick = gemm_shape_[k];
      for (int sh = 0; sh < 2; ++sh) {
        const int tab[4] = {sh, sh, sh, sh};
        Plan pl, p4, pr;
        build_fp64_plans(pl, p4, pr, k, tab);
        double t = 0.0;
        for (const Plan *p : {&pl, &p4, &pr}) {
          float tbest = 1e30f;
          for (int rep = 0; rep < 3; ++rep) tbest = std::min(tbest, ev.time(st_, [&] { run_plan(*p); }));
          t += tbest;
        }
        ms[2 * k + sh] = t;
        if (t < best) { best = t; pick = sh; }
      }
      gemm_shape_[k] = pick;
      shapes[k] = pick;
    }
    bytes_ = held;
    build_fp64_plans(planLadder_, planI4_, planRing_, -1, nullptr);
    mixed_ready_ = false;  // the mixed residual's FP64 plans are rebuilt with the new shapes
    oz_ready_ = false;
  }

  // Launch form of each BF16x3 / TF32x3 correction product (pp + hh ladders, dI4 + dX,
  // ring): one launch per bucket of the column count, or one launch over all its tiles,
  // whichever runs the engine's own tiles faster (best of 3 each).  The products write
  // only what the next residual writes again first (R', dI4, dX, dR_ph).
  void autotune_tc(int precision, int merged[3], double ms[6]) override {
    require_ready();
    if (precision != 1 && precision != 2) throw EngineError(1, "tensor-core autotune needs a mixed precision");
    prepare_mixed(precision == 2 ? kTcTF32 : kTcBF16);
    EventPair ev;
    TcPlan *plans[3] = {&tcPP_, &tcI4_, &tcR1_};
    for (int p = 0; p < 3; ++p) {
      double t[2];
      for (int v = 0; v < 2; ++v) {
        plans[p]->merged[0] = plans[p]->merged[1] = v;
        float best = 1e30f;
        for (int rep = 0; rep < 3; ++rep) best = std::min(best, ev.time(st_, [&] { run_tc(*plans[p]); }));
        t[v] = best;
        ms[2 * p + v] = best;
      }
      const int pick = t[1] <= t[0] ? 1 : 0;
      plans[p]->merged[0] = plans[p]->merged[1] = pick;
      tc_choice_[p] = pick;
      merged[p] = pick;
    }
    int err = 0;
    CK(cudaMemcpyAsync(&err, tcerr_.p, sizeof(int), cudaMemcpyDeviceToHost, st_));
    CK(cudaStreamSynchronize(st_));
    if (err) {
      CK(cudaMemsetAsync(tcerr_.p, 0, sizeof(int), st_));
      throw EngineError(2, "tensor-core GEMM reported error code " + std::to_string(err) + " during the autotune");
    }
    ++plan_epoch_;  // the replayed residual graphs are captured again with the chosen launches
  }

  // ================================================================== iteration
  void mark(int i) {
    if (timing_) CK(cudaEventRecord(ev_[i], st_));
  }
  // The residual launch sequences replayed as CUDA graphs, one per kind (plain FP64,
  // FP64 re-base, digit re-base, mixed).  Their arguments are fixed device buffers and
  // plans; plan_epoch_ moves whenever a plan or buffer they use is rebuilt, and the
  // graph of that kind is captured again.  With the event timers on, launched directly.
  struct Replay {
    cudaGraphExec_t exec = nullptr;
    int64_t launches = 0, epoch = -1;
  };
  Replay replay_[4];
  int64_t plan_epoch_ = 0;
  template <class F>
  void replayed(int kind, F &&body) {
    if (timing_) {
      body();
      return;
    }
    Replay &r = replay_[kind];
    if (r.exec && r.epoch != plan_epoch_) {
      CK(cudaGraphExecDestroy(r.exec));
      r.exec = nullptr;
    }
    if (!r.exec) {
      const int64_t l0 = launches_;
      cudaGraph_t g = nullptr;
      CK(cudaStreamBeginCapture(st_, cudaStreamCaptureModeRelaxed));
      try {
        body();
      } catch (...) {
        cudaStreamEndCapture(st_, &g);
        if (g) cudaGraphDestroy(g);
        launches_ = l0;
        throw;
      }
      CK(cudaStreamEndCapture(st_, &g));
      const cudaError_t ie = cudaGraphInstantiate(&r.exec, g, 0);
      cudaGraphDestroy(g);
      CK(ie);
      r.launches = launches_ - l0;
      r.epoch = plan_epoch_;
      launches_ = l0;
    }
    CK(cudaGraphLaunch(r.exec, st_));
    launches_ += r.launches;
  }
  // X = V_hhpp'^T T' and what hangs on it (I9, I7, their splits) need only T: they go to
  // the side stream, forked at the start of a residual and joined before the R' pieces
  // that read them.  Serial on the main stream while the event timers are on.
  cudaStream_t fork_side() {
    if (timing_) return st_;
    CK(cudaEventRecord(xev_[0], st_));
    CK(cudaStreamWaitEvent(xs_, xev_[0], 0));
    return xs_;
  }
  void join_side(cudaStream_t xs, int ev = 1) {
    if (xs == st_) return;
    CK(cudaEventRecord(xev_[ev], xs));
    CK(cudaStreamWaitEvent(st_, xev_[ev], 0));
  }
  void residual(bool /*unused*/) {
    mark(0);
    launch_gather_tph<S>(D_, T_.as<S>(), Tph_.as<S>(), st_);
    mark(1);
    kbegin(kKX);
    run_x();
    kend();
    launch_i7<S>(D_, X_.as<S>(), fdiag_.as<S>(), f7_.as<S>(), d2ij_.as<S>(), i7off_.as<S>(), st_);
    launch_i9<S>(D_, n_hh2_, Vhh_.as<S>(), X_.as<S>(), I9_.as<S>(), st_);
    mark(2);
    launch_i6<S>(D_, (const int2 *)i6rows_.p, ni6rows_, i6dots_.as<S>(), T_.as<S>(), Vhp_.as<S>(), fdiag_.as<S>(),
                 f6_.as<S>(), d2ab_.as<S>(), i6off_.as<S>(), st_);
    mark(3);
    kbegin(kKI4);
    run_plan(planI4_);
    kend();
    mark(4);
    kbegin(kKRing);
    run_plan(planRing_);
    kend();
    mark(5);
    launch_rinit<S>(D_, omap_.as<int4>(), rmap_.as<int4>(), T_.as<S>(), Vhp_.as<S>(), Rph_.as<S>(), i6off_.as<S>(),
                    i7off_.as<S>(), nullptr, nullptr, R_.as<S>(), st_);
    mark(6);
    kbegin(kKLadder);
    run_plan(planLadder_);
    kend();
    mark(7);
    launches_ += 5;
    if (timing_) accumulate_timers(0, 7);
  }
  // Event pairs around individual launches (slots kK*), read back with the phase timers.
  void kbegin(int slot) {
    kcur_ = -1;
    if (!timing_ || kn_ >= kKernelEvents) return;
    CK(cudaEventRecord(kev_[2 * kn_], st_));
    kcur_ = slot;
  }
  void kend() {
    if (kcur_ < 0) return;
    CK(cudaEventRecord(kev_[2 * kn_ + 1], st_));
    kslot_[kn_++] = kcur_;
    kcur_ = -1;
  }
  void kflush() {
    for (int i = 0; i < kn_; ++i) {
      CK(cudaEventSynchronize(kev_[2 * i + 1]));
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, kev_[2 * i], kev_[2 * i + 1]));
      ktimers_[kslot_[i]] += ms;
      ++kcount_[kslot_[i]];
    }
    kn_ = 0;
  }
  void accumulate_timers(int first, int last) {
    kflush();
    CK(cudaEventSynchronize(ev_[last]));
    for (int i = first; i < last; ++i) {
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, ev_[i], ev_[i + 1]));
      timers_[i] += ms;
    }
  }
  // the per-iteration log: one record per residual, its term times the differences of
  // the running per-term timers since the previous record
  void log_begin() {
    ilog_.clear();
    for (int i = 0; i < 9; ++i) ilog_prev_[i] = timers_[i];
    ilog_t_ = std::chrono::steady_clock::now();
  }
  void log_record(int it, int kind, const double e[2], double de, double rn) {
    IterRecord rec;
    rec.iteration = it;
    rec.kind = kind;
    rec.e[0] = e[0];
    rec.e[1] = e[1];
    rec.de = de;
    rec.res_norm = rn;
    const auto t = std::chrono::steady_clock::now();
    rec.ms = std::chrono::duration<double, std::milli>(t - ilog_t_).count();
    ilog_t_ = t;
    for (int i = 0; i < 9; ++i) {
      rec.term_ms[i] = timers_[i] - ilog_prev_[i];
      ilog_prev_[i] = timers_[i];
    }
    ilog_.push_back(rec);
  }
  // the standard loop's DIIS extrapolation runs after its iteration's record
  void log_amend_diis() {
    if (ilog_.empty()) return;
    ilog_.back().term_ms[8] += timers_[8] - ilog_prev_[8];
    ilog_prev_[8] = timers_[8];
  }
  void fetch_res(int n) {
    CK(cudaMemcpyAsync(host_res_, res_.p, n * sizeof(double), cudaMemcpyDeviceToHost, st_));
    CK(cudaStreamSynchronize(st_));
    if (!std::isfinite(host_res_[0]) || !std::isfinite(host_res_[1]))
      throw EngineError(5, "non-finite energy: the iteration diverged or the input holds NaN/Inf");
  }

  // diis_t1t2 (ccm_diis.f90:74-249) on the packed vectors; the reference's column
  // shift of t2_diis is a rotation of the physical column ids here.
  void reference_update(int count) {
    if (nstep_ > subspace_) {
      nstep_ = subspace_;
      const int first = phys_[0];
      for (int i = 0; i < subspace_ - 1; ++i) phys_[i] = phys_[i + 1];
      phys_[subspace_ - 1] = first;
    }
    S *col = hist_.as<S>() + (int64_t)phys_[nstep_ - 1] * n_t_;
    mark(7);
    launch_update<S>(D_, 0, T_.as<S>(), R_.as<S>(), Vhp_.as<S>(), d2ij_.as<S>(), d2ab_.as<S>(), col, nullptr,
                     partial_.as<double>(), res_.as<double>(), st_);
    launches_ += 2;
    fetch_res(3);
    last_rn_ = 2.0 * std::sqrt(host_res_[2]);
    mark(8);
    if (timing_) accumulate_timers(7, 8);
    if (count != diis_step_) return;
    const int ns = nstep_;
    if (ns < 2) return;
    std::vector<const S *> cols(ns);
    for (int i = 0; i < ns; ++i) cols[i] = hist_.as<S>() + (int64_t)phys_[i] * n_t_;
    launch_diis_gram<S>(n_t_, cols.data(), ns, partial_.as<double>(), res_.as<double>(), st_);
    launches_ += 2;
    fetch_res(30);
    std::vector<std::complex<double>> B((size_t)ns * ns, 0.0), sol(ns, 0.0);
    const int nd = ns - 1;
    int k = 0;
    for (int i = 0; i < 5; ++i)
      for (int j = i; j < 5; ++j) {
        if (i < nd && j < nd) {
          // x4: the ordered vectors hold each packed amplitude four times
          const std::complex<double> v(4.0 * host_res_[2 * k], 4.0 * host_res_[2 * k + 1]);
          B[i + (size_t)ns * j] = v;
          B[j + (size_t)ns * i] = v;
        }
        ++k;
      }
    for (int i = 0; i < nd; ++i) { B[i + (size_t)ns * nd] = -1.0; B[nd + (size_t)ns * i] = -1.0; }
    B[nd + (size_t)ns * nd] = 0.0;
    sol[nd] = -1.0;
    // A singular system (the reference prints ZGESV's info and goes on with an undefined
    // solution, ccm_diis.f90:173-180) keeps the damped step already written to T.
    bool ok = zsolve(ns, B, sol);
    for (int i = 0; i < ns && ok; ++i) ok = std::isfinite(sol[i].real()) && std::isfinite(sol[i].imag());
    if (!ok) {
      ++diis_fallbacks_;
      mark(9);
      if (timing_) accumulate_timers(8, 9);
      return;
    }
    std::vector<double> coef(2 * nd);
    for (int i = 0; i < nd; ++i) { coef[2 * i] = sol[i].real(); coef[2 * i + 1] = ScalarOf<S>::complex ? sol[i].imag() : 0.0; }
    launch_combine<S>(n_t_, cols.data(), coef.data(), nd, T_.as<S>(), st_);
    ++launches_;
    mark(9);
    if (timing_) accumulate_timers(8, 9);
  }

  void iterate_reference(const IterOpts &o, IterResult &r) {
    log_begin();
    diis_setup(6, 6);
    int count = 0;
    std::complex<double> e1(r.e_mbpt2[0], r.e_mbpt2[1]), e2(0.0, 0.0), de(4.0, 0.0);
    int it = 0;
    for (it = 1; it <= o.max_iter; ++it) {
      if (!(std::abs(de) > o.tol)) break;
      residual(true);
      ++count;
      ++nstep_;
      reference_update(count);
      if (count == diis_step_) count = 0;
      r.res_norm = last_rn_;
      // energy of the updated (or extrapolated) amplitudes
      double e[2];
      energy(e);
      e2 = std::complex<double>(e[0], e[1]);
      de = e2 - e1;
      e1 = e2;
      r.iterations = it;
      log_record(it, 0, e, de.real(), r.res_norm);
      if (o.verbose) std::printf("ccx it %3d dE %.3e E %.12f |R| %.3e\n", it, de.real(), e2.real(), r.res_norm);
    }
    r.converged = !(std::abs(de) > o.tol);
    r.e_ccd[0] = e2.real();
    r.e_ccd[1] = e2.imag();
  }

  // Standard mode: Jacobi step + Pulay DIIS on the steps.  With mixed precision the
  // residual is evaluated as R(T_b) [cached, FP64] + tensor-core corrections in
  // T - T_b (defect correction); an FP64 residual re-bases T_b when the mixed residual
  // has dropped by rebase_drop (default kRebaseDrop) since the last FP64 one, stalls,
  // reaches the tolerance,
  // or every defect_period iterations, and only an FP64 residual can end the solve.
  //
  // The loop is a state machine so that a batch of engines can run it in lockstep:
  //   std_begin; repeat { std_launch_residual; std_launch_update; std_launch_dots; [sync]
  //   std_after_update (true: finished); std_after_dots }.  The DIIS Gram row needs no
  //   host decision, so the dots are queued behind the update and one synchronisation
  //   per iteration serves both.
  struct StdState {
    IterOpts o;
    IterResult *r = nullptr;
    bool mixed = false, need_fp64 = false, exact = false, done = false;
    int m = 8, nh = 0, head = 0, it = 0, stall = 0, since = 0;
    double e[2] = {0, 0}, phase_r0 = -1.0, best = 1e300;
    std::vector<double> B;
    S *ht = nullptr;
    E *he = nullptr;
  };
  StdState ss_;
  static constexpr double kRebaseDrop = 1e-4;

  void std_begin(const IterOpts &o, IterResult &r) override {
    require_ready();
    if (o.precision < 0 || o.precision > 2) throw EngineError(1, "unknown precision");
    if (o.rebase < 0 || o.rebase > 1) throw EngineError(1, "unknown re-base product kind");
    if (o.mode != 1) throw EngineError(1, "the batched iteration runs the standard (DIIS) mode");
    r = IterResult();
    double e0[2];
    energy(e0);
    r.e_mbpt2[0] = e0[0];
    r.e_mbpt2[1] = e0[1];
    StdState &s = ss_;
    s = StdState();
    s.o = o;
    s.r = &r;
    s.mixed = o.precision != 0;
    if (s.mixed) {
      prepare_mixed(o.precision == 2 ? kTcTF32 : kTcBF16);
      if (o.rebase == 1) prepare_oz();
      set_base_zero();
    }
    s.m = std::max(2, std::min(o.diis_dim, 15));
    hist_t_.alloc((size_t)s.m * n_t_ * sizeof(S), &bytes_);
    hist_e_.alloc((size_t)s.m * n_t_ * sizeof(E), &bytes_);
    s.B.assign((size_t)s.m * s.m, 0.0);
    s.e[0] = r.e_mbpt2[0];
    s.e[1] = r.e_mbpt2[1];
    s.done = o.max_iter < 1;
    log_begin();
  }
  // the one-time set-up a solve with these options needs (operand tiles, digit planes
  // of the interaction, DIIS history), without solving
  void prepare(const IterOpts &o) override {
    require_ready();
    if (o.precision < 0 || o.precision > 2) throw EngineError(1, "unknown precision");
    if (o.rebase < 0 || o.rebase > 1) throw EngineError(1, "unknown re-base product kind");
    if (o.precision != 0) {
      prepare_mixed(o.precision == 2 ? kTcTF32 : kTcBF16);
      if (o.rebase == 1) prepare_oz();
    }
    if (o.mode == 1) {
      const int m = std::max(2, std::min(o.diis_dim, 15));
      hist_t_.alloc((size_t)m * n_t_ * sizeof(S), &bytes_);
      hist_e_.alloc((size_t)m * n_t_ * sizeof(E), &bytes_);
    }
    CK(cudaStreamSynchronize(st_));
  }
  bool std_done() const override { return ss_.done; }
  void std_launch_residual() override {
    StdState &s = ss_;
    ++s.it;
    s.exact = !s.mixed || s.need_fp64;
    if (!s.mixed) replayed(0, [&] { residual(true); });
    else if (s.exact) {
      const bool digits = s.o.rebase == 1;
      replayed(digits ? 2 : 1, [&] { residual_fp64_rebase(digits); });
      ++s.r->fp64_sweeps;
    } else {
      replayed(3, [&] { residual_mixed(); });
      ++s.r->mixed_iterations;
    }
  }
  void std_launch_update() override {
    StdState &s = ss_;
    s.ht = hist_t_.as<S>() + (int64_t)s.head * n_t_;
    s.he = hist_e_.as<E>() + (int64_t)s.head * n_t_;
    mark(7);
    {  // the Gram row of the new step against every stored one rides on the same pass
      const int nh = std::min(s.nh + 1, s.m);
      if (nh > 16 || s.head >= nh) throw EngineError(1, "DIIS history larger than the fused Gram row");
      std::vector<const E *> es(nh);
      for (int j = 0; j < nh; ++j) es[j] = hist_e_.as<E>() + (int64_t)j * n_t_;
      launch_update_std<S>(D_, T_.as<S>(), R_.as<S>(), Vhp_.as<S>(), d2ij_.as<S>(), d2ab_.as<S>(), s.ht, s.he,
                           es.data(), nh, s.head, s.mixed ? tcerr_.as<int>() : nullptr, partial_.as<double>(),
                           res_.as<double>(), st_);
    }
    launches_ += 2;
    // energy, norm, tensor-core error word and Gram row come back in one copy
    CK(cudaMemcpyAsync(host_res_, res_.p, (4 + std::min(s.nh + 1, s.m)) * sizeof(double), cudaMemcpyDeviceToHost,
                       st_));
  }
  bool std_after_update() override {
    StdState &s = ss_;
    IterResult &r = *s.r;
    if (!std::isfinite(host_res_[0]) || !std::isfinite(host_res_[1]))
      throw EngineError(5, "non-finite energy: the iteration diverged or the input holds NaN/Inf");
    mark(8);
    if (timing_) accumulate_timers(7, 8);
    const double de = host_res_[0] - s.e[0];
    s.e[0] = host_res_[0];
    s.e[1] = host_res_[1];
    const double rn = 2.0 * std::sqrt(host_res_[2]);
    const int tc_word = (int)host_res_[3];
    if (s.mixed && tc_word) {
      const int err = tc_word;
      CK(cudaMemsetAsync(tcerr_.p, 0, sizeof(int), st_));
      throw EngineError(2, "tensor-core GEMM reported error code " + std::to_string(err));
    }
    if (s.exact) r.res_norm = rn;
    r.iterations = s.it - 1;
    r.e_ccd[0] = s.e[0];
    r.e_ccd[1] = s.e[1];
    log_record(s.it, s.exact ? 1 : 2, s.e, de, rn);
    if (s.o.verbose) std::printf("ccx it %3d %s |R| %.3e E %.12f\n", s.it, s.exact ? "fp64 " : "mixed", rn, s.e[0]);
    if (s.exact && rn < s.o.tol) {
      r.converged = 1;
      s.done = true;
      return true;
    }
    if (s.mixed) {
      if (s.exact) {
        s.need_fp64 = false;
        s.phase_r0 = rn;
        s.best = rn;
        s.stall = 0;
        s.since = 0;
      } else {
        ++s.since;
        if (s.phase_r0 < 0) s.phase_r0 = rn;
        if (rn < 0.9 * s.best) { s.best = rn; s.stall = 0; } else ++s.stall;
        const bool periodic = s.o.defect_period > 0 && s.since >= s.o.defect_period;
        const double drop = s.o.rebase_drop > 0.0 ? s.o.rebase_drop : kRebaseDrop;
        const bool dropped = s.o.defect_period <= 0 && rn < drop * s.phase_r0;
        if (rn < s.o.tol || s.stall >= 2 || periodic || dropped) s.need_fp64 = true;
      }
    }
    return false;
  }
  // the Gram row of the new step (Re of the conjugated products) is computed by the update
  // pass and copied with its sums: nothing to launch here
  void std_launch_dots() override {
    StdState &s = ss_;
    if (s.nh < s.m) ++s.nh;
  }
  void std_after_dots() override {
    StdState &s = ss_;
    const int m = s.m, nh = s.nh, slot = s.head;
    for (int j = 0; j < nh; ++j) {
      s.B[slot + (size_t)m * j] = host_res_[4 + j];
      s.B[j + (size_t)m * slot] = host_res_[4 + j];
    }
    s.head = (s.head + 1) % m;
    std::vector<double> coef;
    bool ok = false;
    if (nh >= 2) {
      const int n1 = nh + 1;
      std::vector<double> Bm((size_t)n1 * n1, 0.0), rhs(n1, 0.0);
      for (int i = 0; i < nh; ++i)
        for (int j = 0; j < nh; ++j) Bm[i + (size_t)n1 * j] = s.B[i + (size_t)m * j];
      for (int i = 0; i < nh; ++i) { Bm[i + (size_t)n1 * nh] = -1.0; Bm[nh + (size_t)n1 * i] = -1.0; }
      rhs[nh] = -1.0;
      ok = dsolve(n1, Bm, rhs);
      for (int i = 0; i < n1 && ok; ++i) ok = std::isfinite(rhs[i]);
      if (!ok) ++diis_fallbacks_;
      if (ok) {
        coef.resize(2 * nh);
        for (int i = 0; i < nh; ++i) { coef[2 * i] = rhs[i]; coef[2 * i + 1] = 0.0; }
      }
    }
    mark(8);
    if (ok) {
      std::vector<const S *> ts(nh);
      for (int j = 0; j < nh; ++j) ts[j] = hist_t_.as<S>() + (int64_t)j * n_t_;
      launch_combine<S>(n_t_, ts.data(), coef.data(), nh, T_.as<S>(), st_);
    } else {
      CK(cudaMemcpyAsync(T_.p, s.ht, n_t_ * sizeof(S), cudaMemcpyDeviceToDevice, st_));
    }
    ++launches_;
    mark(9);
    if (timing_) accumulate_timers(8, 9);
    log_amend_diis();
    s.r->iterations = s.it;
    if (s.it >= s.o.max_iter) s.done = true;
  }
  void sync() override { CK(cudaStreamSynchronize(st_)); }
  void set_timing(bool on) override { timing_ = on; }
  void set_profiling(bool on) override { profiling_ = on; }

  void iterate_standard(const IterOpts &o, IterResult &r) {
    std_begin(o, r);
    while (!ss_.done) {
      std_launch_residual();
      std_launch_update();
      std_launch_dots();  // needs no host decision: one synchronisation per iteration
      sync();
      if (std_after_update()) break;
      std_after_dots();
    }
  }

  // ================================================================== mixed precision
  // Tensor-core products on FP64 data of either scalar kind.  A real product is one
  // problem.  A complex product C += a A B becomes four real ones on the re / im parts
  // of the interleaved operands, in two launch phases so that no two CTAs update the
  // same C entries at once: phase 0 C_re += a Are Bre, C_im += a Are Bim; phase 1
  // C_re -= a Aim Bim, C_im += a Aim Bre.
  static constexpr int kNComp = ScalarOf<S>::complex ? 2 : 1;
  // Tiles bucketed by padded N, so that small problems run with small shared-memory
  // stages (and more CTAs per SM) instead of the largest problem's footprint.
  static constexpr int kTcBuckets = 4;
  // One product's tensor-core tiles, listed twice: per bucket of the column count (one
  // launch each, with as many shared-memory stages as the bucket's widest tile leaves)
  // and all together (one launch, stages for the widest tile of all).  merged picks the
  // launch form per phase: one launch by default; the tensor-core autotuner times both.
  struct TcPlan {
    DBuf probs;
    DBuf tiles[2][kTcBuckets], tiles_m[2];
    int ntiles[2][kTcBuckets] = {}, npad_max[2][kTcBuckets] = {}, max_nk[2][kTcBuckets] = {};
    int ntiles_m[2] = {0, 0}, npad_m[2] = {16, 16}, nk_m[2] = {1, 1};
    int merged[2] = {0, 0};
  };
  struct SplitPlan {
    DBuf jobs, chunks;
    int nchunks = 0;
  };
  struct TileBuf {
    DBuf hi, lo;
    int64_t n = 0;  // elements of one scalar component; the buffer holds kNComp of them
  };
  // problems, their launch phase and their row tiles, built on the host
  struct TcList {
    std::vector<TcProb> probs;
    std::vector<int> phase;
    std::vector<TcTile> tiles;
  };
  void finalize_tc(TcPlan &pl, const TcList &l, int choice = -1) {
    upload(pl.probs, l.probs, &bytes_);
    std::vector<TcTile> b[2][kTcBuckets], m[2];
    for (int ph = 0; ph < 2; ++ph)
      for (int k = 0; k < kTcBuckets; ++k) { pl.npad_max[ph][k] = 16; pl.max_nk[ph][k] = 1; }
    for (const TcTile &t : l.tiles) {
      const TcProb &p = l.probs[t.prob];
      const int ph = l.phase[t.prob];
      const int k = p.npad <= 32 ? 0 : p.npad <= 64 ? 1 : p.npad <= 128 ? 2 : 3;
      b[ph][k].push_back(t);
      m[ph].push_back(t);
      int nk = p.nk;
      for (int e = 0; e < p.next; ++e) nk += p.ext[e].nk;
      pl.npad_max[ph][k] = std::max(pl.npad_max[ph][k], p.npad);
      pl.max_nk[ph][k] = std::max(pl.max_nk[ph][k], nk);
    }
    // longest tiles first: the persistent CTAs take tiles in strides of the grid
    auto work = [&](const TcTile &t) {
      const TcProb &p = l.probs[t.prob];
      int nk = p.nk;
      for (int e = 0; e < p.next; ++e) nk += p.ext[e].nk;
      return nk;
    };
    auto by_work = [&](const TcTile &x, const TcTile &y) { return work(x) > work(y); };
    for (int ph = 0; ph < 2; ++ph) {
      int np = 16, nk = 1;
      for (int k = 0; k < kTcBuckets; ++k) {
        std::stable_sort(b[ph][k].begin(), b[ph][k].end(), by_work);
        upload(pl.tiles[ph][k], b[ph][k], &bytes_);
        pl.ntiles[ph][k] = (int)b[ph][k].size();
        if (!b[ph][k].empty()) { np = std::max(np, pl.npad_max[ph][k]); nk = std::max(nk, pl.max_nk[ph][k]); }
      }
      std::stable_sort(m[ph].begin(), m[ph].end(), by_work);
      upload(pl.tiles_m[ph], m[ph], &bytes_);
      pl.ntiles_m[ph] = (int)m[ph].size();
      pl.npad_m[ph] = np;
      pl.nk_m[ph] = nk;
      // one launch unless the autotuner found the bucket launches faster: the persistent
      // grid then has no tail per bucket, and on every lattice measured it won even where
      // the widest tile leaves the kernel only two shared-memory stages
      pl.merged[ph] = choice >= 0 ? choice : 1;
    }
  }
  void finalize_split(SplitPlan &pl, const std::vector<TcSplitJob> &jobs) {
    upload(pl.jobs, jobs, &bytes_);
    const std::vector<int4> ch = tc_split_chunks(jobs);
    upload(pl.chunks, ch, &bytes_);
    pl.nchunks = (int)ch.size();
  }
  void run_tc(const TcPlan &pl) {
    for (int ph = 0; ph < 2; ++ph) {
      if (pl.merged[ph]) {
        if (!pl.ntiles_m[ph]) continue;
        launch_tc_gemm(tc_kind_, (const TcProb *)pl.probs.p, (const TcTile *)pl.tiles_m[ph].p, pl.ntiles_m[ph],
                       pl.npad_m[ph], pl.nk_m[ph], tcerr_.as<int>(), st_);
        ++launches_;
        continue;
      }
      for (int k = 0; k < kTcBuckets; ++k) {
        if (!pl.ntiles[ph][k]) continue;
        launch_tc_gemm(tc_kind_, (const TcProb *)pl.probs.p, (const TcTile *)pl.tiles[ph][k].p, pl.ntiles[ph][k],
                       pl.npad_max[ph][k], pl.max_nk[ph][k], tcerr_.as<int>(), st_);
        ++launches_;
      }
    }
  }
  void run_split(const SplitPlan &pl, cudaStream_t s = nullptr) {
    if (!pl.nchunks) return;
    launch_tc_split(tc_kind_, (const TcSplitJob *)pl.jobs.p, (const int4 *)pl.chunks.p, pl.nchunks, s ? s : st_);
    ++launches_;
  }
  // split jobs of one matrix operand (element (r, k) at src[r sr + k sk] in S units,
  // minus sub when given), one per scalar component, into tile buffer b at offset off
  void add_split(std::vector<TcSplitJob> &js, const S *src, const S *sub, int64_t sr, int64_t sk, int rows, int cols,
                 int tile_rows, int rows_pad, TileBuf &b, int64_t off, int add = 0, TileBuf *b2 = nullptr,
                 int64_t off2 = 0) {
    const size_t es = tc_kind_ == kTcBF16 ? 2 : 4;
    const int tk = tc_tile_k(tc_kind_);
    for (int c = 0; c < kNComp; ++c) {
      TcSplitJob j{};
      j.src = (const double *)src + c;
      j.sub = sub ? (const double *)sub + c : nullptr;
      j.sr = sr * kNComp;
      j.sk = sk * kNComp;
      j.rows = rows; j.cols = cols; j.tile_rows = tile_rows; j.nk = (cols + tk - 1) / tk; j.rows_pad = rows_pad;
      j.add = add;
      if (add == 2) {  // src into b, src + sub into b2 (same geometry)
        j.hi2 = (char *)b2->hi.p + (off2 + c * b2->n) * es;
        j.lo2 = (char *)b2->lo.p + (off2 + c * b2->n) * es;
      }
      j.hi = (char *)b.hi.p + (off + c * b.n) * es;
      j.lo = (char *)b.lo.p + (off + c * b.n) * es;
      js.push_back(j);
    }
  }
  // Map and gather jobs filling tile region (b, off) from the packed split of T - T_b:
  // element (r, k) is packed entry ind ? ind[base + r sr + k sk] : base + r sr + k sk
  // (scalar elements), one job per scalar component
  void add_gather(std::vector<TcMapJob> &mj, std::vector<TcGatherJob> &gj, int64_t base, const int32_t *ind,
                  int64_t sr, int64_t sk, int rows, int cols, int tile_rows, int rows_pad, TileBuf &b, DBuf &map,
                  int64_t off) {
    const size_t es = tc_kind_ == kTcBF16 ? 2 : 4;
    const int tk = tc_tile_k(tc_kind_);
    for (int c = 0; c < kNComp; ++c) {
      TcMapJob m{};
      m.base = base; m.sr = sr; m.sk = sk;
      m.rows = rows; m.cols = cols; m.tile_rows = tile_rows; m.nk = (cols + tk - 1) / tk; m.rows_pad = rows_pad;
      m.ind = ind;
      m.map = map.as<int32_t>() + off + c * b.n;
      mj.push_back(m);
      TcGatherJob g{};
      g.map = m.map;
      g.phl = (const char *)phl_.p + (size_t)c * n_t_ * 2 * es;
      g.hi = (char *)b.hi.p + (off + c * b.n) * es;
      g.lo = (char *)b.lo.p + (off + c * b.n) * es;
      gj.push_back(g);
    }
  }
  // C (S units, strides sCm, sCn) += alpha A B with A (M x K) in tile buffer a at ao and
  // B (N x K) in b at bo.  N beyond one accumulator (256 columns) runs as column blocks
  // of at most 256 that step through the whole B operand's K tiles.
  void add_tc(TcList &l, TileBuf &a, int64_t ao, TileBuf &b, int64_t bo, int M, int N, int K, S *C, int64_t sCm,
              int64_t sCn, double alpha) {
    const size_t es = tc_kind_ == kTcBF16 ? 2 : 4;
    const int tk = tc_tile_k(tc_kind_);
    const int npad_all = (N + 15) / 16 * 16;
    auto one = [&](int ca, int cb, int cc, double al, int ph) {
      for (int n0 = 0; n0 < N; n0 += 256) {
        const int nb = std::min(256, N - n0);
        TcProb p{};
        p.Ahi = (char *)a.hi.p + (ao + ca * a.n) * es;
        p.Alo = (char *)a.lo.p + (ao + ca * a.n) * es;
        p.Bhi = (char *)b.hi.p + (bo + cb * b.n) * es + (size_t)n0 * 128;
        p.Blo = (char *)b.lo.p + (bo + cb * b.n) * es + (size_t)n0 * 128;
        p.M = M; p.N = nb; p.nk = (K + tk - 1) / tk; p.npad = (nb + 15) / 16 * 16;
        p.bstride = npad_all > 256 ? (int64_t)npad_all * 128 : 0;
        p.C = (double *)C + cc + (int64_t)n0 * sCn * kNComp; p.sCm = sCm * kNComp; p.sCn = sCn * kNComp; p.alpha = al;
        for (int mt = 0; mt < (M + 127) / 128; ++mt) l.tiles.push_back(TcTile{(int)l.probs.size(), mt});
        l.probs.push_back(p);
        l.phase.push_back(ph);
      }
    };
    if (kNComp == 1) {
      one(0, 0, 0, alpha, 0);
    } else {
      one(0, 0, 0, alpha, 0);
      one(0, 1, 1, alpha, 0);
      one(1, 1, 0, -alpha, 1);
      one(1, 0, 1, alpha, 1);
    }
  }
  // Up to three products accumulated into one output tile and written once:
  // C = (overwrite ? 0 : C) + C0 + alpha sum_op A_op B_op, every op with the same M, N.
  struct TcOp {
    TileBuf *a;
    int64_t ao;
    TileBuf *b;
    int64_t bo;
    int K;
  };
  void add_tc_multi(TcList &l, const std::vector<TcOp> &ops, int M, int N, S *C, int64_t sCm, int64_t sCn, double alpha,
                    const S *C0, int overwrite) {
    const size_t es = tc_kind_ == kTcBF16 ? 2 : 4;
    const int tk = tc_tile_k(tc_kind_);
    const int npad_all = (N + 15) / 16 * 16;
    // One problem per output component cc, summing the products of every op with operand
    // components (ca, cb) listed in parts (neg: subtracted).  A complex product is
    // Re = Ar Br - Ai Bi and Im = Ar Bi + Ai Br: both outputs in one launch, each C
    // element read and written once.
    struct Part { int ca, cb, neg; };
    auto one = [&](int cc, std::initializer_list<Part> parts) {
      for (int n0 = 0; n0 < N; n0 += 256) {
        const int nb = std::min(256, N - n0);
        TcProb p{};
        int q = 0;
        for (const Part &pt : parts)
          for (const TcOp &o : ops) {
            TcSeg g{};
            g.Ahi = (char *)o.a->hi.p + (o.ao + pt.ca * o.a->n) * es;
            g.Alo = (char *)o.a->lo.p + (o.ao + pt.ca * o.a->n) * es;
            g.Bhi = (char *)o.b->hi.p + (o.bo + pt.cb * o.b->n) * es + (size_t)n0 * 128;
            g.Blo = (char *)o.b->lo.p + (o.bo + pt.cb * o.b->n) * es + (size_t)n0 * 128;
            g.nk = (o.K + tk - 1) / tk;
            g.bstride = npad_all > 256 ? (int64_t)npad_all * 128 : 0;
            g.neg = pt.neg;
            if (q == 0) {
              if (g.neg) throw EngineError(2, "the first product of a tensor-core problem cannot be subtracted");
              p.Ahi = g.Ahi; p.Alo = g.Alo; p.Bhi = g.Bhi; p.Blo = g.Blo; p.nk = g.nk; p.bstride = g.bstride;
            } else {
              if (q >= kTcMaxSegs) throw EngineError(2, "too many products for one tensor-core problem");
              p.ext[q - 1] = g;
            }
            ++q;
          }
        p.next = q - 1;
        p.M = M; p.N = nb; p.npad = (nb + 15) / 16 * 16;
        const int64_t coff = cc + (int64_t)n0 * sCn * kNComp;
        p.C = (double *)C + coff; p.sCm = sCm * kNComp; p.sCn = sCn * kNComp; p.alpha = alpha;
        p.C0 = C0 ? (const double *)C0 + coff : nullptr;
        p.overwrite = overwrite;
        for (int mt = 0; mt < (M + 127) / 128; ++mt) l.tiles.push_back(TcTile{(int)l.probs.size(), mt});
        l.probs.push_back(p);
        l.phase.push_back(0);
      }
    };
    if (kNComp == 1) {
      one(0, {{0, 0, 0}});
    } else {
      one(0, {{0, 0, 0}, {1, 1, 1}});
      one(1, {{0, 1, 0}, {1, 0, 0}});
    }
  }

  // ---- FP64-accurate re-base products as exact digit products (Ozaki scheme) ----
  struct OzSplitPlan {
    DBuf jobs, rows, chunks;
    int nrows = 0, nchunks = 0;
  };
  struct OzPlan {
    DBuf probs, tiles[2];
    int ntiles[2] = {0, 0};
  };
  // digit planes of one operand kind: kNComp x (kOzSlices planes of n elements), and
  // kNComp x rows exponents
  struct OzBuf {
    DBuf planes, exps;
    int64_t n = 0, rows = 0;
  };
  struct OzList {
    std::vector<OzProb> probs;
    std::vector<int> phase;
    std::vector<OzTile> tiles;
  };
  void alloc_oz(OzBuf &b, int64_t n, int64_t rows) {
    b.n = std::max<int64_t>(n, 8);
    b.rows = std::max<int64_t>(rows, 1);
    b.planes.alloc((size_t)b.n * kOzSlices * kNComp * 2, &bytes_);
    b.exps.alloc((size_t)b.rows * kNComp * 4, &bytes_);
    CK(cudaMemset(b.planes.p, 0, b.planes.bytes));  // padding row groups stay zero
  }
  void finalize_oz_split(OzSplitPlan &pl, const std::vector<OzSplitJob> &jobs) {
    upload(pl.jobs, jobs, &bytes_);
    const std::vector<int2> rows = oz_row_table(jobs);
    const std::vector<int4> ch = oz_split_chunks(jobs);
    upload(pl.rows, rows, &bytes_);
    upload(pl.chunks, ch, &bytes_);
    pl.nrows = (int)rows.size();
    pl.nchunks = (int)ch.size();
  }
  void finalize_oz(OzPlan &pl, const OzList &l) {
    upload(pl.probs, l.probs, &bytes_);
    std::vector<OzTile> t[2];
    for (const OzTile &x : l.tiles) t[l.phase[x.prob]].push_back(x);
    for (int ph = 0; ph < 2; ++ph) {
      upload(pl.tiles[ph], t[ph], &bytes_);
      pl.ntiles[ph] = (int)t[ph].size();
    }
  }
  void run_oz_split(const OzSplitPlan &pl) {
    launch_oz_split((const OzSplitJob *)pl.jobs.p, (const int2 *)pl.rows.p, pl.nrows, (const int4 *)pl.chunks.p,
                    pl.nchunks, st_);
    launches_ += 2;
  }
  void run_oz(const OzPlan &pl) {
    for (int ph = 0; ph < 2; ++ph) {
      if (!pl.ntiles[ph]) continue;
      launch_oz_gemm((const OzProb *)pl.probs.p, (const OzTile *)pl.tiles[ph].p, pl.ntiles[ph], tcerr_.as<int>(), st_);
      ++launches_;
    }
  }
  // digit jobs of one operand (element (r, k) at src[r sr + k sk], S units), one per
  // scalar component, into b at element offset off and exponent offset xoff
  void add_oz_split(std::vector<OzSplitJob> &js, const S *src, int64_t sr, int64_t sk, int rows, int cols,
                    int tile_rows, int rows_pad, OzBuf &b, int64_t off, int64_t xoff) {
    for (int c = 0; c < kNComp; ++c) {
      OzSplitJob j{};
      j.src = (const double *)src + c;
      j.sr = sr * kNComp;
      j.sk = sk * kNComp;
      j.rows = rows; j.cols = cols; j.tile_rows = tile_rows; j.nk = (cols + 63) / 64; j.rows_pad = rows_pad;
      j.planes = ((uint16_t *)b.planes.p) + (int64_t)c * b.n * kOzSlices + off;
      j.plane_elems = b.n;
      j.exps = ((int *)b.exps.p) + (int64_t)c * b.rows + xoff;
      js.push_back(j);
    }
  }
  void add_oz(OzList &l, OzBuf &a, int64_t ao, int64_t axo, OzBuf &b, int64_t bo, int64_t bxo, int M, int N, int K,
              S *C, int64_t sCm, int64_t sCn, double alpha) {
    auto one = [&](int ca, int cb, int cc, double al, int ph) {
      OzProb p{};
      p.A = ((uint16_t *)a.planes.p) + (int64_t)ca * a.n * kOzSlices + ao;
      p.eA = ((int *)a.exps.p) + (int64_t)ca * a.rows + axo;
      p.B = ((uint16_t *)b.planes.p) + (int64_t)cb * b.n * kOzSlices + bo;
      p.eB = ((int *)b.exps.p) + (int64_t)cb * b.rows + bxo;
      p.a_plane = a.n;
      p.b_plane = b.n;
      p.M = M; p.N = N; p.nk = (K + 63) / 64; p.npad = (N + 15) / 16 * 16;
      p.C = (double *)C + cc; p.sCm = sCm * kNComp; p.sCn = sCn * kNComp; p.alpha = al;
      l.probs.push_back(p);
      l.phase.push_back(ph);
      return (int)l.probs.size() - 1;
    };
    // tiles of the problems that share an A operand side by side, so that the CTAs that
    // read the same A digit tile run at the same time and the second read hits L2
    auto tiles = [&](int pa, int pb) {
      const OzProb &p = l.probs[pa];
      for (int mt = 0; mt < (M + 127) / 128; ++mt)
        for (int n0 = 0; n0 < p.npad; n0 += kOzN) {
          l.tiles.push_back(OzTile{pa, mt, n0});
          if (pb >= 0) l.tiles.push_back(OzTile{pb, mt, n0});
        }
    };
    if (kNComp == 1) {
      tiles(one(0, 0, 0, alpha, 0), -1);
    } else {
      const int p0 = one(0, 0, 0, alpha, 0), p1 = one(0, 1, 1, alpha, 0);
      tiles(p0, p1);
      const int p2 = one(1, 1, 0, -alpha, 1), p3 = one(1, 0, 1, alpha, 1);
      tiles(p2, p3);
    }
  }

  // Digit planes of V_pppp' and V_ph (static), of T_b', T_ph and I4 (per re-base), and
  // the problem lists of PP_b = V_pppp' T_b, I4 = W + 1/2 V_ph T_ph and R_ph = T_ph I4.
  void prepare_oz() {
    if (oz_ready_ && oz_v_version_ == v_version_) return;
    if (oz_ready_) {  // plans unchanged: digits of the new V only
      run_oz_split(ozsV_);
      CK(cudaStreamSynchronize(st_));
      oz_v_version_ = v_version_;
      return;
    }
    const Layout &L = *L_;
    const int nc = L.fam[3].count(), nq = L.ph[1].count();
    auto mpad = [](int x) { return (x + 127) / 128 * 128; };
    auto npadf = [](int x) { return (x + 15) / 16 * 16; };
    auto nkf = [](int x) { return (x + 63) / 64; };
    int64_t pa = 0, pb = 0, ra = 0, rb = 0, px = 0, rx = 0, pta = 0, rta = 0, pi9 = 0, ri9 = 0;
    for (int c = 0; c < nc; ++c) {
      const auto &pk = L.pk[c];
      if (pk.P <= 0 || pk.H <= 0) continue;
      pa += (int64_t)mpad(pk.P) * nkf(pk.P) * 64;
      pb += (int64_t)npadf(pk.H) * nkf(pk.P) * 64;
      ra += pk.P;
      rb += npadf(pk.H);
      px += (int64_t)mpad(pk.H) * nkf(pk.P) * 64;     // A = V_hhpp'^T (H x P)
      rx += pk.H;
      pta += (int64_t)mpad(pk.P) * nkf(pk.H) * 64;    // A = T' (P x H)
      rta += pk.P;
      pi9 += (int64_t)npadf(pk.H) * nkf(pk.H) * 64;   // B = I9' (K H, N H)
      ri9 += npadf(pk.H);
    }
    int64_t pv = 0, pt = 0, pr = 0, pi = 0, rv = 0, rt = 0, rr = 0, ri = 0;
    for (int q = 0; q < nq; ++q) {
      const int nph = L.ph[1].side1[q].size(), nhp = L.ph[1].side2[q].size();
      if (nph <= 0 || nhp <= 0) continue;
      pv += (int64_t)mpad(nhp) * nkf(nph) * 64;   // A = V_ph (n_hp x n_ph)
      pt += (int64_t)npadf(nhp) * nkf(nph) * 64;  // B = T_ph (K n_ph, N n_hp)
      pr += (int64_t)mpad(nph) * nkf(nhp) * 64;   // A = T_ph (n_ph x n_hp)
      pi += (int64_t)npadf(nhp) * nkf(nhp) * 64;  // B = I4 (K n_hp, N n_hp)
      rv += nhp; rt += npadf(nhp); rr += nph; ri += npadf(nhp);
    }
    alloc_oz(ozVpp_, pa, ra);
    alloc_oz(ozTb_, pb, rb);
    alloc_oz(ozVph_, pv, rv);
    alloc_oz(ozTphB_, pt, rt);
    alloc_oz(ozTphA_, pr, rr);
    alloc_oz(ozI4B_, pi, ri);
    alloc_oz(ozVhpA_, px, rx);
    alloc_oz(ozTA_, pta, rta);
    alloc_oz(ozI9B_, pi9, ri9);
    if (!tcerr_.p) {
      tcerr_.alloc(sizeof(int), &bytes_);
      CK(cudaMemset(tcerr_.p, 0, sizeof(int)));
    }
    std::vector<OzSplitJob> jv, jb, jt, ji, j9;
    OzList lpp, l4, lr, lx, lhh;
    {
      int64_t qa = 0, qb = 0, xa = 0, xb = 0, voff = 0, hoff = 0;
      int64_t qx = 0, xx = 0, qta = 0, xta = 0, q9 = 0, x9 = 0;
      for (int c = 0; c < nc; ++c) {
        const auto &pk = L.pk[c];
        if (pk.P > 0 && pk.H > 0) {
          add_oz_split(jv, Vpp_.as<S>() + voff, pk.P, 1, pk.P, pk.P, 128, mpad(pk.P), ozVpp_, qa, xa);
          add_oz_split(jb, T_.as<S>() + pk.t_off, pk.P, 1, pk.H, pk.P, npadf(pk.H), npadf(pk.H), ozTb_, qb, xb);
          add_oz(lpp, ozVpp_, qa, xa, ozTb_, qb, xb, pk.P, pk.H, pk.P, PPb_.as<S>() + pk.t_off, 1, pk.P, 1.0);
          // X(kl, ij) = sum_cd V_hhpp'(cd, kl) T'(cd, ij): A = V_hhpp'^T, B the T' digits above
          add_oz_split(jv, Vhp_.as<S>() + pk.t_off, pk.P, 1, pk.H, pk.P, 128, mpad(pk.H), ozVhpA_, qx, xx);
          add_oz(lx, ozVhpA_, qx, xx, ozTb_, qb, xb, pk.H, pk.H, pk.P, X_.as<S>() + hoff, 1, pk.H, 1.0);
          // HH_b(ab, ij) = sum_kl T'(ab, kl) I9'(kl, ij)
          add_oz_split(jb, T_.as<S>() + pk.t_off, 1, pk.P, pk.P, pk.H, 128, mpad(pk.P), ozTA_, qta, xta);
          add_oz_split(j9, I9_.as<S>() + hoff, pk.H, 1, pk.H, pk.H, npadf(pk.H), npadf(pk.H), ozI9B_, q9, x9);
          add_oz(lhh, ozTA_, qta, xta, ozI9B_, q9, x9, pk.P, pk.H, pk.H, PPb_.as<S>() + pk.t_off, 1, pk.P, 1.0);
          qa += (int64_t)mpad(pk.P) * nkf(pk.P) * 64;
          qb += (int64_t)npadf(pk.H) * nkf(pk.P) * 64;
          xa += pk.P;
          xb += npadf(pk.H);
          qx += (int64_t)mpad(pk.H) * nkf(pk.P) * 64;
          xx += pk.H;
          qta += (int64_t)mpad(pk.P) * nkf(pk.H) * 64;
          xta += pk.P;
          q9 += (int64_t)npadf(pk.H) * nkf(pk.H) * 64;
          x9 += npadf(pk.H);
        }
        voff += (int64_t)pk.P * pk.P;
        hoff += (int64_t)pk.H * pk.H;
      }
    }
    {
      int64_t qv = 0, qt = 0, qr = 0, qi = 0, xv = 0, xt = 0, xr = 0, xi = 0, toff = 0, ioff = 0;
      for (int q = 0; q < nq; ++q) {
        const int nph = L.ph[1].side1[q].size(), nhp = L.ph[1].side2[q].size();
        if (nph > 0 && nhp > 0) {
          add_oz_split(jv, Vph_.as<S>() + toff, 1, nhp, nhp, nph, 128, mpad(nhp), ozVph_, qv, xv);
          add_oz_split(jt, Tph_.as<S>() + toff, nph, 1, nhp, nph, npadf(nhp), npadf(nhp), ozTphB_, qt, xt);
          add_oz_split(jt, Tph_.as<S>() + toff, 1, nph, nph, nhp, 128, mpad(nph), ozTphA_, qr, xr);
          add_oz_split(ji, I4_.as<S>() + ioff, nhp, 1, nhp, nhp, npadf(nhp), npadf(nhp), ozI4B_, qi, xi);
          add_oz(l4, ozVph_, qv, xv, ozTphB_, qt, xt, nhp, nhp, nph, I4_.as<S>() + ioff, 1, nhp, 0.5);
          add_oz(lr, ozTphA_, qr, xr, ozI4B_, qi, xi, nph, nhp, nhp, Rph_.as<S>() + toff, 1, nph, 1.0);
          qv += (int64_t)mpad(nhp) * nkf(nph) * 64;
          qt += (int64_t)npadf(nhp) * nkf(nph) * 64;
          qr += (int64_t)mpad(nph) * nkf(nhp) * 64;
          qi += (int64_t)npadf(nhp) * nkf(nhp) * 64;
          xv += nhp; xt += npadf(nhp); xr += nph; xi += npadf(nhp);
        }
        toff += (int64_t)nph * nhp;
        ioff += (int64_t)nhp * nhp;
      }
    }
    finalize_oz_split(ozsV_, jv);
    finalize_oz_split(ozsTb_, jb);
    finalize_oz_split(ozsTph_, jt);
    finalize_oz_split(ozsI4_, ji);
    finalize_oz_split(ozsI9_, j9);
    finalize_oz(ozPP_, lpp);
    finalize_oz(ozX_, lx);
    finalize_oz(ozHH_, lhh);
    finalize_oz(ozI4_, l4);
    finalize_oz(ozRing_, lr);
    run_oz_split(ozsV_);
    CK(cudaStreamSynchronize(st_));
    oz_ready_ = true;
    oz_v_version_ = v_version_;
    ++plan_epoch_;
  }

  // Tile buffers, split jobs and tensor-core problem lists of the mixed residual.
  void prepare_mixed(int kind) {
    if (mixed_ready_ && tc_kind_ == kind && mixed_v_version_ == v_version_) return;
    if (mixed_ready_ && tc_kind_ == kind) {
      // same layout and operand kind: only the split of the new V is redone
      commit();
      run_split(spStatic_);
      CK(cudaStreamSynchronize(st_));
      mixed_v_version_ = v_version_;
      return;
    }
    oz_ready_ = false;  // the re-base problem list points into buffers allocated here
    const Layout &L = *L_;
    tc_kind_ = kind;
    const int tk = tc_tile_k(kind);
    const size_t es = kind == kTcBF16 ? 2 : 4;
    auto mpad = [](int x) { return (x + 127) / 128 * 128; };
    auto npadf = [](int x) { return (x + 15) / 16 * 16; };
    auto nkf = [&](int x) { return (x + tk - 1) / tk; };
    const int nc = L.fam[3].count(), nq = L.ph[1].count();
    // sizes
    TileBuf *bufs[13] = {&tVpp_, &tD_, &tVph_, &tDphB_, &tTphbA_, &tDphA_, &tdI4B_, &tI4B_,
                         &tDA_, &tI9B_, &tTbA_, &tdI9B_, &tVhT_};
    for (TileBuf *b : bufs) b->n = 0;
    for (int c = 0; c < nc; ++c) {
      const auto &pk = L.pk[c];
      if (pk.P <= 0 || pk.H <= 0) continue;
      tVpp_.n += (int64_t)mpad(pk.P) * nkf(pk.P) * tk;
      tVhT_.n += (int64_t)mpad(pk.H) * nkf(pk.P) * tk;   // A = V_hhpp'^T (H x P)
      tD_.n += (int64_t)npadf(pk.H) * nkf(pk.P) * tk;
      tDA_.n += (int64_t)mpad(pk.P) * nkf(pk.H) * tk;    // A = dT' (P x H)
      tTbA_.n += (int64_t)mpad(pk.P) * nkf(pk.H) * tk;   // A = T_b' (P x H)
      tI9B_.n += (int64_t)npadf(pk.H) * nkf(pk.H) * tk;  // B = I9' (K H, N H)
      tdI9B_.n += (int64_t)npadf(pk.H) * nkf(pk.H) * tk; // B = I9' - I9_b'
    }
    for (int q = 0; q < nq; ++q) {
      const int nph = L.ph[1].side1[q].size(), nhp = L.ph[1].side2[q].size();
      if (nph <= 0 || nhp <= 0) continue;
      tVph_.n += (int64_t)mpad(nhp) * nkf(nph) * tk;
      tDphB_.n += (int64_t)npadf(nhp) * nkf(nph) * tk;
      tTphbA_.n += (int64_t)mpad(nph) * nkf(nhp) * tk;
      tDphA_.n += (int64_t)mpad(nph) * nkf(nhp) * tk;
      tdI4B_.n += (int64_t)npadf(nhp) * nkf(nhp) * tk;
      tI4B_.n += (int64_t)npadf(nhp) * nkf(nhp) * tk;
    }
    for (TileBuf *b : bufs) {  // zeroed once: the splits never write all-padding row groups
      b->n = std::max<int64_t>(b->n, 16);
      b->hi.alloc((size_t)b->n * kNComp * es, &bytes_);
      b->lo.alloc((size_t)b->n * kNComp * es, &bytes_);
      CK(cudaMemset(b->hi.p, 0, b->hi.bytes));
      CK(cudaMemset(b->lo.p, 0, b->lo.bytes));
    }
    const size_t sz = sizeof(S);
    Tb_.alloc(std::max<int64_t>(n_t_, 1) * sz, &bytes_);
    PPb_.alloc(std::max<int64_t>(n_t_, 1) * sz, &bytes_);
    Tphb_.alloc(std::max<int64_t>(n_ph_, 1) * sz, &bytes_);
    Rringb_.alloc(std::max<int64_t>(n_t_, 1) * sz, &bytes_);
    I4b_.alloc(std::max<int64_t>(n_i4_, 1) * sz, &bytes_);
    dI4_.alloc(std::max<int64_t>(n_i4_, 1) * sz, &bytes_);
    // the tensor-core product overwrites dI4 block by block; blocks of channels without
    // particle-hole pairs (K = 0) have no product and stay zero
    CK(cudaMemset(dI4_.p, 0, std::max<int64_t>(n_i4_, 1) * sz));
    Xb_.alloc(std::max<int64_t>(n_hh2_, 1) * sz, &bytes_);
    dI9_.alloc(std::max<int64_t>(n_hh2_, 1) * sz, &bytes_);
    // dX = V_hhpp'^T dT' is written block by block by the tensor cores; blocks of channels
    // without pp pairs stay zero
    CK(cudaMemset(dI9_.p, 0, std::max<int64_t>(n_hh2_, 1) * sz));
    xd7_.alloc((size_t)std::max(2 * D_.A * D_.A, 1) * sz, &bytes_);
    HHb_.alloc(std::max<int64_t>(n_t_, 1) * sz, &bytes_);
    tcerr_.alloc(sizeof(int), &bytes_);
    CK(cudaMemset(tcerr_.p, 0, sizeof(int)));
    std::vector<TcSplitJob> js_static, js_tphb, js_it2, js_it3;
    // dT' is split once into packed hi/lo arrays per iteration; its tiled copies (dT' as
    // A and B, dT_ph as A and B) are gathered through maps built here, once per layout
    phl_.alloc(std::max<int64_t>(n_t_, 1) * kNComp * 2 * es, &bytes_);
    tphmap_.alloc(std::max<int64_t>(n_ph_, 1) * sizeof(int32_t), &bytes_);
    launch_tph_map(D_, tphmap_.as<int32_t>(), st_);
    for (auto pr : {std::make_pair(&mD_, &tD_), std::make_pair(&mDA_, &tDA_), std::make_pair(&mDphB_, &tDphB_),
                    std::make_pair(&mDphA_, &tDphA_)})
      pr.first->alloc((size_t)pr.second->n * kNComp * sizeof(int32_t), &bytes_);
    std::vector<TcMapJob> mjobs;
    std::vector<TcGatherJob> gjobs;
    TcList pp, p4, pr1;
    {
      int64_t oa = 0, ob = 0, voff = 0, hoff = 0, oda = 0, otb = 0, oi9 = 0, ovt = 0;
      for (int c = 0; c < nc; ++c) {
        const auto &pk = L.pk[c];
        if (pk.P > 0 && pk.H > 0) {
          S *tb = Tb_.as<S>() + pk.t_off;
          add_split(js_static, Vpp_.as<S>() + voff, nullptr, pk.P, 1, pk.P, pk.P, 128, mpad(pk.P), tVpp_, oa);
          // dX = X - X_b = V_hhpp'^T dT' (H x H, K = P): static A = V_hhpp'^T, B = dT' as
          // the pp-ladder reads it; in the dI4 launch, written over dI9 = I9' - I9_b'
          add_split(js_static, Vhp_.as<S>() + pk.t_off, nullptr, pk.P, 1, pk.H, pk.P, 128, mpad(pk.H), tVhT_, ovt);
          add_tc_multi(p4, {{&tVhT_, ovt, &tD_, ob, pk.P}}, pk.H, pk.H, dI9_.as<S>() + hoff, 1, pk.H, 1.0, nullptr, 1);
          ovt += (int64_t)mpad(pk.H) * nkf(pk.P) * tk;
          add_gather(mjobs, gjobs, pk.t_off, nullptr, pk.P, 1, pk.H, pk.P, npadf(pk.H), npadf(pk.H), tD_, mD_, ob);
          // hh-ladder: R' += HH_b + dT' I9' + T_b' (I9' - I9_b')
          add_gather(mjobs, gjobs, pk.t_off, nullptr, 1, pk.P, pk.P, pk.H, 128, mpad(pk.P), tDA_, mDA_, oda);
          add_split(js_tphb, tb, nullptr, 1, pk.P, pk.P, pk.H, 128, mpad(pk.P), tTbA_, otb);
          add_split(js_it3, I9_.as<S>() + hoff, nullptr, pk.H, 1, pk.H, pk.H, npadf(pk.H), npadf(pk.H), tI9B_, oi9);
          add_split(js_it3, dI9_.as<S>() + hoff, nullptr, pk.H, 1, pk.H, pk.H, npadf(pk.H), npadf(pk.H), tdI9B_, oi9);
          // R' += PP_b + HH_b + V_pppp' dT' + dT' I9' + T_b' (I9' - I9_b'), written once
          add_tc_multi(pp, {{&tVpp_, oa, &tD_, ob, pk.P}, {&tDA_, oda, &tI9B_, oi9, pk.H}, {&tTbA_, otb, &tdI9B_, oi9, pk.H}},
                       pk.P, pk.H, R_.as<S>() + pk.t_off, 1, pk.P, 1.0, PPb_.as<S>() + pk.t_off, 0);
          oa += (int64_t)mpad(pk.P) * nkf(pk.P) * tk;
          ob += (int64_t)npadf(pk.H) * nkf(pk.P) * tk;
          oda += (int64_t)mpad(pk.P) * nkf(pk.H) * tk;
          otb += (int64_t)mpad(pk.P) * nkf(pk.H) * tk;
          oi9 += (int64_t)npadf(pk.H) * nkf(pk.H) * tk;
        }
        hoff += (int64_t)pk.H * pk.H;
        voff += (int64_t)pk.P * pk.P;
      }
    }
    {
      int64_t ov = 0, odb = 0, ota = 0, oda = 0, oi = 0, oib = 0, toff = 0, ioff = 0;
      for (int q = 0; q < nq; ++q) {
        const int nph = L.ph[1].side1[q].size(), nhp = L.ph[1].side2[q].size();
        if (nph > 0 && nhp > 0) {
          S *tphb = Tphb_.as<S>() + toff;
          // static A = V_ph (n_hp x n_ph, column-major)
          add_split(js_static, Vph_.as<S>() + toff, nullptr, 1, nhp, nhp, nph, 128, mpad(nhp), tVph_, ov);
          // per iteration, gathered: B = dT_ph (rows n_hp, K = n_ph), A = dT_ph (rows n_ph, K = n_hp)
          add_gather(mjobs, gjobs, toff, tphmap_.as<int32_t>(), nph, 1, nhp, nph, npadf(nhp), npadf(nhp), tDphB_, mDphB_,
                     odb);
          add_gather(mjobs, gjobs, toff, tphmap_.as<int32_t>(), 1, nph, nph, nhp, 128, mpad(nph), tDphA_, mDphA_, oda);
          // at re-base: A = Tph_b
          add_split(js_tphb, tphb, nullptr, 1, nph, nph, nhp, 128, mpad(nph), tTphbA_, ota);
          // after dI4: B = dI4 and B = I4 = I4_b + dI4 (rows n_hp, K = n_hp; I4 is split
          // from its two parts and never formed in FP64 between re-bases)
          add_split(js_it2, dI4_.as<S>() + ioff, I4b_.as<S>() + ioff, nhp, 1, nhp, nhp, npadf(nhp), npadf(nhp), tdI4B_,
                    oi, 2, &tI4B_, oib);
          // dI4 = 1/2 V_ph dT_ph, written without reading it
          add_tc_multi(p4, {{&tVph_, ov, &tDphB_, odb, nph}}, nhp, nhp, dI4_.as<S>() + ioff, 1, nhp, 0.5, nullptr, 1);
          // dR_ph = R_ph - R_ph,b = T_ph,b dI4 + dT_ph I4, written without reading it; R_ph,b
          // enters R' through the ring terms the re-base stored per amplitude
          add_tc_multi(pr1, {{&tTphbA_, ota, &tdI4B_, oi, nhp}, {&tDphA_, oda, &tI4B_, oib, nhp}}, nph, nhp,
                       Rph_.as<S>() + toff, 1, nph, 1.0, nullptr, 1);
          ov += (int64_t)mpad(nhp) * nkf(nph) * tk;
          odb += (int64_t)npadf(nhp) * nkf(nph) * tk;
          ota += (int64_t)mpad(nph) * nkf(nhp) * tk;
          oda += (int64_t)mpad(nph) * nkf(nhp) * tk;
          oi += (int64_t)npadf(nhp) * nkf(nhp) * tk;
          oib += (int64_t)npadf(nhp) * nkf(nhp) * tk;
        }
        toff += (int64_t)nph * nhp;
        ioff += (int64_t)nhp * nhp;
      }
    }
    finalize_split(spStatic_, js_static);
    finalize_split(spTphb_, js_tphb);
    {  // the maps, and the gather plan over the same units
      std::vector<int4> ch;
      for (size_t j = 0; j < mjobs.size(); ++j)
        split_ranges((int)j, mjobs[j].rows, mjobs[j].rows_pad, mjobs[j].tile_rows, mjobs[j].nk, ch);
      DBuf mj;
      upload(mj, mjobs, &bytes_);
      upload(gplan_.chunks, ch, &bytes_);
      upload(gplan_.jobs, gjobs, &bytes_);
      gplan_.nchunks = (int)ch.size();
      launch_tc_build_map(tc_kind_, (const TcMapJob *)mj.p, (const int4 *)gplan_.chunks.p, gplan_.nchunks, st_);
      CK(cudaStreamSynchronize(st_));  // the map job table goes out of scope
    }
    finalize_split(spIter2_, js_it2);
    finalize_split(spIter3_, js_it3);
    finalize_tc(tcPP_, pp, tc_choice_[0]);
    finalize_tc(tcI4_, p4, tc_choice_[1]);
    finalize_tc(tcR1_, pr1, tc_choice_[2]);
    // FP64 plans of the re-base: PP_b = V_pppp' T, and R' += T I9
    {
      PlanBuilder bp, bh;
      bp.shape_of = bh.shape_of = gemm_shape_;
      int64_t hoff = 0, voff = 0;
      for (int c = 0; c < nc; ++c) {
        const auto &pk = L.pk[c];
        if (pk.H > 0 && pk.P > 0) {
          GemmProb<S> a{};
          a.nseg = 1;
          a.M = pk.P; a.N = pk.H;
          a.seg[0] = GemmSeg<S>{Vpp_.as<S>() + voff, T_.as<S>() + pk.t_off, pk.P, 1, 1, pk.P, pk.P, 1.0};
          a.C = PPb_.as<S>() + pk.t_off; a.sCm = 1; a.sCn = pk.P; a.accumulate = 0;
          bp.add(a, (int64_t)pk.P * pk.P * pk.H);
          GemmProb<S> h{};
          h.nseg = 1;
          h.M = pk.P; h.N = pk.H;
          h.seg[0] = GemmSeg<S>{T_.as<S>() + pk.t_off, I9_.as<S>() + hoff, 1, pk.P, 1, pk.H, pk.H, 1.0};
          h.C = HHb_.as<S>() + pk.t_off; h.sCm = 1; h.sCn = pk.P; h.accumulate = 0;
          bh.add(h, (int64_t)pk.P * pk.H * pk.H);
        }
        hoff += (int64_t)pk.H * pk.H;
        voff += (int64_t)pk.P * pk.P;
      }
      finalize_plan(planPP_, bp);
      finalize_plan(planHH_, bh);
    }
    commit();
    run_split(spStatic_);
    CK(cudaStreamSynchronize(st_));
    mixed_ready_ = true;
    mixed_v_version_ = v_version_;
    ++plan_epoch_;
  }

  // base T_b = 0: every cached product vanishes except I4_b = W
  void set_base_zero() {
    CK(cudaMemsetAsync(Tb_.p, 0, Tb_.bytes, st_));
    CK(cudaMemsetAsync(PPb_.p, 0, PPb_.bytes, st_));
    CK(cudaMemsetAsync(Xb_.p, 0, Xb_.bytes, st_));
    CK(cudaMemsetAsync(Tphb_.p, 0, Tphb_.bytes, st_));
    CK(cudaMemsetAsync(Rringb_.p, 0, Rringb_.bytes, st_));
    CK(cudaMemcpyAsync(I4b_.p, W_.p, std::max<int64_t>(n_i4_, 1) * sizeof(S), cudaMemcpyDeviceToDevice, st_));
    run_split(spTphb_);
  }

  // FP64 residual at T that also becomes the new base of the defect correction.  With
  // digits, every product of it on the FP64 pipe except the one-body dots moves to the
  // exact digit-product GEMM: X = V_hhpp'^T T', I4, the ring, PP_b = V_pppp' T' and
  // HH_b = T' I9'.
  void residual_fp64_rebase(bool digits) {
    mark(0);
    launch_gather_tph<S>(D_, T_.as<S>(), Tph_.as<S>(), st_);
    mark(1);
    cudaStream_t xs;
    if (digits) {
      // T' digits as the B operand (X, PP_b) and as the A operand (HH_b)
      kbegin(kKSplit);
      run_oz_split(ozsTb_);
      kend();
      CK(cudaMemsetAsync(X_.p, 0, std::max<int64_t>(n_hh2_, 1) * sizeof(S), st_));
      kbegin(kKXOz);
      run_oz(ozX_);
      kend();
      xs = fork_side();
    } else {
      xs = fork_side();
      kbegin(kKX);
      run_x(xs);
      kend();
    }
    launch_i7<S>(D_, X_.as<S>(), fdiag_.as<S>(), f7_.as<S>(), d2ij_.as<S>(), i7off_.as<S>(), xs);
    launch_i9<S>(D_, n_hh2_, Vhh_.as<S>(), X_.as<S>(), I9_.as<S>(), xs);
    mark(2);
    launch_i6<S>(D_, (const int2 *)i6rows_.p, ni6rows_, i6dots_.as<S>(), T_.as<S>(), Vhp_.as<S>(), fdiag_.as<S>(),
                 f6_.as<S>(), d2ab_.as<S>(), i6off_.as<S>(), xs);
    mark(3);
    if (digits) {  // I4 = W + 1/2 V_ph T_ph and R_ph = T_ph I4 as digit products
      kbegin(kKSplit);
      run_oz_split(ozsTph_);
      kend();
      CK(cudaMemcpyAsync(I4_.p, W_.p, std::max<int64_t>(n_i4_, 1) * sizeof(S), cudaMemcpyDeviceToDevice, st_));
      kbegin(kKI4Oz);
      run_oz(ozI4_);
      kend();
      kbegin(kKSplit);
      run_oz_split(ozsI4_);
      kend();
      mark(4);
      CK(cudaMemsetAsync(Rph_.p, 0, std::max<int64_t>(n_ph_, 1) * sizeof(S), st_));
      kbegin(kKRingOz);
      run_oz(ozRing_);
      kend();
    } else {
      kbegin(kKI4);
      run_plan(planI4_);
      kend();
      mark(4);
      kbegin(kKRing);
      run_plan(planRing_);
      kend();
    }
    mark(5);
    join_side(xs);
    if (!digits && xs != st_) run_plan(planHH_, xs);  // HH_b = T' I9' beside the pp-ladder product
    launch_rinit<S>(D_, omap_.as<int4>(), rmap_.as<int4>(), T_.as<S>(), Vhp_.as<S>(), Rph_.as<S>(), i6off_.as<S>(),
                    i7off_.as<S>(), nullptr, Rringb_.as<S>(), R_.as<S>(), st_);
    mark(6);
    if (digits) {
      // PP_b and then HH_b accumulate into PP_b (two launches in stream order)
      kbegin(kKSplit);
      run_oz_split(ozsI9_);
      kend();
      CK(cudaMemsetAsync(PPb_.p, 0, n_t_ * sizeof(S), st_));
      kbegin(kKPPOz);
      run_oz(ozPP_);
      kend();
      kbegin(kKHHOz);
      run_oz(ozHH_);
      kend();
    } else {
      kbegin(kKPP64);
      run_plan(planPP_);
      kend();
      if (xs == st_) {
        kbegin(kKHH64);
        run_plan(planHH_);  // HH_b = T' I9'
        kend();
      }
      join_side(xs, 2);
      launch_axpy<S>(n_t_, HHb_.as<S>(), PPb_.as<S>(), st_);
    }
    // the cached products of the new base, PP_b + HH_b, and R' += them
    launch_axpy<S>(n_t_, PPb_.as<S>(), R_.as<S>(), st_);
    // the new base
    CK(cudaMemcpyAsync(Xb_.p, X_.p, std::max<int64_t>(n_hh2_, 1) * sizeof(S), cudaMemcpyDeviceToDevice, st_));
    CK(cudaMemcpyAsync(Tb_.p, T_.p, n_t_ * sizeof(S), cudaMemcpyDeviceToDevice, st_));
    CK(cudaMemcpyAsync(Tphb_.p, Tph_.p, std::max<int64_t>(n_ph_, 1) * sizeof(S), cudaMemcpyDeviceToDevice, st_));
    CK(cudaMemcpyAsync(I4b_.p, I4_.p, std::max<int64_t>(n_i4_, 1) * sizeof(S), cudaMemcpyDeviceToDevice, st_));
    run_split(spTphb_);
    mark(7);
    launches_ += 6;
    if (timing_) accumulate_timers(0, 7);
  }

  // mixed residual: the one-body, I9/I7 and I6 pieces in FP64, the ladder and ring
  // contractions as cached FP64 products at T_b plus tensor-core corrections
  void residual_mixed() {
    mark(0);
    const cudaStream_t xs = fork_side();
    kbegin(kKSplit);
    // dT' = T' - T_b' split once; dT' (B and A) and dT_ph (B and A) gathered from it
    // (T_ph itself is not needed in FP64 between re-bases)
    for (int c = 0; c < kNComp; ++c)
      launch_tc_split_packed(tc_kind_, (const double *)T_.p + c, (const double *)Tb_.p + c, n_t_, kNComp,
                             (char *)phl_.p + (size_t)c * n_t_ * (tc_kind_ == kTcBF16 ? 4 : 8), st_);
    launch_tc_gather(tc_kind_, (const TcGatherJob *)gplan_.jobs.p, (const int4 *)gplan_.chunks.p, gplan_.nchunks, st_);
    launches_ += kNComp + 1;
    kend();
    mark(1);
    // X in FP64: it feeds the dressed hole denominators of every amplitude through I7
    // (a tensor-core X, X_b + V_hhpp'^T dT', costs the solve an iteration); I9' - I9_b'
    // = X - X_b for the hh-ladder correction
    // I7 in FP64 from the X entries it reads, beside the tensor-core work; the rest of
    // X enters only through I9' - I9_b' = dX, a tensor-core correction in the dI4 launch
    kbegin(kKI7);
    launch_i7_direct<S>(D_, Vhp_.as<S>(), T_.as<S>(), xd7_.as<S>(), fdiag_.as<S>(), f7_.as<S>(), d2ij_.as<S>(),
                        i7off_.as<S>(), xs);
    kend();
    mark(2);
    launch_i6<S>(D_, (const int2 *)i6rows_.p, ni6rows_, i6dots_.as<S>(), T_.as<S>(), Vhp_.as<S>(), fdiag_.as<S>(),
                 f6_.as<S>(), d2ab_.as<S>(), i6off_.as<S>(), xs);
    mark(3);
    kbegin(kKTcI4);
    run_tc(tcI4_);  // dI4 = 1/2 V_ph dT_ph, dI9 = dX = V_hhpp'^T dT'
    kend();
    launch_i9b<S>(n_hh2_, Vhh_.as<S>(), Xb_.as<S>(), dI9_.as<S>(), I9_.as<S>(), st_);
    kbegin(kKSplit);
    run_split(spIter2_);  // dI4 (B), I4 = I4_b + dI4 (B)
    run_split(spIter3_);  // I9' (B), I9' - I9_b' (B)
    kend();
    mark(4);
    kbegin(kKTcRing);
    run_tc(tcR1_);  // dR_ph = T_ph,b dI4 + dT_ph I4 (R_ph,b enters through the stored ring terms)
    kend();
    mark(5);
    join_side(xs);
    launch_rinit<S>(D_, omap_.as<int4>(), rmap_.as<int4>(), T_.as<S>(), Vhp_.as<S>(), Rph_.as<S>(), i6off_.as<S>(),
                    i7off_.as<S>(), Rringb_.as<S>(), nullptr, R_.as<S>(), st_);
    mark(6);
    kbegin(kKTcPP);
    run_tc(tcPP_);  // R' += PP_b + HH_b + V_pppp' dT' + dT' I9' + T_b' (I9' - I9_b')
    kend();
    mark(7);
    launches_ += 6;  // i7 (2), i9, i6 (2), rinit
    if (timing_) accumulate_timers(0, 7);
  }

  // ================================================================== state
  std::shared_ptr<const Layout> L_;
  int device_ = 0;
  cudaStream_t st_ = nullptr, xs_ = nullptr;
  cudaEvent_t xev_[3] = {};
  cudaEvent_t ev_[12] = {};
  double timers_[10] = {};
  bool timing_ = false, profiling_ = false;
  int64_t diis_fallbacks_ = 0;  // DIIS systems found singular: the plain step was kept
  bool triples_fp32_ = true;    // (T) contractions in FP32 (FP64 accumulation)
  static constexpr int kKernelEvents = 32;
  cudaEvent_t kev_[2 * kKernelEvents] = {};
  int kslot_[kKernelEvents] = {};
  int kn_ = 0, kcur_ = -1;
  double ktimers_[kKernelSlots] = {};
  int64_t kcount_[kKernelSlots] = {};
  int64_t bytes_ = 0, launches_ = 0;
  DevLayout D_{};
  DevOrbits O_{};
  DevPotential pot_{};
  std::vector<int> partner_, hhhh_to_hhpp_;
  std::vector<int64_t> ppsgn_off_, hhsgn_off_, v4_off_h_;
  int64_t n_t_ = 0, n_vpp_ = 0, n_hh2_ = 0, n_ph_ = 0, n_i4_ = 0, max_stage_ = 0;
  int n_ttile_ = 0;
  // device tables
  DBuf dP_, dH_, dt_off_, dvpp_off_, dhh2_off_, dpp_off_, dhh_off_, dpp_orb_, dhh_orb_, dpp_row_, dhh_row_, dpp_slot_,
      dhh_slot_, dpartner_, dn_ph_, dn_hp_, dtph_off_, di4_off_, dvph_off_, dph_off_, dhp_off_, dph_orb_, dhp_orb_,
      dph_slot_, dhp_slot_, dttile_, dphtile_, dvtile_, pp_sgn_, hh_sgn_, n4_, hp4_slot_, v4_off_, v4_;
  DBuf onx_, ony_, onz_, osz_, otz_, okx_, oky_, okz_, oe_;
  // state
  DBuf T_, R_, Vhp_, Vpp_, Vhh_, X_, I9_, Tph_, Rph_, Vph_, W_, I4_, fdiag_, f6_, f7_, d2ij_, d2ab_, i6off_, i7off_;
  DBuf pairf_;  // per-pair factors of the chiral-like generation
  int npp_total_ = 0, nhh_total_ = 0;  // packed pp and hh pairs over all channels
  DBuf okey_, oof_;                    // orbital -> quantum-number slot, slot -> orbital
  int nkeys_ = 0;
  DBuf partial_, res_, flag_, stage_, hist_, hist_t_, hist_e_, xwork_, xgroups_, xpart_, i6rows_, i6dots_, omap_, rmap_;
  int nxwork_ = 0, nxgroups_ = 0, ni6rows_ = 0;
  Plan planLadder_, planI4_, planRing_, planPP_, planHH_;
  // mixed precision
  bool mixed_ready_ = false;
  int tc_kind_ = 0;
  int64_t v_version_ = 0, mixed_v_version_ = -1;
  DBuf Tb_, PPb_, Tphb_, Rringb_, I4b_, dI4_, tcerr_, Xb_, dI9_, HHb_, xd7_;
  OzBuf ozVpp_, ozTb_, ozVph_, ozTphB_, ozTphA_, ozI4B_, ozVhpA_, ozTA_, ozI9B_;
  OzSplitPlan ozsV_, ozsTb_, ozsTph_, ozsI4_, ozsI9_;
  OzPlan ozPP_, ozI4_, ozRing_, ozX_, ozHH_;
  bool oz_ready_ = false;
  int64_t oz_v_version_ = -1;
  TileBuf tVpp_, tD_, tVph_, tDphB_, tTphbA_, tDphA_, tdI4B_, tI4B_, tDA_, tI9B_, tTbA_, tdI9B_, tVhT_;
  TcPlan tcPP_, tcI4_, tcR1_;
  int tc_choice_[3] = {-1, -1, -1};  // launch form of each correction product picked by the autotuner
  SplitPlan spStatic_, spTphb_, spIter2_, spIter3_;
  DBuf phl_, tphmap_, mD_, mDA_, mDphB_, mDphA_;  // packed split of dT' (hi/lo pairs), gather maps
  SplitPlan gplan_;                                     // gather jobs (TcGatherJob) and chunks
  double *host_res_ = nullptr;
  int host_flag_ = 0;
  int gemm_shape_[4] = {kShape128x32, kShape128x32, kShape64x64, kShape64x64};
  cudaStream_t cs_ = nullptr;       // copy stream of ccx_set_vblocks
  cudaEvent_t sev_[5] = {};         // copied[2], packed[2], compute-stream mark
  DBuf stage2_, copyjobs_;
  double e0_[2] = {0, 0};
  double last_rn_ = 0.0;
  std::vector<IterRecord> ilog_;
  double ilog_prev_[9] = {};
  std::chrono::steady_clock::time_point ilog_t_;
  bool have_fock_ = false, have_t_ = false, dirty_ = true, vph_ready_ = false, generated_ = false;
  // W built on the device by generate(); caller V block kinds since then (bit = kind)
  bool w_generated_ = false;
  unsigned user_set_ = 0;
  int subspace_ = 0, diis_step_ = 6, nstep_ = 0;
  std::vector<int> phys_;
  std::unique_ptr<ITriples<S>> tr_;
};

double fp64_peak(int device) { return measure_fp64_peak(device); }

std::unique_ptr<IEngine> make_engine(std::shared_ptr<const Layout> L, int device, bool complex_scalars) {
  if (complex_scalars) return std::unique_ptr<IEngine>(new Engine<cplx>(std::move(L), device));
  return std::unique_ptr<IEngine>(new Engine<double>(std::move(L), device));
}

}  // namespace ccx
