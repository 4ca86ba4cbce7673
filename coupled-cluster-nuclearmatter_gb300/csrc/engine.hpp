// CCD engine: device image of a layout plus the iteration driver.
#pragma once

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "layout.hpp"
#include "learner.hpp"

namespace ccx {

struct EngineError : std::runtime_error {
  int code;
  EngineError(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

struct IterOpts {
  int mode = 0;          // 0 reference, 1 standard
  int precision = 0;     // 0 FP64, 1 mixed BF16x3, 2 mixed TF32x3
  int max_iter = 100;
  double tol = 1e-6;
  int diis_dim = 8;
  int defect_period = 0;  // mixed: FP64 re-base every k iterations; 0 adaptive
  int verbose = 0;
  int rebase = 0;        // mixed: products of a re-base as 0 FP64 FMA GEMMs, 1 exact digit products (tensor cores)
  double rebase_drop = 0.0;  // mixed, adaptive: re-base once the mixed residual fell by this factor (0: 1e-4)
};
struct IterResult {
  int iterations = 0, converged = 0;
  int fp64_sweeps = 0, mixed_iterations = 0;
  double e_mbpt2[2] = {0, 0}, e_ccd[2] = {0, 0};
  double res_norm = 0.0, seconds = 0.0;
};
// One residual evaluation of the last ccd_iter (or batched solve): what the loop decided
// on, for a structured per-iteration log.
struct IterRecord {
  int iteration = 0;
  int kind = 0;            // 0 reference-loop step, 1 FP64 residual, 2 mixed-precision residual
  double e[2] = {0, 0};    // correlation energy after the update
  double de = 0.0;         // Re of the change since the previous record (the first: since MP2)
  double res_norm = 0.0;   // ||R - D T|| of this residual
  double ms = 0.0;         // host wall-clock since the previous record (the loop synchronises once an iteration)
  double term_ms[9] = {};  // profiling on: device ms of this iteration per residual term; else 0
};
struct PotentialSpec {
  int kind = 0;
  uint64_t lec_seed = 20261203ULL;
  int f32_literals = 1;
};

// Per-kernel timer slots: device time of individual launches inside ccx_ccd_iter.
enum KernelSlot {
  kKX = 0,      // k_gemm: X = V_hhpp' T' (split-K + reduce)
  kKI4 = 1,     // k_gemm: I4 = W + 1/2 V_ph T_ph (FP64)
  kKRing = 2,   // k_gemm: R_ph = T_ph I4 (FP64)
  kKLadder = 3, // k_gemm: fused pp+hh ladder (FP64 solve)
  kKPP64 = 4,   // k_gemm: V_pppp' T' at a mixed-precision re-base (FP64)
  kKHH64 = 5,   // k_gemm: T' I9' hh-ladder of the mixed-precision residual (FP64)
  kKTcPP = 6,   // k_tc_gemm: V_pppp' dT' + dT' I9' + T_b' dI9' + PP_b + HH_b, one launch
  kKTcI4 = 7,   // k_tc_gemm: dI4 = 1/2 V_ph dT_ph
  kKTcRing = 8, // k_tc_gemm: dR_ph = T_ph,b dI4 + dT_ph I4, one launch
  kKSplit = 9,  // k_tc_split: per-iteration operand splits
  kKPPOz = 10,  // k_oz_gemm: V_pppp' T' at a re-base as exact digit products
  kKI4Oz = 11,  // k_oz_gemm: I4 at a re-base as exact digit products
  kKRingOz = 12,  // k_oz_gemm: ring at a re-base as exact digit products
  kKI7 = 13,    // k_i7dots + k_i7sum: I7 of a mixed residual from the X entries it reads
  kKXOz = 14,   // k_oz_gemm: X = V_hhpp'^T T' at a re-base as exact digit products
  kKHHOz = 15,  // k_oz_gemm: HH_b = T' I9' at a re-base as exact digit products
  kKernelSlots = 16
};

class IEngine {
 public:
  virtual ~IEngine() = default;
  virtual bool is_complex() const = 0;
  virtual int64_t device_bytes() const = 0;
  virtual int64_t launches() const = 0;
  virtual int64_t diis_fallbacks() const = 0;
  virtual void set_triples_precision(int p) = 0;  // 0 FP64 contractions, 1 FP32 contractions
  virtual void timers(double ms[10]) const = 0;
  virtual void kernel_timers(double ms[kKernelSlots], int64_t n[kKernelSlots]) const = 0;
  virtual const std::vector<IterRecord> &iter_log() const = 0;
  virtual void set_fock(const double *fock, const double e0[2]) = 0;
  virtual void set_vblock(int kind, int ch, const double *v) = 0;
  virtual void set_vblocks(int kind, int n, const int *chs, const double *const *vs) = 0;
  virtual void generate(const PotentialSpec &p) = 0;
  virtual void get_e0(double e0[2]) = 0;
  virtual void get_vblock(int kind, int ch, double *v) = 0;
  virtual void get_fock(double *f) = 0;
  virtual void *stream() const = 0;
  virtual void mp2() = 0;
  virtual void set_t2(int ch, const double *t) = 0;
  virtual void get_t2(int ch, double *t) = 0;
  virtual void get_r2(int ch, double *r) = 0;
  virtual void set_t2_all(const double *t) = 0;
  virtual void get_t2_all(double *t) = 0;
  virtual void get_denominators(double *d2ij, double *d2ab) = 0;
  virtual void t2_intermediate() = 0;
  virtual void diis_setup(int subspace, int step) = 0;
  virtual void diis_t1t2(int *count) = 0;
  virtual void energy(double e[2]) = 0;
  virtual double residual_norm() = 0;
  virtual void ccd_iter(const IterOpts &o, IterResult &r) = 0;
  virtual void triples(double et[2]) = 0;
  // standard-mode iteration as a state machine (see Engine::iterate_standard), for
  // solving several engines in lockstep
  virtual void std_begin(const IterOpts &o, IterResult &r) = 0;
  virtual void prepare(const IterOpts &o) = 0;
  virtual bool std_done() const = 0;
  virtual void std_launch_residual() = 0;
  virtual void std_launch_update() = 0;
  virtual bool std_after_update() = 0;
  virtual void std_launch_dots() = 0;
  virtual void std_after_dots() = 0;
  virtual void sync() = 0;
  virtual void set_timing(bool on) = 0;
  // per-term and per-kernel event timers of ccd_iter (off by default)
  virtual void set_profiling(bool on) = 0;
  // FP64 GEMM tile-shape autotuner: chosen shape per N bucket, ms[2 k + shape]
  virtual void autotune(int shapes[4], double ms[8]) = 0;
  // launch form of each tensor-core correction product: 1 one launch, 0 one per bucket
  virtual void autotune_tc(int precision, int merged[3], double ms[6]) = 0;
  // device view for the learned warm start (real engines only; false for complex)
  virtual bool ml_view(MLView &v, bool need_t) = 0;
  virtual void mark_t_set() = 0;
};

std::unique_ptr<IEngine> make_engine(std::shared_ptr<const Layout> L, int device, bool complex_scalars);

// contact LECs of the chiral-like synthetic potential drawn from a seed
void draw_lecs(uint64_t seed, double out[9]);
// FP64 FMA throughput probe (TFLOP/s)
double fp64_peak(int device);
// message returned by ccx_last_error() on the calling thread
void set_last_error(const std::string &msg);
// tensor-core split GEMM self-test (tc_selftest.cu)
void tc_selftest(int device, int kind, int nprob, const int *Ms, const int *Ns, const int *Ks, int use_alo, uint64_t seed,
                 double *max_rel, double *ms,
                 long long wait_budget = 0, int *kernel_err = nullptr);

}  // namespace ccx
