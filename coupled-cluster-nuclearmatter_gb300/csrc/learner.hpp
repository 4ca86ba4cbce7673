// Learned warm start: a 4-layer MLP (width 128, SiLU) that predicts, per packed T2
// amplitude, the difference between the converged CCD amplitude and its MP2 value from
// transferable features of the amplitude and, when the host sets one, a prior: the same
// difference interpolated from solutions converged at neighbouring densities.  With a
// prior the network predicts what the prior leaves over, and the prior is added back in
// FP32 (a skip connection), so the BF16 inference perturbs only that remainder.  Trained in FP32 on amplitudes the solver
// converged on other lattices (densities, twists); inference in BF16 on the tensor
// cores writes T2 = T_MP2 + correction straight into an engine.  The CCD iteration that
// follows is unchanged, so the converged energy does not depend on the start.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>

#include "devlayout.hpp"

namespace ccx {

constexpr int kMlIn = 18;    // features: 16 of the amplitude, the prior correction and its flag
constexpr int kMlW = 128;    // hidden width
// parameter vector: W1[128][18] b1[128] W2[128][128] b2[128] W3[128][128] b3[128] w4[128] b4
constexpr int kMlOffW1 = 0, kMlOffB1 = kMlOffW1 + kMlW * kMlIn, kMlOffW2 = kMlOffB1 + kMlW,
              kMlOffB2 = kMlOffW2 + kMlW * kMlW, kMlOffW3 = kMlOffB2 + kMlW, kMlOffB3 = kMlOffW3 + kMlW * kMlW,
              kMlOffW4 = kMlOffB3 + kMlW, kMlOffB4 = kMlOffW4 + kMlW, kMlParams = kMlOffB4 + 1;

// Device view of one real engine: what the feature function reads and where the warm
// start is written.
struct MLView {
  DevLayout L;
  DevOrbits O;
  const double *fdiag = nullptr;  // Fock diagonal
  const double *Vhp = nullptr;    // packed V_hhpp' (same layout as T')
  double *T = nullptr;            // packed T'
  int64_t n_t = 0;
  // orbitals by quantum numbers: okey[p] is orbital p's slot in the (nx, ny, nz, spin,
  // isospin) table, oof[slot] the orbital there (-1 if none); nkeys slots.  The index
  // sort orders the states of a degenerate shell by rounding-level differences of |k|^2,
  // so one quantum-number state has different orbital numbers at different densities.
  const int *okey = nullptr, *oof = nullptr;
  int nkeys = 0;
  double rho = 0, kF = 0, eF = 0, vol = 0, theta[3] = {0, 0, 0};
  cudaStream_t st = nullptr;
};

class ILearner {
 public:
  virtual ~ILearner() = default;
  // features and targets (converged T minus MP2) of the view's current amplitudes, every
  // stride-th packed amplitude
  virtual void add_solution(const MLView &v, int stride) = 0;
  // Prior for the features of later add_solution / warm_start calls on target: per packed
  // amplitude of target, sum_i w[i] times the target correction of views[i]'s current
  // (converged) amplitudes at the same quantum numbers (the same lattice and twist at
  // other densities).  n = 0 clears it (the prior feature and its flag read 0).
  virtual void set_prior(const MLView &target, const MLView *views, const double *w, int n) = 0;
  virtual void clear() = 0;
  virtual int64_t samples() const = 0;
  // Adam on shuffled minibatches; returns the mean loss of the last 10 steps
  virtual double train(int steps, int batch, double lr, uint64_t seed) = 0;
  // T' = T_MP2 + network correction (BF16 tensor-core inference)
  virtual void warm_start(const MLView &v) = 0;
  virtual void get_params(float *p) const = 0;
  virtual void set_params(const float *p) = 0;
  // loss = mean (f(x) - y)^2 and its gradient on a host batch, with the training kernels
  virtual void loss_grad(const float *X, const float *y, int n, double *loss, float *grad) = 0;
  // f(x) on host features: tensor_cores 0 = the FP32 training forward, 1 = the BF16 kernel
  virtual void infer(const float *X, int n, float *out, int tensor_cores) = 0;
};

std::unique_ptr<ILearner> make_learner(int device, uint64_t seed);

}  // namespace ccx
