// Perturbative triples (T) on the device: pert_triples2 (ccm_triples.f90:528-735).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>

#include "devlayout.hpp"
#include "kernels.hpp"
#include "layout.hpp"

namespace ccx {

template <typename S>
class ITriples {
 public:
  virtual ~ITriples() = default;
  virtual bool has_v() const = 0;
  // vnn_hhhp(ch)%val (n_hh x n_hp) / vnn_hppp(ch)%val (n_hp x n_pp), ordered, complex interleaved
  virtual void set_hhhp(int ch, const double *v, cudaStream_t st) = 0;
  virtual void set_hppp(int ch, const double *v, cudaStream_t st) = 0;
  virtual void generate_v(const DevPotential &pot, cudaStream_t st) = 0;
  // fp32: the 18 gather-contractions of each (abc, ijk) pair in FP32 on FP32 copies of T
  // (n_t packed elements) and V; the |W|^2 / D accumulation is FP64 either way
  virtual void energy(const S *T, int64_t n_t, const S *fdiag, double et[2], cudaStream_t st, bool fp32) = 0;
  virtual int64_t launches() const = 0;
  virtual int64_t count() const = 0;  // number of (abc, ijk) pairs
};

template <typename S>
std::unique_ptr<ITriples<S>> make_triples(const Layout &L, const DevLayout &D, const DevOrbits &O, int device);

}  // namespace ccx
