// ccd_energy_save on caller-owned device buffers, with no allocation at all.
//
// Some callers cannot allocate device memory: a host program that owns every device
// buffer through its own pool (the Fortran host keeps t2_ccm and vnn_hhpp in arrays it
// manages), or code running where an allocation would be an error.  For them this
// entry point evaluates E = 1/4 sum_ch sum_{ab,ij} T(ab,ij) V(ij,ab) directly on their
// buffers, in the reference's layout (ccm_energy.f90:4-71).  Its scratch -- per-channel
// offsets and partial sums -- is the file-scope array g_energy_slots below, at most
// kMaxChannels channels (512 KiB), held by every GPU that loads the library until the
// process exits.
//
// Set-up: the first call in a CUDA context (with that context's device current) looks
// up the device address of g_energy_slots with cudaGetSymbolAddress; make that first
// call before any stream capture.  The address is cached with the context's unique id
// (cuCtxGetId), so a context that is destroyed and created again (cudaDeviceReset, a
// reset primary context, a caller's own context) is seen as new and its address is
// looked up again on its first call.  Every call in a context shares the one array and
// it keeps the last call's contents: each call rewrites every slot it reads, and calls
// whose work overlaps on the GPU race on it.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>

#include "ccx.h"
#include "engine.hpp"

namespace {

constexpr int kMaxChannels = 16384;
constexpr int kMaxDevices = 64;

struct __align__(16) EnergySlot {
  long long off;  // first element of the channel's blocks
  double re, im;  // channel partial sum
  long long pad;
};

static __device__ __align__(256) EnergySlot g_energy_slots[kMaxChannels];

// per device: the context the cached address belongs to, and the address
struct SlotCache {
  unsigned long long ctx_id = 0;
  EnergySlot *addr = nullptr;
};
SlotCache g_slot_cache[kMaxDevices];
std::mutex g_setup_mutex;

using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);

// Unique id of the calling thread's current context, 0 if there is none yet.  The two
// driver functions are reached through the runtime, so the library needs no libcuda
// at link time.
unsigned long long current_context_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  if (!get_current || !get_id) {
    void *f0 = nullptr, *f1 = nullptr;
    cudaDriverEntryPointQueryResult q0 = cudaDriverEntryPointSymbolNotFound, q1 = q0;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess || !f0 || !f1)
      return 0;
    get_current = (CtxGetCurrentFn)f0;
    get_id = (CtxGetIdFn)f1;
  }
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// exclusive prefix sum of n_hh * n_pp into the slot offsets (one block)
__global__ void k_noalloc_offsets(int nch, const int *__restrict__ dims, EnergySlot *slots) {
  __shared__ long long part[1024];
  const int per = (nch + blockDim.x - 1) / blockDim.x;
  const int lo = threadIdx.x * per, hi = min(nch, lo + per);
  long long s = 0;
  for (int c = lo; c < hi; ++c) s += (long long)dims[2 * c] * dims[2 * c + 1];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long acc = 0;
    for (int t = 0; t < (int)blockDim.x; ++t) {
      const long long v = part[t];
      part[t] = acc;
      acc += v;
    }
  }
  __syncthreads();
  long long off = part[threadIdx.x];
  for (int c = lo; c < hi; ++c) {
    slots[c].off = off;
    off += (long long)dims[2 * c] * dims[2 * c + 1];
  }
}

// one block per channel: 1/4 sum T(ab,ij) V(ij,ab), T (n_pp x n_hh), V (n_hh x n_pp)
__global__ void k_noalloc_channel(const int *__restrict__ dims, const double *__restrict__ t2,
                                  const double *__restrict__ v, EnergySlot *slots) {
  const int c = blockIdx.x;
  const int nh = dims[2 * c], np = dims[2 * c + 1];
  const long long off = slots[c].off;
  double re = 0.0, im = 0.0;
  for (long long e = threadIdx.x; e < (long long)nh * np; e += blockDim.x) {
    const long long ab = e % np, ij = e / np;
    const double *t = t2 + 2 * (off + ab + (long long)np * ij);
    const double *w = v + 2 * (off + ij + (long long)nh * ab);
    re += 0.25 * (t[0] * w[0] - t[1] * w[1]);
    im += 0.25 * (t[0] * w[1] + t[1] * w[0]);
  }
  __shared__ double sr[32], si[32];
  for (int o = 16; o > 0; o >>= 1) {
    re += __shfl_xor_sync(0xffffffffu, re, o);
    im += __shfl_xor_sync(0xffffffffu, im, o);
  }
  if ((threadIdx.x & 31) == 0) {
    sr[threadIdx.x >> 5] = re;
    si[threadIdx.x >> 5] = im;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      a += sr[w];
      b += si[w];
    }
    slots[c].re = a;
    slots[c].im = b;
  }
}

// fixed-order sum of the channel partials
__global__ void k_noalloc_finish(int nch, const EnergySlot *slots, double *energy) {
  __shared__ double sr[256], si[256];
  double a = 0.0, b = 0.0;
  for (int c = threadIdx.x; c < nch; c += blockDim.x) {
    a += slots[c].re;
    b += slots[c].im;
  }
  sr[threadIdx.x] = a;
  si[threadIdx.x] = b;
  __syncthreads();
  if (threadIdx.x == 0) {
    double x = 0.0, y = 0.0;
    for (int t = 0; t < (int)blockDim.x; ++t) {
      x += sr[t];
      y += si[t];
    }
    energy[0] = x;
    energy[1] = y;
  }
}

}  // namespace

extern "C" int ccx_ccd_energy_noalloc(int32_t nch, const int32_t *dims, const double *t2, const double *vhhpp,
                                      double *energy, void *stream) {
  if (nch < 1 || !dims || !t2 || !vhhpp || !energy) {
    ccx::set_last_error("ccx_ccd_energy_noalloc: null pointer or nch < 1");
    return CCX_EINVAL;
  }
  if (nch > kMaxChannels) {
    ccx::set_last_error("ccx_ccd_energy_noalloc: more than 16384 channels (the size of its static scratch)");
    return CCX_EINVAL;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    ccx::set_last_error("ccx_ccd_energy_noalloc: no current CUDA device");
    return CCX_ENOGPU;
  }
  EnergySlot *slots = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    SlotCache &c = g_slot_cache[dev];
    const unsigned long long id = current_context_id();
    if (id == 0 || id != c.ctx_id || !c.addr) {
      // first call in this context (or no context yet): look the address up; the
      // lookup creates the device's primary context if the thread has none
      void *p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_energy_slots);
      if (e != cudaSuccess || !p) {
        ccx::set_last_error(cudaGetErrorString(e));
        return CCX_ECUDA;
      }
      c.addr = (EnergySlot *)p;
      c.ctx_id = current_context_id();
    }
    slots = c.addr;
  }
  cudaStream_t st = (cudaStream_t)stream;
  k_noalloc_offsets<<<1, 1024, 0, st>>>(nch, dims, slots);
  k_noalloc_channel<<<nch, 256, 0, st>>>(dims, t2, vhhpp, slots);
  k_noalloc_finish<<<1, 256, 0, st>>>(nch, slots, energy);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    ccx::set_last_error(cudaGetErrorString(e));
    return CCX_ECUDA;
  }
  return CCX_OK;
}
