// Device-side scalar types and helpers shared by the CCD kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ccx {

// complex*16 as the reference stores it: interleaved (re, im)
struct __align__(16) cplx {
  double re, im;
  cplx() = default;
  __host__ __device__ cplx(double r) : re(r), im(0.0) {}
  __host__ __device__ cplx(double r, double i) : re(r), im(i) {}
};

__host__ __device__ inline cplx operator+(cplx a, cplx b) { return cplx(a.re + b.re, a.im + b.im); }
__host__ __device__ inline cplx operator-(cplx a, cplx b) { return cplx(a.re - b.re, a.im - b.im); }
__host__ __device__ inline cplx operator-(cplx a) { return cplx(-a.re, -a.im); }
__host__ __device__ inline cplx operator*(cplx a, cplx b) {
  return cplx(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
__host__ __device__ inline cplx operator*(double s, cplx a) { return cplx(s * a.re, s * a.im); }
__host__ __device__ inline cplx operator*(cplx a, double s) { return cplx(s * a.re, s * a.im); }
__host__ __device__ inline cplx &operator+=(cplx &a, cplx b) { a.re += b.re; a.im += b.im; return a; }
__host__ __device__ inline cplx &operator-=(cplx &a, cplx b) { a.re -= b.re; a.im -= b.im; return a; }
// a / b with the textbook formula (Smith's scaling is not needed at these magnitudes)
__host__ __device__ inline cplx operator/(cplx a, cplx b) {
  double d = b.re * b.re + b.im * b.im;
  return cplx((a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d);
}

__host__ __device__ inline double conj_(double x) { return x; }
__host__ __device__ inline cplx conj_(cplx x) { return cplx(x.re, -x.im); }
__host__ __device__ inline double abs2(double x) { return x * x; }
__host__ __device__ inline double abs2(cplx x) { return x.re * x.re + x.im * x.im; }
__host__ __device__ inline double real_(double x) { return x; }
__host__ __device__ inline double real_(cplx x) { return x.re; }
__host__ __device__ inline double imag_(double) { return 0.0; }
__host__ __device__ inline double imag_(cplx x) { return x.im; }
__host__ __device__ inline bool is_zero(double x) { return x == 0.0; }
__host__ __device__ inline bool is_zero(cplx x) { return x.re == 0.0 && x.im == 0.0; }
__host__ __device__ inline double cabs_(double x) { return x < 0 ? -x : x; }

template <typename S> struct ScalarOf;
template <> struct ScalarOf<double> { static constexpr bool complex = false; };
template <> struct ScalarOf<cplx> { static constexpr bool complex = true; };

template <typename S> __host__ __device__ inline S make_scalar(double re, double im);
template <> __host__ __device__ inline double make_scalar<double>(double re, double) { return re; }
template <> __host__ __device__ inline cplx make_scalar<cplx>(double re, double im) { return cplx(re, im); }

// signed packed index: v = +/-(idx+1), 0 = structurally zero
__host__ __device__ inline int sidx(int v) { return v > 0 ? v - 1 : -v - 1; }
__host__ __device__ inline double ssign(int v) { return v > 0 ? 1.0 : -1.0; }

__device__ inline double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace ccx
