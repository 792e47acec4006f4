// Float-float arithmetic for the FP32-vector kernels.
//
// GB300 executes FP64 at 1/64 of its FP32 rate, so an FP64 loop over FP32
// vectors is bound by FP64 issue long before HBM: a compensated FP64 dot
// product (about 12 FP64 operations per complex entry) runs near 0.4 TB/s.
// These helpers keep about 48 bits with FP32 instructions only, using the
// error-free transformations two-sum (Knuth) and two-product (one FMA):
//   s + e == a + b exactly,  p + e == a * b exactly.
// The _rn intrinsics keep the compiler from contracting the steps into FMAs,
// which would break the exactness.
#pragma once
#include <cuda_runtime.h>

namespace edg {

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = __fmul_rn(a, b);
  e = fmaf(a, b, -p);
}

// Running sum hi + lo; the rounding errors of each step go into lo.  The
// error of the sum is about n * 2^-48 of the magnitudes, not n * 2^-24.
struct FFAcc {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float x) {
    float s, e;
    two_sum(hi, x, s, e);
    hi = s;
    lo = __fadd_rn(lo, e);
  }
  // add the exact product a * b
  __device__ __forceinline__ void add_prod(float a, float b) {
    float p, pe;
    two_prod(a, b, p, pe);
    add(p);
    lo = __fadd_rn(lo, pe);
  }
  // add the exact product -a * b
  __device__ __forceinline__ void sub_prod(float a, float b) {
    float p, pe;
    two_prod(a, b, p, pe);
    add(-p);
    lo = __fsub_rn(lo, pe);
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

// Running sum with Kahan's compensation, for dot products whose products
// may be rounded: each product enters as fma(a, b, -c), rounded once, so a
// term costs four FP32 instructions instead of add_prod's ten.  The products'
// own rounding errors total at most 2^-24 sum |a_i b_i| (at most 2^-24 |a||b|
// by Cauchy-Schwarz, below the FP32 rounding of the vectors themselves); the
// summation error is about 2^-23 of the sum plus n 2^-48 of the magnitudes.
struct KahanAcc {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add_y(float y) {
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  }
  __device__ __forceinline__ void add_prod(float a, float b) { add_y(fmaf(a, b, -c)); }
  __device__ __forceinline__ void sub_prod(float a, float b) { add_y(fmaf(-a, b, -c)); }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// x - a*u - b*w for an FP64 scalar pair (a, b) split into FP32 heads and
// tails, rounded once to FP32 at the end: the result agrees with the FP64
// expression rounded to FP32 except in near-ties.
struct FFScalar {
  float h, l;
  __device__ __forceinline__ explicit FFScalar(double x) {
    h = (float)x;
    l = (float)(x - (double)h);
  }
};

__device__ __forceinline__ float ff_axpy2(float x, FFScalar a, float u, FFScalar b, float w) {
  float p, pe, s, e;
  two_prod(a.h, u, p, pe);
  two_sum(x, -p, s, e);
  float err = __fsub_rn(e, pe);
  err = fmaf(-a.l, u, err);
  two_prod(b.h, w, p, pe);
  float s2, e2;
  two_sum(s, -p, s2, e2);
  err = __fadd_rn(err, __fsub_rn(e2, pe));
  err = fmaf(-b.l, w, err);
  return __fadd_rn(s2, err);
}

}  // namespace edg
