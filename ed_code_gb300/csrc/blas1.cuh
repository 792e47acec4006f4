// Vector kernels for the Lanczos drivers (BLAS-1 on complex vectors).
//
// Reductions are deterministic: a fixed grid of kRedBlocks CTAs each sums a
// fixed strided slice in a fixed order, then one CTA sums the partials in
// order -- the result does not depend on timing or on the device.  (The
// reference's OpenMP reduction at lanczos.cpp:36 changes with the thread
// count, about 3e-12 in the eigenvalues.)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace edg {

constexpr int kRedBlocks = 1024;
constexpr int kRedThreads = 256;

struct cd {  // complex double in registers
  double re, im;
};

// Interleaved complex vector element access for FP64 (double2) and FP32 (float2).
template <typename T>
struct VecTraits;
template <>
struct VecTraits<double2> {
  static __device__ __forceinline__ cd load(const double2* p, int64_t i) {
    const double2 x = p[i];
    return {x.x, x.y};
  }
  static __device__ __forceinline__ void store(double2* p, int64_t i, cd v) { p[i] = make_double2(v.re, v.im); }
};
template <>
struct VecTraits<float2> {
  static __device__ __forceinline__ cd load(const float2* p, int64_t i) {
    const float2 x = p[i];
    return {(double)x.x, (double)x.y};
  }
  static __device__ __forceinline__ void store(float2* p, int64_t i, cd v) {
    p[i] = make_float2((float)v.re, (float)v.im);
  }
};

// Compensated (Kahan-Babuska / Neumaier) accumulation in FP64.
struct Acc {
  double s = 0.0, c = 0.0;
  __device__ __forceinline__ void add(double x) {
    const double t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
  }
  __device__ __forceinline__ double value() const { return s + c; }
};

}  // namespace edg
