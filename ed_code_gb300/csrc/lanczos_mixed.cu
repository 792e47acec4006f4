// Mixed-precision Lanczos: Krylov vectors and H*v in FP32 complex, FP64 only
// where stability needs it.
//
//  * one Lanczos run (no restarts, no deflation) of `iterations` steps from a
//    seeded start vector; alpha_j = Re<v_j|Hv_j> and beta_{j+1} = |w| are
//    reduced in FP64 with compensated (Neumaier) sums over the FP32 vectors,
//    on the device, so a step needs no host round trip;
//  * reorth_every > 0 keeps every Krylov vector (FP32) and, every
//    reorth_every steps, orthogonalises the last two vectors against all of
//    them, twice (classical Gram-Schmidt with FP64 coefficients).  With FP32
//    vectors orthogonality decays within a few steps once a level converges:
//    every step (1) or every few steps keeps T exact; every 20 steps does not;
//    reorth_every = -1 keeps every vector and reorthogonalises w against
//    v_{j-1}, v_j every step and against all of them only where Simon's
//    estimates of the lost orthogonality call for it (pro_step,
//    lanczos_common.cuh);
//    reorth_every = 0 reorthogonalises w locally against the two latest
//    vectors each step and removes the copies of converged levels
//    afterwards; it keeps every vector when they fit with room to spare,
//    else as many as fit (the 36-site case: 2 GB each) and the later ones in
//    a ring of up to eight;
//  * T's lowest eigenvalues by bisection and their eigenvectors by inverse
//    iteration, in FP64 on the device (tridiag_dev.cu), T read where the
//    recurrence wrote it; Ritz values that T shares with
//    T-without-its-first-row are copies produced by lost orthogonality and
//    are dropped (Cullum and Willoughby's test);
//  * Ritz vectors in FP64 -- from the stored vectors, plus, when only the
//    first k were stored, a re-run of the recurrence from v_{k-1} with the
//    same alpha/beta for the later ones;
//  * one FP64 H*v per Ritz vector x: the reported eigenvalue is the Rayleigh
//    quotient <x|Hx>/<x|x>, and |Hx - theta x|/|x| is its residual.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/edgpu.h"
#include "blas1.cuh"
#include "edg_sector.cuh"
#include "ff.cuh"
#include "tridiag.cuh"
#include "lanczos_common.cuh"

namespace edg {

int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

namespace {


// Precision policies of the vector kernels.  Both keep the scalars of the
// recurrence in FP64 on the device.
//   P32: FP32 complex vectors; sums of exact products in float-float, the
//        three-term update with FP64 scalars split into FP32 heads and tails
//        and rounded once to the FP32 storage (ff.cuh);
//   P64: FP64 complex vectors and plain FP64 arithmetic (products summed with
//        FMAs, as an FP64 zdotc does), the same algorithm with nothing
//        reduced -- the FP64 arm that the FP32 form is compared with.
__device__ __forceinline__ float fmr(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmr(double a, double b, double c) { return fma(a, b, c); }

struct DAcc {  // FP64 products summed in FP64, one FMA each
  double s = 0.0;
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ void add_prod(double x, double y) { s = fma(x, y, s); }
  __device__ __forceinline__ void sub_prod(double x, double y) { s = fma(-x, y, s); }
  __device__ __forceinline__ double value() const { return s; }
};
struct DScalar {
  double v;
  __device__ __forceinline__ explicit DScalar(double x) : v(x) {}
};
struct P32 {
  using V = float2;
  using Real = float;
  using A = FFAcc;
  using S = FFScalar;
  static constexpr bool kFp64 = false;
  static __device__ __forceinline__ float axpy2(float x, S a, float u, S b, float w) { return ff_axpy2(x, a, u, b, w); }
  static __device__ __forceinline__ float scale(float x, S s) { return fmaf(x, s.l, __fmul_rn(x, s.h)); }
};
struct P64 {
  using V = double2;
  using Real = double;
  using A = DAcc;
  using S = DScalar;
  static constexpr bool kFp64 = true;
  static __device__ __forceinline__ double axpy2(double x, S a, double u, S b, double w) {
    return fma(-b.v, w, fma(-a.v, u, x));
  }
  static __device__ __forceinline__ double scale(double x, S s) { return x * s.v; }
};
template <class P>
__device__ __forceinline__ typename P::V mk(typename P::Real x, typename P::Real y) {
  typename P::V r;
  r.x = x;
  r.y = y;
  return r;
}

// partial sums of sum conj(a) b: exact (P32) or FP64 (P64) products summed per
// thread, FP64 across threads; part[(k*gridDim.x + b)*2 + {0,1}], k =
// blockIdx.y selects a = V + k*ld
template <class P>
__global__ void __launch_bounds__(kRedThreads) k_dot(const typename P::V* __restrict__ V, int64_t ld,
                                                     const typename P::V* __restrict__ x, int64_t n,
                                                     double* __restrict__ part, const double* run = nullptr,
                                                     const int* kf = nullptr, int k0 = 0) {
  if (run && *run == 0.0) return;
  if (kf && k0 + (int)blockIdx.y < *kf) return;  // before this step's Gram-Schmidt range
  const typename P::V* a = V + (int64_t)blockIdx.y * ld;
  typename P::A sr, si;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const typename P::V p = a[i], q = x[i];
    sr.add_prod(p.x, q.x);
    sr.add_prod(p.y, q.y);
    si.add_prod(p.x, q.y);
    si.sub_prod(p.y, q.x);
  }
  __shared__ double rr[kRedThreads], ri[kRedThreads];
  rr[threadIdx.x] = sr.value();
  ri[threadIdx.x] = si.value();
  __syncthreads();
  for (int h = kRedThreads / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) {
      rr[threadIdx.x] += rr[threadIdx.x + h];
      ri[threadIdx.x] += ri[threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const int64_t o = ((int64_t)blockIdx.y * gridDim.x + blockIdx.x) * 2;
    part[o] = rr[0];
    part[o + 1] = ri[0];
  }
}

// Sum the partials of vector k (one CTA per k); mode 0: complex result to
// out[2k], mode 1: real part to out[0], mode 2: sqrt of the real part to out[0].
__global__ void __launch_bounds__(kRedThreads) k_finish(const double* __restrict__ part, int nb, double* out,
                                                        int mode, const double* run = nullptr,
                                                        const int* kf = nullptr, int k0 = 0) {
  if (run && *run == 0.0) return;
  if (kf && k0 + (int)blockIdx.x < *kf) return;
  const double* p = part + (int64_t)blockIdx.x * nb * 2;
  __shared__ double rr[kRedThreads], ri[kRedThreads];
  double a = 0, b = 0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    a += p[2 * i];
    b += p[2 * i + 1];
  }
  rr[threadIdx.x] = a;
  ri[threadIdx.x] = b;
  __syncthreads();
  for (int h = kRedThreads / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) {
      rr[threadIdx.x] += rr[threadIdx.x + h];
      ri[threadIdx.x] += ri[threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (mode == 0) {
      out[2 * blockIdx.x] = rr[0];
      out[2 * blockIdx.x + 1] = ri[0];
    } else if (mode == 1) {
      out[0] = rr[0];
    } else {
      out[0] = sqrt(rr[0]);
    }
  }
}

// w = w - alpha v - beta vprev (FP64 alpha/beta; P32: float-float, one final
// rounding to the FP32 storage), and partial sums of |w|^2 of the stored values.
template <class P>
__global__ void __launch_bounds__(kRedThreads) k_step(typename P::V* __restrict__ w, const typename P::V* __restrict__ v,
                                                      const typename P::V* __restrict__ vprev,
                                                      const double* __restrict__ alpha,
                                                      const double* __restrict__ beta, int64_t n,
                                                      double* __restrict__ part) {
  using V = typename P::V;
  const typename P::S a(*alpha), b(vprev ? *beta : 0.0);
  typename P::A s;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const V wi = w[i], vi = v[i];
    const V pi = vprev ? vprev[i] : mk<P>(0, 0);
    const V o = mk<P>(P::axpy2(wi.x, a, vi.x, b, pi.x), P::axpy2(wi.y, a, vi.y, b, pi.y));
    w[i] = o;
    s.add_prod(o.x, o.x);
    s.add_prod(o.y, o.y);
  }
  __shared__ double rr[kRedThreads];
  rr[threadIdx.x] = s.value();
  __syncthreads();
  for (int h = kRedThreads / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) rr[threadIdx.x] += rr[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = rr[0];
    part[2 * blockIdx.x + 1] = 0.0;
  }
}

// Block sums of kQ complex accumulators into part[(k*gridDim.x + b)*2 + {0,1}].
template <int kQ, class A>
__device__ __forceinline__ void block_partials(const A (&r)[kQ], const A (&i)[kQ], double* part) {
  __shared__ double rr[kRedThreads], ri[kRedThreads];
  for (int k = 0; k < kQ; ++k) {
    rr[threadIdx.x] = r[k].value();
    ri[threadIdx.x] = i[k].value();
    __syncthreads();
    for (int h = kRedThreads / 2; h > 0; h >>= 1) {
      if ((int)threadIdx.x < h) {
        rr[threadIdx.x] += rr[threadIdx.x + h];
        ri[threadIdx.x] += ri[threadIdx.x + h];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      const int64_t o = ((int64_t)k * gridDim.x + blockIdx.x) * 2;
      part[o] = rr[0];
      part[o + 1] = ri[0];
    }
    __syncthreads();
  }
}

// The local form's step in one pass: w = w - alpha v - beta vprev as k_step,
// then the partials of <v|w> and <vprev|w> (0 without vprev) for the local
// reorthogonalisation, k = 0 and 1 in k_finish's layout.
template <class P>
__global__ void __launch_bounds__(kRedThreads) k_step_dots(typename P::V* __restrict__ w,
                                                           const typename P::V* __restrict__ v,
                                                           const typename P::V* __restrict__ vprev,
                                                           const double* __restrict__ alpha,
                                                           const double* __restrict__ beta, int64_t n,
                                                           double* __restrict__ part) {
  using V = typename P::V;
  const typename P::S a(*alpha), b(vprev ? *beta : 0.0);
  typename P::A r[2], im[2];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const V wi = w[i], vi = v[i];
    const V pi = vprev ? vprev[i] : mk<P>(0, 0);
    const V o = mk<P>(P::axpy2(wi.x, a, vi.x, b, pi.x), P::axpy2(wi.y, a, vi.y, b, pi.y));
    w[i] = o;
    r[0].add_prod(vi.x, o.x);
    r[0].add_prod(vi.y, o.y);
    im[0].add_prod(vi.x, o.y);
    im[0].sub_prod(vi.y, o.x);
    r[1].add_prod(pi.x, o.x);
    r[1].add_prod(pi.y, o.y);
    im[1].add_prod(pi.x, o.y);
    im[1].sub_prod(pi.y, o.x);
  }
  block_partials<2>(r, im, part);
}

// w -= q0 v + q1 vprev (q complex, device; arithmetic in the vectors'
// precision, as k_sub) and the partials of |w|^2 in k_finish's layout.
template <class P>
__global__ void __launch_bounds__(kRedThreads) k_sub2_norm(typename P::V* __restrict__ w,
                                                           const typename P::V* __restrict__ v,
                                                           const typename P::V* __restrict__ vprev,
                                                           const double* __restrict__ q, int64_t n,
                                                           double* __restrict__ part) {
  using V = typename P::V;
  using R = typename P::Real;
  const R q0r = (R)q[0], q0i = (R)q[1], q1r = (R)q[2], q1i = (R)q[3];
  typename P::A r[1], im[1];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const V y0 = w[i], vi = v[i];
    R re = fmr(-q0r, vi.x, fmr(q0i, vi.y, y0.x));
    R ii = fmr(-q0r, vi.y, fmr(-q0i, vi.x, y0.y));
    if (vprev) {
      const V pi = vprev[i];
      re = fmr(-q1r, pi.x, fmr(q1i, pi.y, re));
      ii = fmr(-q1r, pi.y, fmr(-q1i, pi.x, ii));
    }
    w[i] = mk<P>(re, ii);
    r[0].add_prod(re, re);
    r[0].add_prod(ii, ii);
  }
  block_partials<1>(r, im, part);
}

// dst = src / beta (dst may be src); P32: 1/beta as an FP32 head and tail
template <class P>
__global__ void k_scale_inv(typename P::V* dst, const typename P::V* src, const double* __restrict__ beta, int64_t n) {
  const typename P::S s(1.0 / *beta);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const typename P::V x = src[i];
    dst[i] = mk<P>(P::scale(x.x, s), P::scale(x.y, s));
  }
}

// y -= sum_k q_k V_k with q (complex, device) read into shared memory in the
// vectors' precision.  The q_k are tiny against |y| once the vectors are
// nearly orthogonal, so P32's FP32 arithmetic adds errors far below the FP32
// rounding of y itself.
template <class P>
__global__ void k_sub(typename P::V* __restrict__ y, const typename P::V* __restrict__ V, int64_t ld,
                      const double* __restrict__ q, int K, int64_t n, const double* run = nullptr,
                      const int* kf = nullptr, int k0 = 0) {
  if (run && *run == 0.0) return;
  const int kb = kf ? max(0, *kf - k0) : 0;  // this step's range starts at V_kf
  using R = typename P::Real;
  extern __shared__ __align__(16) unsigned char sraw[];
  R* sq = reinterpret_cast<R*>(sraw);
  for (int k = threadIdx.x; k < 2 * K; k += blockDim.x) sq[k] = (R)q[k];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const typename P::V y0 = y[i];
    R re = y0.x, im = y0.y;
    for (int k = kb; k < K; ++k) {
      const typename P::V vv = V[(int64_t)k * ld + i];
      const R qr = sq[2 * k], qi = sq[2 * k + 1];
      re = fmr(-qr, vv.x, fmr(qi, vv.y, re));
      im = fmr(-qr, vv.y, fmr(-qi, vv.x, im));
    }
    y[i] = mk<P>(re, im);
  }
}

// Whether a classical Gram-Schmidt pass needs a second one (Daniel, Gragg,
// Kaufman and Stewart's criterion): the first removed sum_k |q_k|^2 of
// x's |x|^2; more than 1e-4 of it means x had a component along the V_k large
// enough that the pass's own rounding matters, and the pass is repeated.
// *run = 1.0 or 0.0 for the second pass's kernels.
__global__ void __launch_bounds__(kRedThreads) k_cgs_decide(const double* __restrict__ q, int K,
                                                            const double* __restrict__ xn2, double* run,
                                                            const int* kf) {
  __shared__ double sm[kRedThreads];
  double a = 0;
  for (int k = (kf ? *kf : 0) + threadIdx.x; k < K; k += blockDim.x)
    a += q[2 * k] * q[2 * k] + q[2 * k + 1] * q[2 * k + 1];
  sm[threadIdx.x] = a;
  __syncthreads();
  for (int h = kRedThreads / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) sm[threadIdx.x] += sm[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) *run = sm[0] > 1e-4 * *xn2 ? 1.0 : 0.0;
}

// Partial reorthogonalisation's estimates for this step (pro_step); state =
// {force, kf, full steps}.
__global__ void __launch_bounds__(kProThreads) k_pro(const double* __restrict__ alpha, const double* __restrict__ beta,
                                                     int j, const double* __restrict__ w2, double* omega, int ld,
                                                     int* state) {
  pro_step(alpha, beta, j, *w2, omega, ld, state, state + 1, state + 2);
}

// Second pass of the resident-vector mode: X_e += sum_t y[e*m + j0 + t] V_{j0+t}
// over a window of cnt <= kRing vectors still resident in the ring, so each
// FP64 Ritz vector is read and written once per window instead of once per
// step.  P32: the window sum is float-float; the add to X is FP64.
constexpr int kRing = 8;
template <class P>
struct RingPtrs {
  const typename P::V* v[kRing];
};
template <class P>
__global__ void __launch_bounds__(256) k_ritz_window(double2* __restrict__ X, int64_t n, RingPtrs<P> ring, int cnt,
                                                     const double* __restrict__ y, int m, int j0, int E) {
  __shared__ double sc[kMaxEv * kRing];  // y[e*m + j0 + t] at e*kRing + t
  for (int k = threadIdx.x; k < E * cnt; k += blockDim.x) {
    const int e = k / cnt, t = k % cnt;
    sc[e * kRing + t] = y[(int64_t)e * m + j0 + t];
  }
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    typename P::V v[kRing];
#pragma unroll
    for (int t = 0; t < kRing; ++t)
      if (t < cnt) v[t] = ring.v[t][i];
    for (int e = 0; e < E; ++e) {
      double sr, si;
      if (P::kFp64) {
        DAcc ar, ai;
#pragma unroll
        for (int t = 0; t < kRing; ++t)
          if (t < cnt) {
            const double c = sc[e * kRing + t];
            ar.add_prod(c, (double)v[t].x);
            ai.add_prod(c, (double)v[t].y);
          }
        sr = ar.value();
        si = ai.value();
      } else {
        FFAcc ar, ai;
#pragma unroll
        for (int t = 0; t < kRing; ++t)
          if (t < cnt) {
            const FFScalar c(sc[e * kRing + t]);
            ar.add_prod(c.h, (float)v[t].x);
            ar.lo = fmaf(c.l, (float)v[t].x, ar.lo);
            ai.add_prod(c.h, (float)v[t].y);
            ai.lo = fmaf(c.l, (float)v[t].y, ai.lo);
          }
        sr = ar.value();
        si = ai.value();
      }
      double2 x = X[(int64_t)e * n + i];
      x.x += sr;
      x.y += si;
      X[(int64_t)e * n + i] = x;
    }
  }
}

// FP64 sums over x, Hx: |x|^2, <x|Hx>, and after theta is known |Hx - theta x|^2.
__global__ void __launch_bounds__(kRedThreads) k_rq_partial(const double2* __restrict__ x,
                                                            const double2* __restrict__ hx, int64_t n,
                                                            const double* __restrict__ theta,
                                                            double* __restrict__ part) {
  Acc nx, re, r2;
  const double th = theta ? *theta : 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 a = x[i], b = hx[i];
    nx.add(a.x * a.x + a.y * a.y);
    re.add(a.x * b.x + a.y * b.y);
    const double dr = b.x - th * a.x, di = b.y - th * a.y;
    r2.add(dr * dr + di * di);
  }
  __shared__ double s0[kRedThreads], s1[kRedThreads], s2[kRedThreads];
  s0[threadIdx.x] = nx.value();
  s1[threadIdx.x] = re.value();
  s2[threadIdx.x] = r2.value();
  __syncthreads();
  for (int h = kRedThreads / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) {
      s0[threadIdx.x] += s0[threadIdx.x + h];
      s1[threadIdx.x] += s1[threadIdx.x + h];
      s2[threadIdx.x] += s2[threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[3 * blockIdx.x] = s0[0];
    part[3 * blockIdx.x + 1] = s1[0];
    part[3 * blockIdx.x + 2] = s2[0];
  }
}

// X_q = sum_{j < cnt} y[q*m + j] V_j for q in [q0, q0 + qn), qn <= kRitzChunk:
// each V_j is read once per chunk of Ritz vectors.  P32: the coefficients are
// split into FP32 heads and tails and the sums kept in float-float (ff.cuh);
// P64: FP64 products in compensated FP64 sums.  Written out in FP64.
constexpr int kRitzChunk = 8;
template <class P>
__global__ void __launch_bounds__(256) k_ritz_vectors(double2* __restrict__ X, int64_t n,
                                                      const typename P::V* __restrict__ V, int64_t ldv,
                                                      const double* __restrict__ y, int m, int cnt, int q0, int qn) {
  extern __shared__ __align__(16) unsigned char sraw[];
  if (P::kFp64) {
    double* sy = reinterpret_cast<double*>(sraw);  // qn * cnt coefficients
    for (int k = threadIdx.x; k < qn * cnt; k += blockDim.x) sy[k] = y[(int64_t)(q0 + k / cnt) * m + k % cnt];
    __syncthreads();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
      DAcc ar[kRitzChunk], ai[kRitzChunk];
      for (int j = 0; j < cnt; ++j) {
        const typename P::V v = V[(int64_t)j * ldv + i];
#pragma unroll
        for (int q = 0; q < kRitzChunk; ++q)
          if (q < qn) {
            const double c = sy[q * cnt + j];
            ar[q].add_prod(c, (double)v.x);
            ai[q].add_prod(c, (double)v.y);
          }
      }
#pragma unroll
      for (int q = 0; q < kRitzChunk; ++q)
        if (q < qn) X[(int64_t)(q0 + q) * n + i] = make_double2(ar[q].value(), ai[q].value());
    }
  } else {
    float2* sy2 = reinterpret_cast<float2*>(sraw);  // qn * cnt (head, tail)
    for (int k = threadIdx.x; k < qn * cnt; k += blockDim.x) {
      const FFScalar c(y[(int64_t)(q0 + k / cnt) * m + k % cnt]);
      sy2[k] = make_float2(c.h, c.l);
    }
    __syncthreads();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
      FFAcc ar[kRitzChunk], ai[kRitzChunk];
      for (int j = 0; j < cnt; ++j) {
        const typename P::V v = V[(int64_t)j * ldv + i];
#pragma unroll
        for (int q = 0; q < kRitzChunk; ++q)
          if (q < qn) {
            const float2 c = sy2[q * cnt + j];
            ar[q].add_prod(c.x, (float)v.x);
            ar[q].lo = fmaf(c.y, (float)v.x, ar[q].lo);
            ai[q].add_prod(c.x, (float)v.y);
            ai[q].lo = fmaf(c.y, (float)v.y, ai[q].lo);
          }
      }
#pragma unroll
      for (int q = 0; q < kRitzChunk; ++q)
        if (q < qn) X[(int64_t)(q0 + q) * n + i] = make_double2(ar[q].value(), ai[q].value());
    }
  }
}

// Sum k_rq_partial's partials in one CTA.  mode 0: out = {|x|^2, <x|Hx>,
// theta = <x|Hx>/|x|^2}; mode 1: out[3] = |Hx - theta x| / |x|.
__global__ void __launch_bounds__(kRedThreads) k_rq_sum(const double* __restrict__ part, int nb, double* out,
                                                        int mode) {
  __shared__ double s0[kRedThreads], s1[kRedThreads], s2[kRedThreads];
  double a = 0, b = 0, c = 0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    a += part[3 * i];
    b += part[3 * i + 1];
    c += part[3 * i + 2];
  }
  s0[threadIdx.x] = a;
  s1[threadIdx.x] = b;
  s2[threadIdx.x] = c;
  __syncthreads();
  for (int h = kRedThreads / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) {
      s0[threadIdx.x] += s0[threadIdx.x + h];
      s1[threadIdx.x] += s1[threadIdx.x + h];
      s2[threadIdx.x] += s2[threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (mode == 0) {
      out[0] = s0[0];
      out[1] = s1[0];
      out[2] = s1[0] / s0[0];
    } else {
      out[3] = sqrt(s2[0] / out[0]);
    }
  }
}

int grid_n(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16)); }

struct Dev {
  std::vector<void*> ptrs;
  template <class T>
  cudaError_t alloc(T** p, size_t n) {
    cudaError_t e = cudaMalloc(p, sizeof(T) * std::max<size_t>(n, 1));
    if (e == cudaSuccess) ptrs.push_back(*p);
    return e;
  }
  ~Dev() {
    for (void* p : ptrs) cudaFree(p);
  }
};

}  // namespace

MixedFinish::~MixedFinish() {
  void* p[] = {y, X, HX, part, res};
  for (void* q : p)
    if (q) cudaFree(q);
}

static cudaError_t grow(void** p, size_t bytes, size_t& have) {
  if (bytes <= have) return cudaSuccess;
  if (*p) cudaFree(*p);
  *p = nullptr;
  have = 0;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e == cudaSuccess) have = bytes;
  return e;
}

cudaError_t MixedFinish::reserve(int64_t n, int m, int n_res) {
  cudaError_t e = cudaSuccess;
  if (!part && (e = cudaMalloc(&part, sizeof(double) * 3 * kRedBlocks)) != cudaSuccess) return e;
  if ((e = grow((void**)&y, sizeof(double) * kMaxEv * m, y_bytes)) != cudaSuccess) return e;
  if ((e = grow((void**)&HX, sizeof(double2) * n, hx_bytes)) != cudaSuccess) return e;
  return grow((void**)&res, sizeof(double) * 4 * std::max(n_res, kMaxEv), res_bytes);
}

cudaError_t MixedFinish::reserve_x(int64_t n, int na) {
  return grow((void**)&X, sizeof(double2) * n * na, x_bytes);
}

template <class P>
static int ritz_stored_t(MixedFinish& F, cudaStream_t st, const typename P::V* V, int64_t n, int m, int na, int cnt,
                         const double* ycoef, double2* dst = nullptr) {
  const double* yc = ycoef ? ycoef : F.y;
  double2* X = dst ? dst : F.X;
  // the coefficients of up to kRitzChunk Ritz vectors sit in shared memory:
  // 64 bytes a Krylov vector, past the default 48 KB above 768 vectors
  // (the solvers cap the steps at 2000, i.e. 128 KB, within the opt-in limit)
  const size_t smem_max = 8 * std::min(kRitzChunk, na) * (size_t)cnt;
  if (smem_max > 48 * 1024) {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (smem_max > (size_t)optin)
      return fail(EDG_ERR_UNSUPPORTED, "mixed Lanczos: too many stored steps for the Ritz-vector kernel");
    const cudaError_t ea = cudaFuncSetAttribute(k_ritz_vectors<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)smem_max);
    if (ea != cudaSuccess) return cuda_fail(ea, "mixed Lanczos: Ritz-vector kernel shared memory");
  }
  for (int q0 = 0; q0 < na; q0 += kRitzChunk) {
    const int qn = std::min(kRitzChunk, na - q0);
    k_ritz_vectors<P><<<grid_n(n), 256, 8 * (size_t)qn * cnt, st>>>(X, n, V, n, yc, m, cnt, q0, qn);
  }
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? EDG_OK : cuda_fail(e, "mixed Lanczos: Ritz vectors");
}

int MixedFinish::ritz_stored(cudaStream_t st, const float2* V, int64_t n, int m, int na, int cnt,
                             const double* ycoef) {
  return ritz_stored_t<P32>(*this, st, V, n, m, na, cnt, ycoef);
}

int MixedFinish::ritz_stored(cudaStream_t st, const double2* V, int64_t n, int m, int na, int cnt,
                             const double* ycoef) {
  return ritz_stored_t<P64>(*this, st, V, n, m, na, cnt, ycoef);
}

int MixedFinish::ritz_stored_to(cudaStream_t st, const float2* V, int64_t n, int m, int na, int cnt,
                                const double* ycoef, double2* dst) {
  return ritz_stored_t<P32>(*this, st, V, n, m, na, cnt, ycoef, dst);
}

cudaError_t MixedFinish::rayleigh_async(Sector& S, cudaStream_t st, int64_t n, int na, double* res_dev) {
  for (int q = 0; q < na; ++q) {
    double2* x = X + (int64_t)q * n;
    cudaError_t e = launch_hv(S, x, HX, true, st);
    if (e != cudaSuccess) return e;
    k_rq_partial<<<kRedBlocks, kRedThreads, 0, st>>>(x, HX, n, nullptr, part);
    k_rq_sum<<<1, kRedThreads, 0, st>>>(part, kRedBlocks, res_dev + 4 * q, 0);
    k_rq_partial<<<kRedBlocks, kRedThreads, 0, st>>>(x, HX, n, res_dev + 4 * q + 2, part);
    k_rq_sum<<<1, kRedThreads, 0, st>>>(part, kRedBlocks, res_dev + 4 * q, 1);
  }
  return cudaGetLastError();
}

// A Rayleigh quotient within 1e-8 relative of an earlier one is the same level
// again (a copy that slipped through the test on T) and is dropped, as is a
// Ritz vector of zero or non-finite norm (no level to report).
void pick_levels(const std::vector<double>& rr, const std::vector<double>& th, const std::vector<int>& acc_h, int na,
                 int want, double* eigs, double* ritz, double* resid, std::vector<int>& keep) {
  keep.clear();
  for (int q = 0; q < na; ++q) {
    const double rq = rr[4 * q + 2];
    if (!(rr[4 * q] > 0.0) || !std::isfinite(rq) || !std::isfinite(rr[4 * q + 3])) continue;
    bool dup = false;
    for (int k : keep)
      if (std::fabs(rr[4 * k + 2] - rq) <= 1e-8 * std::fabs(rq)) dup = true;
    if (dup || (int)keep.size() >= want) continue;
    const int slot = (int)keep.size();
    keep.push_back(q);
    eigs[slot] = rq;
    if (ritz) ritz[slot] = th[acc_h[q]];
    if (resid) resid[slot] = rr[4 * q + 3];
  }
}

template <class P>
static int solve_mixed_t(Sector& S, const edg_mixed_opts& o, double* eigs, double* ritz, double* resid,
                         int64_t* n_out, double* evecs, edg_mixed_stats* stats) {
  using Vt = typename P::V;
  constexpr size_t kVB = sizeof(Vt);
  const int64_t n = S.P.n_p;
  const int m = (int)std::min<int64_t>(o.iterations, n);
  const int want = std::min(std::min(o.n_ev, kMaxEv), m);
  if (want <= 0 || m < 2) return fail(EDG_ERR_INVALID, "need n_ev >= 1 and at least 2 iterations");
  const bool partial = o.reorth_every < 0;  // partial reorthogonalisation (pro_step)
  const bool reorth = o.reorth_every > 0 || partial;
  bool store = reorth;  // every Krylov vector kept in HBM
  cudaStream_t st = S.stream;
  using clk = std::chrono::steady_clock;
  const auto t_start = clk::now();
  Dev D;
  Vt *V = nullptr, *w = nullptr, *buf[kRing] = {};
  int ring = 3;  // resident vectors past the stored ones: the recurrence needs 3
  int kept = 0;   // v_0 .. v_{kept-1} stored in V; the later ones live in the ring
  double *alpha, *beta, *part, *scal, *lq;
  cudaError_t e = cudaSuccess;
  if (reorth) {
    if ((e = D.alloc(&V, (size_t)n * (m + 1))) != cudaSuccess)
      return fail(EDG_ERR_NOMEM, "mixed Lanczos: the stored Krylov vectors do not fit (use reorth_every=0)");
    kept = m + 1;
  } else {
    // Without full reorthogonalisation the vectors are still stored, as many
    // as fit beside the FP64 Ritz vectors, the ring and w with room to spare.
    // All of them: the Ritz vectors come from storage and no second pass is
    // needed.  Some of them: the second pass starts where storage ends.  The
    // recurrence is the same in every form.
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const int n_try = std::min(kMaxEv, std::min(want + 4, m));
    const double vb = (double)kVB * (double)n;
    const double rest = 16.0 * n * n_try + vb * (kRing + 2) + double(1 << 30);
    const double fit = std::floor((0.9 * (double)free_b - rest) / vb);
    int k = fit >= (double)(m + 1) ? m + 1 : (int)std::max(0.0, fit);
    // EDG_MIXED_KEEP=k stores at most k vectors (0: the resident form), for
    // comparisons of the three forms
    if (const char* cap = std::getenv("EDG_MIXED_KEEP")) k = std::min(k, std::max(0, std::atoi(cap)));
    if (k < m + 1 && k > m - 8) k = m - 8;  // a second pass of a handful of steps is not worth keeping
    if (k < 8) k = 0;
    if (k > 0) {
      if (D.alloc(&V, (size_t)n * k) == cudaSuccess)
        kept = k;
      else
        cudaGetLastError();
    }
    store = kept == m + 1;
  }
  if (!store) {
    for (int k = 0; k < 3 && e == cudaSuccess; ++k) e = D.alloc(&buf[k], (size_t)n);
    if (e != cudaSuccess) return fail(EDG_ERR_NOMEM, "mixed Lanczos: vectors do not fit");
    // up to kRing - 3 more when they fit with room to spare: the second pass
    // then adds them to the Ritz vectors a window at a time
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const size_t vb = kVB * (size_t)n;
    while (ring < kRing && free_b > vb * (size_t)(kRing - ring + 8) &&
           D.alloc(&buf[ring], (size_t)n) == cudaSuccess)
      ++ring;
    cudaGetLastError();
  }
  if ((e = D.alloc(&w, (size_t)n)) != cudaSuccess) return fail(EDG_ERR_NOMEM, "mixed Lanczos: w");
  const int64_t kparts = (int64_t)std::max(m + 1, 4) * kRedBlocks * 2;
  if ((e = D.alloc(&alpha, m + 1)) != cudaSuccess || (e = D.alloc(&beta, m + 2)) != cudaSuccess ||
      (e = D.alloc(&part, kparts)) != cudaSuccess || (e = D.alloc(&scal, 2 * (m + 2) + 2)) != cudaSuccess ||
      (e = D.alloc(&lq, 4)) != cudaSuccess)
    return fail(EDG_ERR_NOMEM, "mixed Lanczos: scratch");
  cudaMemsetAsync(beta, 0, sizeof(double) * (m + 2), st);
  double* omega = nullptr;
  int* pstate = nullptr;  // {force, kf, full steps}
  if (partial) {
    if ((e = D.alloc(&omega, 2 * (size_t)(m + 2))) != cudaSuccess || (e = D.alloc(&pstate, 3)) != cudaSuccess)
      return fail(EDG_ERR_NOMEM, "mixed Lanczos: scratch");
    cudaMemsetAsync(pstate, 0, sizeof(int) * 3, st);
  }

  auto vec = [&](int j) -> Vt* { return j < kept ? V + (int64_t)j * n : buf[(j - kept) % ring]; };
  auto norm_into = [&](const Vt* x, double* dst) {  // dst = |x| in FP64
    k_dot<P><<<dim3(kRedBlocks, 1), kRedThreads, 0, st>>>(x, 0, x, n, part);
    k_finish<<<1, kRedThreads, 0, st>>>(part, kRedBlocks, dst, 2);
  };
  double t_hv = 0;
  int64_t hv_calls = 0;
  // one Lanczos pass; in the second pass (same recurrence, same alpha/beta)
  // the Ritz vectors X are accumulated from the device coefficients yd.  The
  // second pass starts at the last stored vector, whose predecessors are
  // stored too; the stored vectors' share of X is already in place.
  auto run = [&](bool second, double2* X, int E, const double* yd) -> cudaError_t {
    cudaError_t ce = cudaSuccess;
    const int j0 = second && kept > 0 ? kept - 1 : 0;
    if (j0 == 0) {
      ce = edg_fill_random(w, n, P::kFp64 ? EDG_C128 : EDG_C64, o.seed, st) == EDG_OK ? cudaSuccess
                                                                                    : cudaErrorUnknown;
      if (ce != cudaSuccess) return ce;
      norm_into(w, scal);                                     // |v0 unnormalised|
      k_scale_inv<P><<<grid_n(n), 256, 0, st>>>(vec(0), w, scal, n);
    }
    const int win = std::max(1, ring - 2);  // vectors V_j0..V_j still resident at step j
    int acc_from = second ? kept : 0;
    for (int j = j0; j < m; ++j) {
      if (second) {
        if (j - acc_from + 1 == win || j + 1 == m) {
          RingPtrs<P> rp{};
          for (int t = 0; t <= j - acc_from; ++t) rp.v[t] = vec(acc_from + t);
          k_ritz_window<P><<<grid_n(n), 256, 0, st>>>(X, n, rp, j - acc_from + 1, yd, m, acc_from, E);
          acc_from = j + 1;
        }
        if (j + 1 == m) break;
      }
      auto t0 = clk::now();
      if ((ce = launch_hv(S, vec(j), w, P::kFp64, st)) != cudaSuccess) return ce;
      ++hv_calls;
      if (!second) {
        k_dot<P><<<dim3(kRedBlocks, 1), kRedThreads, 0, st>>>(vec(j), 0, w, n, part);
        k_finish<<<1, kRedThreads, 0, st>>>(part, kRedBlocks, alpha + j, 1);
      }
      if (!reorth) {
        // Local reorthogonalisation of w against v_j and v_{j-1}, the vectors
        // still resident: it slows the growth of the copies that FP32 vectors
        // make without full reorthogonalisation.  Fused: the step and both
        // coefficients in one pass, the subtraction and |w|^2 in another.
        // The second pass repeats it (the kernels are deterministic, so with
        // the same coefficients).
        const Vt* vp = j > 0 ? vec(j - 1) : nullptr;
        k_step_dots<P><<<kRedBlocks, kRedThreads, 0, st>>>(w, vec(j), vp, alpha + j, beta + j, n, part);
        k_finish<<<2, kRedThreads, 0, st>>>(part, kRedBlocks, lq, 0);
        k_sub2_norm<P><<<kRedBlocks, kRedThreads, 0, st>>>(w, vec(j), vp, lq, n, part);
        if (!second) k_finish<<<1, kRedThreads, 0, st>>>(part, kRedBlocks, beta + j + 1, 2);
      } else {
        k_step<P><<<kRedBlocks, kRedThreads, 0, st>>>(w, vec(j), j > 0 ? vec(j - 1) : nullptr, alpha + j, beta + j,
                                                      n, part);
        if (!second && (partial || (j + 1) % o.reorth_every == 0)) {
          // Periodic reorthogonalisation in its two-vector form: between two
          // reorthogonalisations v_j has drifted too, so it is cleaned against
          // v_0..v_{j-1} first, then w against v_0..v_j.  (Cleaning w alone
          // lets the recurrence carry v_j's error into every later vector.)
          // Classical Gram-Schmidt; the coefficients of all K vectors stay in
          // scal[0, 2K).  v_j's cleaning always takes a second pass; w's takes
          // one only when the first removed more than 1e-4 of |w|^2 (decided
          // on the device, lq[1]), as every step's reorthogonalisation needs
          // it only now and then.  With partial reorthogonalisation the range
          // is v_kf..v_j, kf set on the device each step (pro_step): j - 1
          // (local) or 0 (full, when the estimates call for it).
          auto cgs2 = [&](Vt* x, int K, const double* xn2, const int* kf) {
            for (int pass = 0; pass < 2; ++pass) {
              const double* run = pass == 1 && xn2 ? lq + 1 : nullptr;
              for (int k0 = 0; k0 < K; k0 += 512) {
                const int kk = std::min(512, K - k0);
                k_dot<P><<<dim3(kRedBlocks, kk), kRedThreads, 0, st>>>(V + (int64_t)k0 * n, n, x, n, part, run,
                                                                       kf, k0);
                k_finish<<<kk, kRedThreads, 0, st>>>(part, kRedBlocks, scal + 2 * k0, 0, run, kf, k0);
                k_sub<P><<<grid_n(n), 256, sizeof(typename P::Real) * 2 * kk, st>>>(x, V + (int64_t)k0 * n, n,
                                                                                    scal + 2 * k0, kk, n, run, kf, k0);
              }
              if (pass == 0 && xn2) k_cgs_decide<<<1, kRedThreads, 0, st>>>(scal, K, xn2, lq + 1, kf);
            }
          };
          if (!partial && o.reorth_every > 1 && j > 0) {
            cgs2(vec(j), j, nullptr, nullptr);
            norm_into(vec(j), scal + 2 * (m + 1));
            k_scale_inv<P><<<grid_n(n), 256, 0, st>>>(vec(j), vec(j), scal + 2 * (m + 1), n);
          }
          k_finish<<<1, kRedThreads, 0, st>>>(part, kRedBlocks, lq, 1);  // |w|^2 after the step (k_step)
          if (partial) k_pro<<<1, kProThreads, 0, st>>>(alpha, beta, j, lq, omega, m + 2, pstate);
          cgs2(w, j + 1, lq, partial ? pstate + 1 : nullptr);
          norm_into(w, beta + j + 1);
        } else if (!second) {
          k_finish<<<1, kRedThreads, 0, st>>>(part, kRedBlocks, beta + j + 1, 2);
        }
      }
      if (j + 1 < m || second) k_scale_inv<P><<<grid_n(n), 256, 0, st>>>(vec(j + 1), w, beta + j + 1, n);
      if ((ce = cudaGetLastError()) != cudaSuccess) return ce;
      t_hv += std::chrono::duration<double>(clk::now() - t0).count();
    }
    return cudaStreamSynchronize(st);
  };
  if ((e = run(false, nullptr, 0, nullptr)) != cudaSuccess) return cuda_fail(e, "mixed Lanczos");
  // Ritz values and coefficients of T, on the device
  MixedFinish F;
  const int n_try = std::min(kMaxEv, std::min(want + 4, m));
  if ((e = F.reserve(n, m, n_try)) != cudaSuccess) return fail(EDG_ERR_NOMEM, "mixed Lanczos: scratch");
  TdOut sel{};
  int rc = ritz_select_device(alpha, beta, m, n_try, kCand, F.y, st, sel);
  if (rc != EDG_OK) return rc;
  const int na = sel.na;
  std::vector<int> acc_h(na);
  std::vector<double> th(na);
  for (int q = 0; q < na; ++q) {
    acc_h[q] = q;
    th[q] = sel.theta[q];
  }
  if (na == 0) return fail(EDG_ERR_NOT_CONVERGED, "mixed Lanczos: no Ritz value survived the copy test");
  // Ritz vectors in FP64
  if ((e = F.reserve_x(n, na)) != cudaSuccess) return fail(EDG_ERR_NOMEM, "mixed Lanczos: FP64 Ritz vectors do not fit");
  int passes = 1;
  if (store) {
    if ((rc = F.ritz_stored(st, V, n, m, na, m)) != EDG_OK) return rc;
  } else {
    passes = 2;
    if (kept > 0) {
      if ((rc = F.ritz_stored(st, V, n, m, na, kept)) != EDG_OK) return rc;
    } else {
      cudaMemsetAsync(F.X, 0, sizeof(double2) * na * n, st);
    }
    if ((e = run(true, F.X, na, F.y)) != cudaSuccess) return cuda_fail(e, "mixed Lanczos: second pass");
  }
  // FP64 Rayleigh quotient and residual of each Ritz vector
  std::vector<double> rr(4 * (size_t)na);
  if ((e = F.rayleigh_async(S, st, n, na, F.res)) != cudaSuccess) return cuda_fail(e, "mixed Lanczos: FP64 H*v");
  cudaMemcpyAsync(rr.data(), F.res, sizeof(double) * 4 * na, cudaMemcpyDeviceToHost, st);
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(e, "mixed Lanczos: residual");
  std::vector<int> keep;
  pick_levels(rr, th, acc_h, na, want, eigs, ritz, resid, keep);
  if (evecs) {
    // normalised FP64 eigenvectors to the host
    std::vector<double2> hx(n);
    for (size_t slot = 0; slot < keep.size(); ++slot) {
      cudaMemcpyAsync(hx.data(), F.X + (int64_t)keep[slot] * n, sizeof(double2) * n, cudaMemcpyDeviceToHost, st);
      if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(e, "mixed Lanczos: vectors");
      const double sc = 1.0 / std::sqrt(rr[4 * keep[slot]]);
      for (int64_t i = 0; i < n; ++i) {
        evecs[2 * ((int64_t)slot * n + i)] = hx[i].x * sc;
        evecs[2 * ((int64_t)slot * n + i) + 1] = hx[i].y * sc;
      }
    }
  }
  *n_out = (int64_t)keep.size();
  if (stats) {
    stats->reorth_steps = reorth ? m : 0;
    if (partial && cudaMemcpy(&stats->reorth_steps, pstate + 2, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
      stats->reorth_steps = -1;
    if (o.reorth_every > 1) stats->reorth_steps = m / o.reorth_every;
    stats->hv_calls = hv_calls + na;
    stats->hv_seconds = t_hv;
    stats->passes = passes;
    stats->stored_vectors = kept;
    stats->total_seconds = std::chrono::duration<double>(clk::now() - t_start).count();
  }
  return EDG_OK;
}

int solve_mixed(Sector& S, const edg_mixed_opts& o, double* eigs, double* ritz, double* resid, int64_t* n_out,
                double* evecs, edg_mixed_stats* stats) {
  return o.fp64_vectors ? solve_mixed_t<P64>(S, o, eigs, ritz, resid, n_out, evecs, stats)
                        : solve_mixed_t<P32>(S, o, eigs, ritz, resid, n_out, evecs, stats);
}

}  // namespace edg
