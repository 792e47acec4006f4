// Eigensolvers around the GPU H*v.
//
// solve_plain(): the reference's sector eigensolver in FP64 on the GPU --
//   * n_p <= dense_threshold: exact_evecs (lanczos.cpp:81-131): the dense
//     sector matrix (makeH, H_v.cpp:21-190) diagonalised on the device
//     (dense.cu), all eigenvalues returned;
//   * otherwise lanczos_evecs (lanczos.cpp:133-349), step for step: one
//     eigenvalue at a time with deflation against the earlier eigenvectors,
//     `ncycles` restarts of `iterations` steps, three-term recurrence
//     (alpha = <v|Hv>, beta = |w|), classical Gram-Schmidt against the
//     earlier eigenvectors every step and against every stored Krylov vector
//     in the last cycle, the lowest eigenvalue of T after every step and the
//     convergence test |E0 - previous| < tol in the middle cycles, the Ritz
//     vector rebuilt from the stored Krylov vectors at the end of each cycle.
//   The vectors, the scalars of the recurrence and T live in HBM; T's lowest
//   eigenvalue and its eigenvector come from the device tridiagonal kernels
//   (tridiag_dev.cu).  The host reads back only that eigenvalue each step,
//   for the reference's log lines and convergence test.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/edgpu.h"
#include "blas1.cuh"
#include "edg_sector.cuh"
#include "lanczos_common.cuh"
#include "tridiag.cuh"

namespace edg {

int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

namespace {

using cplx = std::complex<double>;

// ---------------------------------------------------------------- kernels ---
template <typename T>
__global__ void __launch_bounds__(kRedThreads) k_dotc_partial(const T* __restrict__ V, int64_t ld,
                                                              const T* __restrict__ x, int64_t n,
                                                              double* __restrict__ part) {
  // part[(k*kRedBlocks + b)*2 + {0,1}] = partial sum of conj(V_k) x, k = blockIdx.y
  const T* a = V + (int64_t)blockIdx.y * ld;
  Acc sr, si;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const cd p = VecTraits<T>::load(a, i), q = VecTraits<T>::load(x, i);
    sr.add(p.re * q.re + p.im * q.im);
    si.add(p.re * q.im - p.im * q.re);
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

// One CTA per vector: sum its kRedBlocks partials in a fixed order.  mode 0:
// the complex sum to out[2k], out[2k+1]; mode 1: out[0] = sqrt(Re sum) (a
// norm); mode 2: out[0] = 1 / sqrt(Re sum) (the normalising factor).
__global__ void __launch_bounds__(kRedThreads) k_dot_finish(const double* __restrict__ part, int nb,
                                                            double* __restrict__ out, int mode) {
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
      out[0] = sqrt(rr[0]);
    } else {
      out[0] = 1.0 / sqrt(rr[0]);
    }
  }
}

// y -= c x with a device scalar c: complex (c[0], c[1]) when cplx, else real c[0]
template <typename T>
__global__ void k_sub_scaled(T* __restrict__ y, const T* __restrict__ x, const double* __restrict__ c, bool cplx,
                             int64_t n) {
  const double cr = c[0], ci = cplx ? c[1] : 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const cd xv = VecTraits<T>::load(x, i);
    cd yv = VecTraits<T>::load(y, i);
    yv.re -= cr * xv.re - ci * xv.im;
    yv.im -= cr * xv.im + ci * xv.re;
    VecTraits<T>::store(y, i, yv);
  }
}

// y = s x with a real device scalar: s = c[0] (inv false) or 1 / c[0] (inv true)
template <typename T>
__global__ void k_scale_dev(T* __restrict__ y, const T* __restrict__ x, const double* __restrict__ c, bool inv,
                            int64_t n) {
  const double sc = inv ? 1.0 / c[0] : c[0];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    cd v = VecTraits<T>::load(x, i);
    v.re *= sc;
    v.im *= sc;
    VecTraits<T>::store(y, i, v);
  }
}

// y -= sum_k q_k V_k  (q: K complex on device)
template <typename T>
__global__ void k_sub_multi(T* __restrict__ y, const T* __restrict__ V, int64_t ld, const double* __restrict__ q,
                            int K, int64_t n) {
  extern __shared__ double sq[];
  for (int k = threadIdx.x; k < 2 * K; k += blockDim.x) sq[k] = q[k];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    cd yv = VecTraits<T>::load(y, i);
    for (int k = 0; k < K; ++k) {
      const cd vv = VecTraits<T>::load(V + (int64_t)k * ld, i);
      const double qr = sq[2 * k], qi = sq[2 * k + 1];
      yv.re -= qr * vv.re - qi * vv.im;
      yv.im -= qr * vv.im + qi * vv.re;
    }
    VecTraits<T>::store(y, i, yv);
  }
}

// out = sum_k c_k V_k with real coefficients c (device)
template <typename T>
__global__ void k_combine(T* __restrict__ out, const T* __restrict__ V, int64_t ld, const double* __restrict__ c,
                          int K, int64_t n) {
  extern __shared__ double sc[];
  for (int k = threadIdx.x; k < K; k += blockDim.x) sc[k] = c[k];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    cd r{0, 0};
    for (int k = 0; k < K; ++k) {
      const cd vv = VecTraits<T>::load(V + (int64_t)k * ld, i);
      r.re += sc[k] * vv.re;
      r.im += sc[k] * vv.im;
    }
    VecTraits<T>::store(out, i, r);
  }
}

int grid_of(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16)); }

// ------------------------------------------------------------ vector ops ---
// Every scalar of the recurrence (alpha, beta, the Gram-Schmidt coefficients,
// the normalising factors) is reduced into device memory and read there by
// the next kernel: a Lanczos step queues its kernels without waiting.
struct Blas {
  cudaStream_t st;
  double* part = nullptr;  // partials for up to kMaxDots vectors
  double* res = nullptr;   // finished dots of up to 2 kMaxDots vectors (device)
  double* scal = nullptr;  // small device scalars
  static constexpr int kMaxDots = 1024;
  cudaError_t init(cudaStream_t s) {
    st = s;
    cudaError_t e = cudaMalloc(&part, sizeof(double) * 2 * kRedBlocks * kMaxDots);
    if (e == cudaSuccess) e = cudaMalloc(&res, sizeof(double) * 4 * kMaxDots);
    if (e == cudaSuccess) e = cudaMalloc(&scal, sizeof(double) * 8);
    return e;
  }
  ~Blas() {
    cudaFree(part);
    cudaFree(res);
    cudaFree(scal);
  }
  // out[k] = <V_k | x> = sum conj(V_k) x for k < K (complex, device), all
  // computed before anything changes x
  template <typename T>
  void dots(const T* V, int64_t ld, int K, const T* x, int64_t n, double* out) {
    for (int k0 = 0; k0 < K; k0 += kMaxDots) {
      const int kk = std::min(kMaxDots, K - k0);
      k_dotc_partial<T><<<dim3(kRedBlocks, kk), kRedThreads, 0, st>>>(V + (int64_t)k0 * ld, ld, x, n, part);
      k_dot_finish<<<kk, kRedThreads, 0, st>>>(part, kRedBlocks, out + 2 * k0, 0);
    }
  }
  // out[0] = sqrt(<x|x>) (mode 1) or 1 / sqrt(<x|x>) (mode 2)
  template <typename T>
  void norm(const T* x, int64_t n, double* out, int mode) {
    k_dotc_partial<T><<<dim3(kRedBlocks, 1), kRedThreads, 0, st>>>(x, 0, x, n, part);
    k_dot_finish<<<1, kRedThreads, 0, st>>>(part, kRedBlocks, out, mode);
  }
  // y -= sum_k q_k V_k, q complex on the device
  template <typename T>
  void sub_multi(T* y, const T* V, int64_t ld, const double* q, int K, int64_t n) {
    for (int k0 = 0; k0 < K; k0 += kMaxDots) {
      const int kk = std::min(kMaxDots, K - k0);
      k_sub_multi<T><<<grid_of(n), 256, sizeof(double) * 2 * kk, st>>>(y, V + (int64_t)k0 * ld, ld, q + 2 * k0, kk,
                                                                        n);
    }
  }
};

// orth_wrt_previous_evecs (lanczos.cpp:57-74): classical Gram-Schmidt, all
// projections <V_k|v> first, then one subtraction pass.
void orth(Blas& B, double2* v, const double2* V, int64_t ld, int K, int64_t n) {
  if (K <= 0) return;
  B.dots(V, ld, K, v, n, B.res);
  B.sub_multi(v, V, ld, B.res, K, n);
}

// normalize (lanczos.cpp:50-55)
void normalize(Blas& B, double2* v, int64_t n) {
  B.norm(v, n, B.scal, 2);
  k_scale_dev<double2><<<grid_of(n), 256, 0, B.st>>>(v, v, B.scal, false, n);
}

void log_line(const edg_solver_opts& o, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
void log_line(const edg_solver_opts& o, const char* fmt, ...) {
  if (!o.log_fn) return;
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  o.log_fn(o.log_ctx, buf);
}

int solve_lanczos(Sector& S, const edg_solver_opts& o, double* eigs, int64_t cap, int64_t* n_out, double* evecs,
                  int64_t evecs_cap, edg_solver_stats* stats) {
  const int64_t n = S.P.n_p;
  const int how_many = (int)std::min<int64_t>(o.n_ev, n);
  if (how_many <= 0) return fail(EDG_ERR_INVALID, "n_ev must be positive");
  if (cap < how_many) return fail(EDG_ERR_INVALID, "eigs_capacity < n_ev");
  if (o.iterations <= 0 || o.ncycles <= 0) return fail(EDG_ERR_INVALID, "iterations and ncycles must be positive");
  // a cycle's Gram-Schmidt coefficients against its stored Krylov vectors sit
  // in a buffer of 2 kMaxDots complex values
  if (o.iterations > 2 * Blas::kMaxDots) return fail(EDG_ERR_UNSUPPORTED, "at most 2048 iterations per cycle");
  int iterations = o.iterations;
  cudaStream_t st = S.stream;
  Blas B;
  cudaError_t ce = B.init(st);
  if (ce != cudaSuccess) return fail(EDG_ERR_NOMEM, "Lanczos: scratch allocation");
  // device storage: v_p, w, the Krylov vectors of a cycle, earlier
  // eigenvectors, and T: alpha (complex), beta (beta[0] = 0, beta[j] the
  // off-diagonal T[j-1][j]), the Ritz coefficients y
  const int64_t max_it = std::min<int64_t>(iterations, n);
  double2 *vp = nullptr, *w = nullptr, *vs = nullptr, *prev = nullptr;
  double *alpha = nullptr, *beta = nullptr, *y = nullptr;
  TdScratch T;
  auto cleanup = [&]() {
    cudaFree(vp);
    cudaFree(w);
    cudaFree(vs);
    cudaFree(prev);
    cudaFree(alpha);
    cudaFree(beta);
    cudaFree(y);
  };
  ce = cudaMalloc(&vp, sizeof(double2) * n);
  if (ce == cudaSuccess) ce = cudaMalloc(&w, sizeof(double2) * n);
  if (ce == cudaSuccess) ce = cudaMalloc(&vs, sizeof(double2) * n * max_it);
  if (ce == cudaSuccess) ce = cudaMalloc(&prev, sizeof(double2) * n * how_many);
  if (ce == cudaSuccess) ce = cudaMalloc(&alpha, sizeof(double) * 2 * (max_it + 1));
  if (ce == cudaSuccess) ce = cudaMalloc(&beta, sizeof(double) * (max_it + 2));
  if (ce == cudaSuccess) ce = cudaMalloc(&y, sizeof(double) * (max_it + 1));
  if (ce == cudaSuccess) ce = T.reserve(1, (int)max_it, 1, 1);
  if (ce != cudaSuccess) {
    cleanup();
    return fail(EDG_ERR_NOMEM, "Lanczos: the stored Krylov vectors do not fit in device memory");
  }
  // the lowest eigenvalue of T_m (and with want_y its eigenvector, into y):
  // the device kernels of tridiag_dev.cu; only the eigenvalue comes back
  auto lowest = [&](int m, bool want_y, double& eig) -> cudaError_t {
    TdProb P{alpha, 2, beta, m, 1, 0, 1, 0, T.vals, y, T.work};
    cudaError_t e = cudaMemcpyAsync(T.probs, &P, sizeof P, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = td_select_async(T.probs, 1, m, 1, T.out, want_y, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&eig, &T.out->theta[0], sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
  };
  using clk = std::chrono::steady_clock;
  const auto t_start = clk::now();
  double t_hv = 0, t_ortho = 0;
  int64_t hv_calls = 0;
  std::vector<double> all_eigs;
  double eig0 = 0;
  cudaMemsetAsync(beta, 0, sizeof(double) * (max_it + 2), st);
  for (int num = 0; num < how_many; ++num) {
    iterations = (int)std::min<int64_t>(iterations, n - num);  // lanczos.cpp:188
    edg_fill_random(vp, n, EDG_C128, o.seed + (uint64_t)num, st);
    double previous_eig = 1000.0;
    for (int cycle = 0; cycle < o.ncycles; ++cycle) {
      orth(B, vp, prev, n, num, n);
      normalize(B, vp, n);
      int n_vs = 0;
      bool stop_cycle = false;
      for (int it = 0; it < iterations && !stop_cycle; ++it) {
        auto t0 = clk::now();
        if ((ce = launch_hv(S, vp, w, true, st)) != cudaSuccess) break;
        if ((ce = cudaStreamSynchronize(st)) != cudaSuccess) break;
        t_hv += std::chrono::duration<double>(clk::now() - t0).count();
        ++hv_calls;
        // w -= beta_it v_{it-1}; alpha = conj(zdotc(w, v_p)) = <v_p|w> (lanczos.cpp:237-238)
        if (it != 0) k_sub_scaled<double2><<<grid_of(n), 256, 0, st>>>(w, vs + (int64_t)(it - 1) * n, beta + it,
                                                                       false, n);
        B.dots(vp, 0, 1, w, n, alpha + 2 * it);
        k_sub_scaled<double2><<<grid_of(n), 256, 0, st>>>(w, vp, alpha + 2 * it, true, n);
        cudaMemcpyAsync(vs + (int64_t)n_vs * n, vp, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st);
        ++n_vs;
        B.norm(w, n, beta + it + 1, 1);  // beta = |w|
        k_scale_dev<double2><<<grid_of(n), 256, 0, st>>>(vp, w, beta + it + 1, true, n);  // v_p = w / beta
        auto t1 = clk::now();
        orth(B, vp, prev, n, num, n);
        if (cycle == o.ncycles - 1) orth(B, vp, vs, n, n_vs, n);
        normalize(B, vp, n);
        // lowest eigenvalue of T (diagonal Re(alpha), off-diagonal beta), on the device
        if ((ce = lowest(it + 1, false, eig0)) != cudaSuccess) break;
        t_ortho += std::chrono::duration<double>(clk::now() - t1).count();
        if (cycle != 0 && cycle != o.ncycles - 1 && it > 1) {
          log_line(o, "Eigs[0]      = %+.15f", eig0);
          log_line(o, "Previous Eig = %+.15f", previous_eig);
          if (std::fabs(eig0 - previous_eig) < o.tol) {
            log_line(o, "Convergence, doing last cycle with orth !!");
            stop_cycle = true;           // it = iterations  (lanczos.cpp:293)
            cycle = o.ncycles - 2;       // next cycle is the last one
          }
          previous_eig = eig0;
        } else if (cycle == o.ncycles - 1) {
          log_line(o, "Final cycle, Eigs[0]      = %+.15f", eig0);
        } else {
          log_line(o, "Eigs[0]      = %+.15f", eig0);
          log_line(o, "Previous Eig = %+.15f", previous_eig);
          previous_eig = eig0;
        }
      }
      if (ce != cudaSuccess) break;
      // Ritz vector from the stored Krylov vectors (lanczos.cpp:311-320): the
      // eigenvector of T on the device, then v_p = sum_k y_k vs_k
      double th = 0;
      if ((ce = lowest(n_vs, true, th)) != cudaSuccess) break;
      k_combine<double2><<<grid_of(n), 256, sizeof(double) * n_vs, st>>>(vp, vs, n, y, n_vs, n);
      orth(B, vp, prev, n, num, n);
      normalize(B, vp, n);
    }
    if (ce != cudaSuccess) break;
    cudaMemcpyAsync(prev + (int64_t)num * n, vp, sizeof(double2) * n, cudaMemcpyDeviceToDevice, st);
    log_line(o, "Eigenvalue number %d = %+.15f", num, eig0);
    all_eigs.push_back(eig0);
  }
  if (ce == cudaSuccess) ce = cudaGetLastError();
  if (ce == cudaSuccess && evecs && evecs_cap > 0) {
    const int64_t nv = std::min<int64_t>(evecs_cap, how_many);
    ce = cudaMemcpyAsync(evecs, prev, sizeof(double2) * n * nv, cudaMemcpyDeviceToHost, st);
  }
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
  cleanup();
  if (ce != cudaSuccess) return cuda_fail(ce, "Lanczos");
  for (size_t k = 0; k < all_eigs.size(); ++k) eigs[k] = all_eigs[k];
  *n_out = (int64_t)all_eigs.size();
  if (stats) {
    stats->path = 0;
    stats->hv_calls = hv_calls;
    stats->hv_seconds = t_hv;
    stats->ortho_seconds = t_ortho;
    stats->total_seconds = std::chrono::duration<double>(clk::now() - t_start).count();
  }
  return EDG_OK;
}

}  // namespace

int solve_plain(Sector& S, const edg_solver_opts& o, double* eigs, int64_t cap, int64_t* n_out, double* evecs,
                int64_t evecs_cap, edg_solver_stats* stats) {
  if (stats) std::memset(stats, 0, sizeof(*stats));
  if (o.dense_threshold >= 0 && S.P.n_p <= o.dense_threshold)
    return solve_dense_device(S, eigs, cap, n_out, evecs, evecs_cap, stats);
  return solve_lanczos(S, o, eigs, cap, n_out, evecs, evecs_cap, stats);
}

}  // namespace edg
