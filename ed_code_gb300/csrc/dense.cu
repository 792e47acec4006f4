// The reference's dense small-sector path on the device: exact_evecs
// (lanczos.cpp:81-131) on the matrix makeH builds (H_v.cpp:21-190), used by
// sector_lanczos for n_p <= 10000 (Lanczos_sector.cpp:105-120).
//
//   1. H assembled in one kernel from the stored rows: per nonzero
//      norm_i * value * norm_inv_j (the same matrix elements the stored-row
//      H*v uses), Ezz_i on the diagonal; without stored rows, column j is
//      H e_j from the matrix-free kernel.  Only the upper triangle is used,
//      as zheev('V','U') does (Matrix_Functions.cpp:39-40).
//   2. Householder reduction to a real symmetric tridiagonal T = Q^H H Q
//      (Golub and Van Loan, "Matrix Computations", sec. 8.3.1, for complex
//      Hermitian matrices: H_k = I - tau_k v_k v_k^H with a complex tau_k
//      that makes the sub-diagonal real).  Step k: the reflector of column k,
//      p = tau A22 v, w = p - (tau/2)(p^H v) v, and the rank-2 update
//      A22 -= v w^H + w v^H, four kernels.
//   3. All n eigenvalues of T, one thread each: bisection on FP32 Sturm
//      counts to about 1e-7 of |T|, then Newton's method on det(T - x I) in
//      FP64 (three-term recurrence for the determinant and its derivative,
//      rescaled by powers of two), checked with FP64 Sturm counts at
//      x -+ 4 eps |T|; an eigenvalue that fails the check (a multiple or a
//      tightly clustered root) is bisected in FP64 instead.  Bisection on all
//      n eigenvalues in FP64 alone would take ~50 n FP64 passes per
//      eigenvalue, and GB300 runs FP64 at 1/64 of its FP32 rate.
//   4. The wanted eigenvectors: inverse iteration on T (tridiag.cuh;
//      orthogonalised within clusters of equal eigenvalues), then x = Q y by
//      applying the reflectors from the last to the first.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/edgpu.h"
#include "blas1.cuh"
#include "edg_sector.cuh"
#include "tridiag.cuh"

namespace edg {

int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

namespace {

constexpr int kDenseThreads = 256;

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cconjmul(double2 a, double2 b) {  // conj(a) * b
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}

// H[j*n + i] += H_ij from the stored rows (one thread per row i)
__global__ void k_dense_rows(const uint64_t* __restrict__ row_ptr, const uint32_t* __restrict__ col,
                             const uint16_t* __restrict__ vid, int cb, const double2* __restrict__ vtab,
                             const double* __restrict__ ezz, const uint8_t* __restrict__ lid,
                             const double* __restrict__ nrm, const double* __restrict__ nrm_inv, int64_t n,
                             double2* __restrict__ H) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double ni = nrm[lid[i]];
    for (uint64_t t = row_ptr[i]; t < row_ptr[i + 1]; ++t) {
      const uint32_t e = col[t];
      uint32_t j;
      int id;
      if (vid) {
        j = e;
        id = vid[t];
      } else {
        j = e & ((1u << cb) - 1u);
        id = (int)(e >> cb);
      }
      const double2 c = vtab[id];
      const double s = ni * nrm_inv[lid[j]];
      double2* h = H + (int64_t)j * n + i;
      h->x += c.x * s;
      h->y += c.y * s;
    }
    H[i * n + i].x += ezz[i];
  }
}

__global__ void k_unit_col(double2* e, int64_t n, int64_t j) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    e[i] = make_double2(i == j ? 1.0 : 0.0, 0.0);
}

// A Hermitian from its upper triangle: A_rc = conj(A_cr) for r > c, real diagonal
__global__ void k_herm_upper(double2* __restrict__ A, int64_t n) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
  if (r >= n) return;
  if (r > c) {
    const double2 u = A[r * n + c];  // (c, r), c < r: upper
    A[c * n + r] = make_double2(u.x, -u.y);
  } else if (r == c) {
    A[c * n + c].y = 0.0;
  }
}

__device__ double block_sum(double x, double* sh) {
  sh[threadIdx.x] = x;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) sh[threadIdx.x] += sh[threadIdx.x + h];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

// Step k, part 1 (one CTA): the reflector of column k below the diagonal,
// x = A[k+1.., k] -> v = (1, x_1/(alpha - beta), ...), stored in place;
// d[k], e[k] = beta, tau[k].
__global__ void __launch_bounds__(kDenseThreads) k_hh_reflect(double2* __restrict__ A, int64_t n, int64_t k,
                                                              double* __restrict__ d, double* __restrict__ e,
                                                              double2* __restrict__ tau) {
  __shared__ double sh[kDenseThreads];
  __shared__ double2 inv;
  __shared__ int apply;
  const int64_t m = n - k - 1;
  double2* x = A + k * n + (k + 1);
  double s = 0.0;
  for (int64_t i = 1 + threadIdx.x; i < m; i += blockDim.x) s += x[i].x * x[i].x + x[i].y * x[i].y;
  s = block_sum(s, sh);
  if (threadIdx.x == 0) {
    d[k] = A[k * n + k].x;
    const double2 alpha = x[0];
    double2 t = make_double2(0.0, 0.0);
    double beta = alpha.x;
    apply = 0;
    if (s != 0.0 || alpha.y != 0.0) {
      beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + s), alpha.x);
      t = make_double2((beta - alpha.x) / beta, -alpha.y / beta);
      const double zr = alpha.x - beta, zi = alpha.y, z2 = zr * zr + zi * zi;
      inv = make_double2(zr / z2, -zi / z2);
      apply = 1;
    }
    e[k] = beta;
    tau[k] = t;
  }
  __syncthreads();
  if (apply)
    for (int64_t i = 1 + threadIdx.x; i < m; i += blockDim.x) x[i] = cmul(x[i], inv);
  __syncthreads();
  if (threadIdx.x == 0) x[0] = make_double2(1.0, 0.0);
}

// Step k, part 2: p_i = tau (A22 v)_i = tau sum_j conj(A22[j][i]) v_j, a warp
// per column i of A22 (A22 is Hermitian, its columns are contiguous)
__global__ void __launch_bounds__(kDenseThreads) k_hh_p(const double2* __restrict__ A, int64_t n, int64_t k,
                                                        const double2* __restrict__ tau, double2* __restrict__ p) {
  const int64_t m = n - k - 1;
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= m) return;
  const double2 t = tau[k];
  if (t.x == 0.0 && t.y == 0.0) {
    if (lane == 0) p[i] = make_double2(0.0, 0.0);
    return;
  }
  const double2* ci = A + (k + 1 + i) * n + (k + 1);
  const double2* v = A + k * n + (k + 1);
  double sr = 0.0, si = 0.0;
  for (int64_t j = lane; j < m; j += 32) {
    const double2 a = ci[j], b = v[j];
    sr += a.x * b.x + a.y * b.y;
    si += a.x * b.y - a.y * b.x;
  }
  for (int o = 16; o > 0; o >>= 1) {
    sr += __shfl_down_sync(0xffffffffu, sr, o);
    si += __shfl_down_sync(0xffffffffu, si, o);
  }
  if (lane == 0) p[i] = cmul(t, make_double2(sr, si));
}

// Step k, part 3 (one CTA): w = p - (tau/2) (p^H v) v
__global__ void __launch_bounds__(kDenseThreads) k_hh_w(const double2* __restrict__ A, int64_t n, int64_t k,
                                                        const double2* __restrict__ tau,
                                                        const double2* __restrict__ p, double2* __restrict__ w) {
  __shared__ double sh[kDenseThreads];
  const int64_t m = n - k - 1;
  const double2* v = A + k * n + (k + 1);
  double sr = 0.0, si = 0.0;
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
    const double2 q = cconjmul(p[i], v[i]);
    sr += q.x;
    si += q.y;
  }
  sr = block_sum(sr, sh);
  si = block_sum(si, sh);
  const double2 t = tau[k];
  const double2 K = cmul(make_double2(-0.5 * t.x, -0.5 * t.y), make_double2(sr, si));
  for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
    const double2 kv = cmul(K, v[i]);
    w[i] = make_double2(p[i].x + kv.x, p[i].y + kv.y);
  }
}

// Step k, part 4: A22 -= v w^H + w v^H (real diagonal kept)
__global__ void k_hh_rank2(double2* __restrict__ A, int64_t n, int64_t k, const double2* __restrict__ tau,
                           const double2* __restrict__ w) {
  const int64_t m = n - k - 1;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
  if (i >= m) return;
  const double2 t = tau[k];
  if (t.x == 0.0 && t.y == 0.0) return;
  const double2* v = A + k * n + (k + 1);
  const double2 vi = v[i], vj = v[j], wi = w[i], wj = w[j];
  double2& a = A[(k + 1 + j) * n + (k + 1 + i)];
  // v_i conj(w_j) + w_i conj(v_j)
  const double2 u1 = cconjmul(wj, vi), u2 = cconjmul(vj, wi);
  a.x -= u1.x + u2.x;
  a.y = i == j ? 0.0 : a.y - (u1.y + u2.y);
}

__global__ void k_last_diag(const double2* __restrict__ A, int64_t n, double* __restrict__ d) {
  d[n - 1] = A[(n - 1) * n + (n - 1)].x;
}

// ---- eigenvalues of T: d[0..n-1], off-diagonal e[0..n-2] (row i to i+1) ----

// eigenvalues of T below x, FP32 Sturm count (pivots q_i; a tiny pivot counts as negative)
__device__ int count32(const float* d, const float* e2, int n, float x, float pivmin) {
  int c = 0;
  float q = d[0] - x;
  if (fabsf(q) < pivmin) q = -pivmin;
  c += q < 0.f;
  for (int i = 1; i < n; ++i) {
    q = d[i] - x - e2[i - 1] / q;
    if (fabsf(q) < pivmin) q = -pivmin;
    c += q < 0.f;
  }
  return c;
}

// the same count in FP64 from the signs of the leading minors p_i = det(T_i - x),
// p_i = (d_i - x) p_{i-1} - e_{i-1}^2 p_{i-2}, rescaled by powers of two; a zero
// minor counts as a sign change (as a tiny negative pivot would)
__device__ int count64(const double* d, const double* e2, int n, double x) {
  int c = 0;
  double pm = 1.0, p = d[0] - x;
  c += p <= 0.0;
  if (p == 0.0) p = -1e-300;
  for (int i = 1; i < n; ++i) {
    double pn = (d[i] - x) * p - e2[i - 1] * pm;
    if (pn == 0.0) pn = p > 0 ? -1e-300 * fabs(p) : 1e-300 * fabs(p);
    c += (pn < 0.0) != (p < 0.0);
    pm = p;
    p = pn;
    const double ap = fabs(p);
    if (ap > 0x1p500) {
      p *= 0x1p-500;
      pm *= 0x1p-500;
    } else if (ap < 0x1p-500 && fabs(pm) < 0x1p-500) {
      p *= 0x1p500;
      pm *= 0x1p500;
    }
  }
  return c;
}

// one Newton step on det(T - x): returns det / det' (rescaled consistently)
__device__ double newton_step(const double* d, const double* e2, int n, double x) {
  double pm = 1.0, p = d[0] - x, dpm = 0.0, dp = -1.0;
  for (int i = 1; i < n; ++i) {
    const double a = d[i] - x;
    const double pn = a * p - e2[i - 1] * pm;
    const double dpn = a * dp - p - e2[i - 1] * dpm;
    pm = p;
    p = pn;
    dpm = dp;
    dp = dpn;
    const double big = fmax(fabs(p), fabs(dp));
    if (big > 0x1p500) {
      p *= 0x1p-500;
      pm *= 0x1p-500;
      dp *= 0x1p-500;
      dpm *= 0x1p-500;
    } else if (big < 0x1p-500 && fmax(fabs(pm), fabs(dpm)) < 0x1p-500) {
      p *= 0x1p500;
      pm *= 0x1p500;
      dp *= 0x1p500;
      dpm *= 0x1p500;
    }
  }
  return p / dp;
}

__global__ void k_tri_prep(const double* __restrict__ d, const double* __restrict__ e, int n, float* __restrict__ d32,
                           float* __restrict__ e232, double* __restrict__ e2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    d32[i] = (float)d[i];
    if (i + 1 < n) {
      e2[i] = e[i] * e[i];
      e232[i] = (float)e[i] * (float)e[i];
    }
  }
}

// eigenvalue k of T, one thread each; bounds [gl, gu] enclose the spectrum
__global__ void k_tri_all(const double* __restrict__ d, const double* __restrict__ e2, const float* __restrict__ d32,
                          const float* __restrict__ e232, int n, double gl, double gu, double tnorm,
                          double* __restrict__ out, int* __restrict__ n_fallback) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float pivf = 1e-30f;
  float lo = (float)gl, hi = (float)gu;
  for (int it = 0; it < 64; ++it) {
    const float mid = 0.5f * (lo + hi);
    if (!(mid > lo && mid < hi)) break;
    if (hi - lo <= 4.f * 1.1920929e-7f * fmaxf(fabsf(lo), fabsf(hi))) break;
    if (count32(d32, e232, n, mid, pivf) > k) hi = mid;
    else lo = mid;
  }
  const double width = (double)hi - (double)lo + 4e-7 * tnorm;
  double x = 0.5 * ((double)lo + (double)hi);
  bool ok = true;
  for (int it = 0; it < 6; ++it) {
    const double s = newton_step(d, e2, n, x);
    if (!isfinite(s) || fabs(s) > width) {
      ok = false;
      break;
    }
    x -= s;
    if (fabs(s) <= 2.2e-16 * fmax(fabs(x), 1e-300)) break;
  }
  const double delta = 4.0 * 2.220446049250313e-16 * fmax(fabs(x), tnorm);
  if (ok) ok = count64(d, e2, n, x - delta) <= k && count64(d, e2, n, x + delta) > k;
  if (!ok) {
    atomicAdd(n_fallback, 1);
    double a = (double)lo - width, b = (double)hi + width;
    if (!(count64(d, e2, n, a) <= k && count64(d, e2, n, b) > k)) {
      a = gl;
      b = gu;
    }
    for (int it = 0; it < 200; ++it) {
      const double mid = 0.5 * (a + b);
      if (!(mid > a && mid < b)) break;
      if (b - a <= 2.0 * 2.220446049250313e-16 * fmax(fabs(a), fabs(b))) break;
      if (count64(d, e2, n, mid) > k) b = mid;
      else a = mid;
    }
    x = 0.5 * (a + b);
  }
  out[k] = x;
}

// eigenvectors of T for lam[0..nv-1] (ascending), one thread in sequence:
// levels within 1e-9 |T| of each other are a cluster, orthogonalised
__global__ void k_tri_vectors(const double* __restrict__ d, const double* __restrict__ eoff, int n,
                              const double* __restrict__ lam, int nv, double tnorm, double* __restrict__ y,
                              double* __restrict__ wk) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  int c0 = 0;  // first level of the current cluster
  for (int q = 0; q < nv; ++q) {
    if (q > 0 && fabs(lam[q] - lam[q - 1]) > 1e-9 * fmax(tnorm, 1.0)) c0 = q;
    tridiag_eigenvector_ex(d, eoff, n, lam[q], y + (int64_t)q * n, wk, y + (int64_t)c0 * n, q - c0, q - c0);
  }
}

// x = Q y for nv vectors (one CTA each): Q = H_0 ... H_{n-2}, applied from the
// last reflector to the first; y real (n doubles), x complex
__global__ void __launch_bounds__(kDenseThreads) k_backtransform(const double2* __restrict__ A, int64_t n,
                                                                 const double2* __restrict__ tau,
                                                                 const double* __restrict__ y,
                                                                 double2* __restrict__ X) {
  __shared__ double sh[kDenseThreads];
  double2* x = X + (int64_t)blockIdx.x * n;
  const double* yq = y + (int64_t)blockIdx.x * n;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) x[i] = make_double2(yq[i], 0.0);
  __syncthreads();
  for (int64_t k = n - 2; k >= 0; --k) {
    const double2 t = tau[k];
    if (t.x == 0.0 && t.y == 0.0) continue;
    const int64_t m = n - k - 1;
    const double2* v = A + k * n + (k + 1);
    double2* z = x + (k + 1);
    double sr = 0.0, si = 0.0;
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
      const double2 q = cconjmul(v[i], z[i]);
      sr += q.x;
      si += q.y;
    }
    sr = block_sum(sr, sh);
    si = block_sum(si, sh);
    const double2 c = cmul(t, make_double2(sr, si));
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) {
      const double2 u = cmul(c, v[i]);
      z[i].x -= u.x;
      z[i].y -= u.y;
    }
    __syncthreads();
  }
}

int grid1(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 16)); }

}  // namespace

int solve_dense_device(Sector& S, double* eigs, int64_t cap, int64_t* n_out, double* evecs, int64_t evecs_cap,
                       edg_solver_stats* stats) {
  const int64_t n = S.P.n_p;
  if (cap < n) return fail(EDG_ERR_INVALID, "dense path returns all n_p eigenvalues: eigs_capacity too small");
  if (n > 46340) return fail(EDG_ERR_UNSUPPORTED, "dense path: sector too large");
  const int64_t nv = (evecs && evecs_cap > 0) ? std::min<int64_t>(evecs_cap, n) : 0;
  cudaStream_t st = S.stream;
  double2 *H = nullptr, *tau = nullptr, *pw = nullptr, *X = nullptr;
  double *d = nullptr, *e = nullptr, *e2 = nullptr, *lam = nullptr, *y = nullptr, *wk = nullptr;
  float* f32 = nullptr;
  int* nfb = nullptr;
  auto cleanup = [&]() {
    void* p[] = {H, tau, pw, X, d, e, e2, lam, y, wk, f32, nfb};
    for (void* q : p)
      if (q) cudaFree(q);
  };
  cudaError_t ce = cudaMalloc(&H, sizeof(double2) * n * n);
  if (ce == cudaSuccess) ce = cudaMalloc(&tau, sizeof(double2) * n);
  if (ce == cudaSuccess) ce = cudaMalloc(&pw, sizeof(double2) * 2 * n);
  if (ce == cudaSuccess) ce = cudaMalloc(&d, sizeof(double) * n);
  if (ce == cudaSuccess) ce = cudaMalloc(&e, sizeof(double) * n);
  if (ce == cudaSuccess) ce = cudaMalloc(&e2, sizeof(double) * n);
  if (ce == cudaSuccess) ce = cudaMalloc(&lam, sizeof(double) * n);
  if (ce == cudaSuccess) ce = cudaMalloc(&f32, sizeof(float) * 2 * n);
  if (ce == cudaSuccess) ce = cudaMalloc(&nfb, sizeof(int));
  if (ce == cudaSuccess && nv > 0) ce = cudaMalloc(&X, sizeof(double2) * n * nv);
  if (ce == cudaSuccess && nv > 0) ce = cudaMalloc(&y, sizeof(double) * n * nv);
  if (ce == cudaSuccess && nv > 0) ce = cudaMalloc(&wk, sizeof(double) * 5 * n);
  if (ce != cudaSuccess) {
    cleanup();
    return fail(EDG_ERR_NOMEM, "dense path: out of device memory");
  }
  using clk = std::chrono::steady_clock;
  const auto t0 = clk::now();
  // 1. H
  cudaMemsetAsync(H, 0, sizeof(double2) * n * n, st);
  cudaMemsetAsync(nfb, 0, sizeof(int), st);
  int64_t hv_calls = 0;
  if (S.col) {
    const double* nrm = reinterpret_cast<const double*>(reinterpret_cast<const char*>(S.dP) +
                                                        offsetof(SectorParams, nrm));
    const double* nrm_inv = reinterpret_cast<const double*>(reinterpret_cast<const char*>(S.dP) +
                                                            offsetof(SectorParams, nrm_inv));
    k_dense_rows<<<grid1(n), 256, 0, st>>>(S.row_ptr, S.col, S.vid, S.pack_cb, S.vtab64, S.ezz, S.lid, nrm, nrm_inv,
                                           n, H);
  } else {
    for (int64_t j = 0; j < n && ce == cudaSuccess; ++j) {
      k_unit_col<<<grid1(n), 256, 0, st>>>(pw, n, j);
      ce = launch_hv(S, pw, H + j * n, true, st);
      ++hv_calls;
    }
  }
  if (ce == cudaSuccess) ce = cudaGetLastError();
  if (ce != cudaSuccess) {
    cleanup();
    return cuda_fail(ce, "dense path: assembling H");
  }
  const auto t1 = clk::now();
  // 2. Householder tridiagonalisation
  k_herm_upper<<<dim3((unsigned)((n + 255) / 256), (unsigned)n), 256, 0, st>>>(H, n);
  for (int64_t k = 0; k + 1 < n; ++k) {
    const int64_t m = n - k - 1;
    k_hh_reflect<<<1, kDenseThreads, 0, st>>>(H, n, k, d, e, tau);
    k_hh_p<<<(unsigned)((m * 32 + kDenseThreads - 1) / kDenseThreads), kDenseThreads, 0, st>>>(H, n, k, tau, pw);
    k_hh_w<<<1, kDenseThreads, 0, st>>>(H, n, k, tau, pw, pw + n);
    k_hh_rank2<<<dim3((unsigned)((m + 127) / 128), (unsigned)m), 128, 0, st>>>(H, n, k, tau, pw + n);
  }
  k_last_diag<<<1, 1, 0, st>>>(H, n, d);
  // 3. eigenvalues: Gershgorin bounds of T on the host (2n doubles)
  std::vector<double> dh(n), eh(n, 0.0);
  cudaMemcpyAsync(dh.data(), d, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
  if (n > 1) cudaMemcpyAsync(eh.data(), e, sizeof(double) * (n - 1), cudaMemcpyDeviceToHost, st);
  if ((ce = cudaStreamSynchronize(st)) != cudaSuccess) {
    cleanup();
    return cuda_fail(ce, "dense path: tridiagonalisation");
  }
  double gl = dh[0], gu = dh[0], tnorm = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    const double r = (i > 0 ? std::fabs(eh[i - 1]) : 0.0) + (i + 1 < n ? std::fabs(eh[i]) : 0.0);
    gl = std::min(gl, dh[i] - r);
    gu = std::max(gu, dh[i] + r);
    tnorm = std::max(tnorm, std::fabs(dh[i]) + r);
  }
  const double pad = 1e-6 * std::max(tnorm, 1.0);
  gl -= pad;
  gu += pad;
  k_tri_prep<<<grid1(n), 256, 0, st>>>(d, e, (int)n, f32, f32 + n, e2);
  k_tri_all<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(d, e2, f32, f32 + n, (int)n, gl, gu, tnorm, lam, nfb);
  // 4. eigenvectors
  if (nv > 0) {
    // off-diagonal in the tridiag.cuh convention: eoff[i] couples rows i-1 and i
    double* eoff = e2;  // e2 is no longer needed once the eigenvalues are in
    cudaMemsetAsync(eoff, 0, sizeof(double), st);
    if (n > 1) cudaMemcpyAsync(eoff + 1, e, sizeof(double) * (n - 1), cudaMemcpyDeviceToDevice, st);
    k_tri_vectors<<<1, 1, 0, st>>>(d, eoff, (int)n, lam, (int)nv, tnorm, y, wk);
    k_backtransform<<<(unsigned)nv, kDenseThreads, 0, st>>>(H, n, tau, y, X);
  }
  std::vector<double> out(n);
  int fallbacks = 0;  // eigenvalues that needed FP64 bisection (multiple or clustered roots)
  cudaMemcpyAsync(out.data(), lam, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(&fallbacks, nfb, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (nv > 0) cudaMemcpyAsync(evecs, X, sizeof(double2) * n * nv, cudaMemcpyDeviceToHost, st);
  ce = cudaStreamSynchronize(st);
  if (ce == cudaSuccess) ce = cudaGetLastError();
  cleanup();
  if (ce != cudaSuccess) return cuda_fail(ce, "dense path");
  // bisection and Newton give the k-th eigenvalue at index k; neighbours
  // within rounding may come out in either order
  std::sort(out.begin(), out.end());
  for (int64_t i = 0; i < n; ++i) eigs[i] = out[i];
  *n_out = n;
  if (stats) {
    stats->path = 1;
    stats->hv_calls = hv_calls;
    stats->hv_seconds = std::chrono::duration<double>(t1 - t0).count();
    stats->ortho_seconds = 0.0;
    stats->total_seconds = std::chrono::duration<double>(clk::now() - t0).count();
  }
  return EDG_OK;
}

}  // namespace edg
