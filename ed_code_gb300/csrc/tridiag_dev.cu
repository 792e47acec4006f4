// The Lanczos T matrix's eigenproblem on the device.
//
// The reference diagonalises the whole T with LAPACK zheev after every step
// (lanczos.cpp:271-286, Matrix_Functions.cpp:28-48) and uses the lowest
// eigenvalue and, at the end of a cycle, its eigenvector.  Here T stays where
// the Lanczos recurrence wrote it (device memory) and three kernels work on a
// batch of problems at once (one problem: one T, blockIdx.y):
//
//   k_td_values   eigenvalues k of T and of T-hat (T without its first row and
//                 column), one warp each: multisection on the Sturm count --
//                 the 32 lanes evaluate the count at 32 interior points of the
//                 bracket and keep the sub-interval where it passes k, 33x
//                 narrower per round (Barth, Martin and Wilkinson's bisection,
//                 Numer. Math. 9 (1967) 386, with the points spread over a warp);
//   k_td_pick     the Ritz values kept: with filtering, Cullum and
//                 Willoughby's test drops a simple eigenvalue of T that T-hat
//                 shares (a copy made by lost orthogonality) and keeps one
//                 value per cluster; without it, the lowest `want`;
//   k_td_vectors  their eigenvectors, one thread each, by inverse iteration
//                 (tridiag.cuh).
//
// Every step is deterministic; results do not depend on the other problems in
// the batch.  All arithmetic is FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "edg_sector.cuh"
#include "lanczos_common.cuh"
#include "tridiag.cuh"

namespace edg {

int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

namespace {

constexpr int kTdWarps = 8;

// d[i] = Re alpha_i (alpha strided by astride doubles), e[i] = beta_i (e[0] = 0)
__device__ void load_t(const TdProb& P, double* d, double* e) {
  for (int i = threadIdx.x; i < P.m; i += blockDim.x) {
    d[i] = P.alpha[(int64_t)i * P.astride];
    e[i] = i > 0 ? P.beta[i] : 0.0;
  }
}

__global__ void __launch_bounds__(32 * kTdWarps) k_td_values(const TdProb* __restrict__ probs) {
  const TdProb P = probs[blockIdx.y];
  extern __shared__ double sm[];
  double* d = sm;
  double* e = sm + P.m;
  const int idx = blockIdx.x * kTdWarps + (threadIdx.x >> 5);
  if (blockIdx.x * kTdWarps >= P.nc + P.nh) return;  // the whole CTA has no work
  load_t(P, d, e);
  __syncthreads();
  if (idx < P.nc) {
    const double th = warp_eigenvalue(d, e, P.m, idx);
    if ((threadIdx.x & 31) == 0) P.vals[idx] = th;
  } else if (idx < P.nc + P.nh) {
    const double th = warp_eigenvalue(d + 1, e + 1, P.m - 1, idx - P.nc);
    if ((threadIdx.x & 31) == 0) P.vals[idx] = th;
  }
}

// One warp per problem.  |T| is the largest absolute row sum.  Copies of a
// converged level built from FP32 vectors agree only to about the FP32
// backward error, ~1e-7 |T| (one is kept per such cluster); T and T-hat share
// a spurious value to FP64 accuracy (within 1e-10 |T|).
__global__ void __launch_bounds__(32) k_td_pick(const TdProb* __restrict__ probs, TdOut* __restrict__ out) {
  const TdProb P = probs[blockIdx.x];
  double s = 0.0;
  for (int i = threadIdx.x; i < P.m; i += 32) {
    const double ei = i > 0 ? fabs(P.beta[i]) : 0.0, en = i + 1 < P.m ? fabs(P.beta[i + 1]) : 0.0;
    s = fmax(s, fabs(P.alpha[(int64_t)i * P.astride]) + ei + en);
  }
  for (int o = 16; o > 0; o >>= 1) s = fmax(s, __shfl_down_sync(0xffffffffu, s, o));
  if (threadIdx.x != 0) return;
  TdOut& O = out[blockIdx.x];
  const double* th = P.vals;
  const double* hat = P.vals + P.nc;
  int na = 0;
  if (!P.filter) {
    for (int k = 0; k < P.nc && na < P.want; ++k) {
      O.acc[na] = k;
      O.theta[na++] = th[k];
    }
  } else {
    const double scale = fmax(s, 1.0);
    const double tol_cluster = 1e-7 * scale, tol_hat = 1e-10 * scale;
    for (int k = 0; k < P.nc && na < P.want; ++k) {
      const bool prev_close = k > 0 && fabs(th[k] - th[k - 1]) < tol_cluster;
      const bool next_close = k + 1 < P.nc && fabs(th[k + 1] - th[k]) < tol_cluster;
      bool in_hat = false;
      for (int q = 0; q < P.nh; ++q)
        if (fabs(hat[q] - th[k]) < tol_hat) in_hat = true;
      if (in_hat && !prev_close && !next_close) continue;  // spurious copy
      if (prev_close) continue;                            // one per cluster
      O.acc[na] = k;
      O.theta[na++] = th[k];
    }
  }
  O.na = na;
}

__global__ void __launch_bounds__(64) k_td_vectors(const TdProb* __restrict__ probs, const TdOut* __restrict__ out) {
  const TdProb P = probs[blockIdx.x];
  extern __shared__ double sm[];
  double* d = sm;
  double* e = sm + P.m;
  load_t(P, d, e);
  __syncthreads();
  const int q = threadIdx.x;
  if (q < out[blockIdx.x].na)
    tridiag_eigenvector(d, e, P.m, out[blockIdx.x].theta[q], P.y + (int64_t)q * P.m,
                        P.work + (int64_t)q * 5 * P.m);
}

}  // namespace

cudaError_t td_select_async(const TdProb* probs_dev, int n_probs, int m_max, int nvals_max, TdOut* out_dev,
                            bool vectors, cudaStream_t st) {
  if (n_probs <= 0) return cudaSuccess;
  const size_t smem = sizeof(double) * 2 * std::max(m_max, 1);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_td_values, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_td_vectors, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  const int gx = (std::max(nvals_max, 1) + kTdWarps - 1) / kTdWarps;
  k_td_values<<<dim3(gx, n_probs), 32 * kTdWarps, smem, st>>>(probs_dev);
  k_td_pick<<<n_probs, 32, 0, st>>>(probs_dev, out_dev);
  if (vectors) k_td_vectors<<<n_probs, 64, smem, st>>>(probs_dev, out_dev);
  return cudaGetLastError();
}

int ritz_select_device(const double* alpha, const double* beta, int m, int want, int n_cand, double* y_dev,
                       cudaStream_t st, TdOut& sel) {
  const int nc = std::min(m, std::max(n_cand, want)), nh = std::min(m - 1, nc + 2);
  TdScratch T;
  cudaError_t e = T.reserve(1, m, nc + std::max(nh, 0), want);
  if (e != cudaSuccess) return fail(EDG_ERR_NOMEM, "Ritz selection: scratch");
  TdProb P{alpha, 1, beta, m, nc, std::max(nh, 0), want, 1, T.vals, y_dev, T.work};
  if ((e = cudaMemcpyAsync(T.probs, &P, sizeof P, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = td_select_async(T.probs, 1, m, nc + P.nh, T.out, true, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(&sel, T.out, sizeof sel, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return cuda_fail(e, "Ritz selection on the device");
  return EDG_OK;
}

TdScratch::~TdScratch() {
  void* p[] = {probs, out, vals, work};
  for (void* q : p)
    if (q) cudaFree(q);
}

cudaError_t TdScratch::reserve(int n_probs, int m_max, int nvals_max, int want_max) {
  auto grow = [](void** ptr, size_t bytes, size_t& have) -> cudaError_t {
    if (bytes <= have) return cudaSuccess;
    if (*ptr) cudaFree(*ptr);
    *ptr = nullptr;
    have = 0;
    const cudaError_t e = cudaMalloc(ptr, bytes);
    if (e == cudaSuccess) have = bytes;
    return e;
  };
  cudaError_t e = grow((void**)&probs, sizeof(TdProb) * n_probs, probs_b);
  if (e == cudaSuccess) e = grow((void**)&out, sizeof(TdOut) * n_probs, out_b);
  if (e == cudaSuccess) e = grow((void**)&vals, sizeof(double) * (size_t)n_probs * std::max(nvals_max, 1), vals_b);
  if (e == cudaSuccess)
    e = grow((void**)&work, sizeof(double) * 5 * (size_t)n_probs * std::max(m_max, 1) * std::max(want_max, 1),
             work_b);
  return e;
}

}  // namespace edg

// Test and utility entry point: the k lowest eigenpairs of one real symmetric
// tridiagonal matrix, computed by the device kernels above; with copy_filter
// the Ritz values the mixed solver keeps (Cullum-Willoughby test over the
// lowest kCand eigenvalues).
extern "C" int edg_tridiag_lowest(const double* d, const double* e, int m, int k, int copy_filter, double* eigs,
                                  double* vecs, int* n_out) {
  using namespace edg;
  if (!d || !eigs || !n_out || m < 1 || (m > 1 && !e)) return fail(EDG_ERR_INVALID, "edg_tridiag_lowest: bad arguments");
  if (k < 1 || k > kMaxEv || k > m) return fail(EDG_ERR_INVALID, "edg_tridiag_lowest: need 1 <= k <= min(m, 32)");
  if (m > 4096) return fail(EDG_ERR_UNSUPPORTED, "edg_tridiag_lowest: at most 4096 rows");
  const int nc = copy_filter ? std::min(m, std::max(kCand, k)) : k;
  const int nh = copy_filter ? std::max(0, std::min(m - 1, nc + 2)) : 0;
  cudaStream_t st = nullptr;
  cudaError_t ce = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (ce != cudaSuccess) return cuda_fail(ce, "edg_tridiag_lowest: stream");
  double *dd = nullptr, *y = nullptr;
  TdScratch T;
  int rc = EDG_OK;
  std::vector<double> bh(m, 0.0);
  for (int i = 1; i < m; ++i) bh[i] = e[i];
  ce = cudaMalloc(&dd, sizeof(double) * 2 * m);
  if (ce == cudaSuccess) ce = cudaMalloc(&y, sizeof(double) * (size_t)k * m);
  if (ce == cudaSuccess) ce = T.reserve(1, m, nc + nh, k);
  if (ce != cudaSuccess) rc = fail(EDG_ERR_NOMEM, "edg_tridiag_lowest: device memory");
  TdOut o{};
  if (rc == EDG_OK) {
    TdProb P{dd, 1, dd + m, m, nc, nh, k, copy_filter ? 1 : 0, T.vals, y, T.work};
    if ((ce = cudaMemcpyAsync(dd, d, sizeof(double) * m, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(dd + m, bh.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(T.probs, &P, sizeof P, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (ce = td_select_async(T.probs, 1, m, nc + nh, T.out, vecs != nullptr, st)) != cudaSuccess ||
        (ce = cudaMemcpyAsync(&o, T.out, sizeof o, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
      rc = cuda_fail(ce, "edg_tridiag_lowest");
    if (rc == EDG_OK && vecs &&
        (ce = cudaMemcpyAsync(vecs, y, sizeof(double) * (size_t)k * m, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
      rc = cuda_fail(ce, "edg_tridiag_lowest: vectors");
    if (rc == EDG_OK && (ce = cudaStreamSynchronize(st)) != cudaSuccess) rc = cuda_fail(ce, "edg_tridiag_lowest");
  }
  if (rc == EDG_OK) {
    for (int q = 0; q < o.na; ++q) eigs[q] = o.theta[q];
    *n_out = o.na;
  }
  cudaFree(dd);
  cudaFree(y);
  cudaStreamDestroy(st);
  return rc;
}
