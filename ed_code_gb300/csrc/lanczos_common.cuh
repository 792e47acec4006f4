// Ritz selection of the Lanczos T matrix on the device (tridiag_dev.cu),
// shared by the single-sector solvers and the batch.
#pragma once
#include <cuda_runtime.h>

#include "tridiag.cuh"

namespace edg {

constexpr int kMaxEv = 32;             // Ritz pairs returned
constexpr int kCand = 2 * kMaxEv + 8;  // eigenvalues of T examined when copies are many

// One tridiagonal problem for the device kernels (tridiag_dev.cu).  T has
// diagonal alpha[i * astride] (the real part when alpha is complex, astride 2)
// and off-diagonal beta[1..m-1].  vals receives the nc lowest eigenvalues of T
// then the nh lowest of T-hat; y the eigenvectors of the kept ones (m each);
// work holds 5 m doubles per kept vector.
struct TdProb {
  const double* alpha;
  int astride;
  const double* beta;
  int m;
  int nc, nh, want, filter;  // filter 1: Cullum-Willoughby copy test; 0: the lowest `want`
  double* vals;
  double* y;
  double* work;
};
struct TdOut {
  int na;                 // Ritz values kept (<= want)
  int acc[kMaxEv];        // their indices among the nc eigenvalues of T
  double theta[kMaxEv];   // their values
};
// Device scratch of the selection, grown on demand.
struct TdScratch {
  TdProb* probs = nullptr;
  TdOut* out = nullptr;
  double* vals = nullptr;
  double* work = nullptr;
  size_t probs_b = 0, out_b = 0, vals_b = 0, work_b = 0;
  ~TdScratch();
  cudaError_t reserve(int n_probs, int m_max, int nvals_max, int want_max);
};
// Queue the selection of n_probs problems (device table probs_dev) on st:
// eigenvalues, kept values into out_dev, and their eigenvectors when asked.
cudaError_t td_select_async(const TdProb* probs_dev, int n_probs, int m_max, int nvals_max, TdOut* out_dev,
                            bool vectors, cudaStream_t st);
// ritz_select on the device for one T held in device memory: the kept Ritz
// values in sel, their eigenvectors (want x m) in y_dev.  Waits for the result.
int ritz_select_device(const double* alpha, const double* beta, int m, int want, int n_cand, double* y_dev,
                       cudaStream_t st, TdOut& sel);

// Partial reorthogonalisation (Simon, "The Lanczos algorithm with partial
// reorthogonalization", Math. Comp. 42 (1984) 115): omega_{j,k} estimates
// v_j^H v_k from T alone,
//   beta_{j+1} omega_{j+1,k} = beta_{k+1} omega_{j,k+1} + (alpha_k - alpha_j) omega_{j,k}
//                              + beta_k omega_{j,k-1} - beta_j omega_{j-1,k} + theta_{j,k},
// with omega_{k,k} = 1 and a rounding term theta = eps (|alpha_k| + beta_{k+1}
// + |alpha_j| + beta_{j+1}) taken with the sign that makes |omega| grow; eps
// is the unit roundoff of the FP32 Krylov vectors.  Every step w is
// reorthogonalised locally, against v_{j-1} and v_j, so the estimates
// against those two restart at eps.  When an estimate against an older vector
// passes kProDelta, w is reorthogonalised against all stored vectors at this
// step and the next (the vector before it carries the same loss), and its
// estimates fall back to eps.  (Simon's sqrt(eps) keeps the eigenvalues of T
// accurate, but with FP32 vectors it let 12 of 1,000 serving requests with 4
// levels stop unconverged after 300 steps; eps^(3/4) converged all of them
// at the same speed.)  beta_{j+1} is |w| before the reorthogonalisation
// (w2 = |w|^2).  The estimates live in two rows of omega (ld doubles each) by
// the parity of j.  Called by all threads of one CTA of kProThreads; thread 0
// sets *kf (the first Krylov index this step's Gram-Schmidt runs over: 0 or
// j-1), *force (the next step reorthogonalises fully) and counts full steps
// in *n_full.
constexpr double kProEps = 5.9604644775390625e-08;   // 2^-24
constexpr double kProDelta = 3.814697265625e-06;     // eps^(3/4) = 2^-18
constexpr int kProThreads = 256;
#if defined(__CUDACC__)
__device__ inline void pro_step(const double* alpha, const double* beta, int j, double w2, double* omega, int ld,
                                int* force, int* kf, int* n_full) {
  double* cur = omega + (int64_t)(j & 1) * ld;        // omega_{j, .}
  double* nxt = omega + (int64_t)((j + 1) & 1) * ld;  // omega_{j-1, .} in, omega_{j+1, .} out
  const double bt = fmax(sqrt(w2), 1e-300);
  const double aj = __ldcg(alpha + j), bj = j > 0 ? __ldcg(beta + j) : 0.0;
  __shared__ double smax[kProThreads];
  __shared__ int s_full;
  if (j == 0 && threadIdx.x == 0) cur[0] = 1.0;
  __syncthreads();
  double mx = 0.0;
  for (int k = threadIdx.x; k + 1 < j; k += blockDim.x) {  // k <= j - 2: older than the local pair
    const double bk1 = __ldcg(beta + k + 1), ak = __ldcg(alpha + k);
    double x = bk1 * __ldcg(cur + k + 1) + (ak - aj) * __ldcg(cur + k) - bj * __ldcg(nxt + k);
    if (k > 0) x += __ldcg(beta + k) * __ldcg(cur + k - 1);
    x = (x + copysign(kProEps * (fabs(ak) + bk1 + fabs(aj) + bt), x)) / bt;
    nxt[k] = x;
    mx = fmax(mx, fabs(x));
  }
  smax[threadIdx.x] = mx;
  __syncthreads();
  for (int h = kProThreads / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + h]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const bool cross = smax[0] > kProDelta;
    const bool full = cross || *force;
    *kf = full ? 0 : (j > 0 ? j - 1 : 0);
    *force = cross ? 1 : 0;
    if (full) ++*n_full;
    if (j > 0) nxt[j - 1] = kProEps;  // the local reorthogonalisation
    nxt[j] = kProEps;
    nxt[j + 1] = 1.0;
    s_full = full;
  }
  __syncthreads();
  if (s_full)
    for (int k = threadIdx.x; k + 1 < j; k += blockDim.x) nxt[k] = kProEps;
}
#endif

}  // namespace edg
