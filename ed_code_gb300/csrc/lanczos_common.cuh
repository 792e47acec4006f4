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

}  // namespace edg
