// Kernels shared by the single-sector and batched mixed-precision solvers.
#pragma once
#include <cuda_runtime.h>

#include "tridiag.cuh"

namespace edg {

constexpr int kMaxEv = 32;             // Ritz pairs returned
constexpr int kCand = 2 * kMaxEv + 8;  // lowest eigenvalues of T examined for copies

namespace {

// Lowest eigenvalues of T (diag alpha[0..m-1], off-diag beta[1..m-1]) and of
// T-hat (first row and column removed), then the Ritz vectors' coefficients
// for the accepted ones.  One CTA; thread k bisects eigenvalue k.
__global__ void k_tridiag(const double* __restrict__ alpha, const double* __restrict__ beta, int m, int want,
                          double* __restrict__ theta, double* __restrict__ theta_hat, double* __restrict__ y,
                          double* __restrict__ work, int* __restrict__ accepted, int* __restrict__ n_acc) {
  extern __shared__ double sh[];
  double* d = sh;          // m
  double* e = sh + m;      // m (e[0] unused)
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    d[i] = alpha[i];
    e[i] = i > 0 ? beta[i] : 0.0;
  }
  __syncthreads();
  const int nc = min(kCand, m);
  for (int k = threadIdx.x; k < nc; k += blockDim.x) theta[k] = tridiag_eigenvalue(d, e, m, k);
  for (int k = threadIdx.x; k < min(kCand, m - 1); k += blockDim.x)
    theta_hat[k] = tridiag_eigenvalue(d + 1, e + 1, m - 1, k);
  __syncthreads();
  if (threadIdx.x == 0) {
    // Cullum-Willoughby: a simple eigenvalue of T that T-hat also has is a copy.
    double scale = 0;
    for (int i = 0; i < m; ++i) scale = fmax(scale, fabs(d[i]) + fabs(e[i]) + (i + 1 < m ? fabs(e[i + 1]) : 0.0));
    scale = fmax(scale, 1.0);
    // Copies of a converged level built from FP32 vectors agree only to about
    // the FP32 backward error, ~1e-7 |T|; T and T-hat share a spurious value to
    // FP64 accuracy.
    const double tol_cluster = 1e-7 * scale, tol_hat = 1e-10 * scale;
    int na = 0;
    for (int k = 0; k < nc && na < want; ++k) {
      const bool prev_close = k > 0 && fabs(theta[k] - theta[k - 1]) < tol_cluster;
      const bool next_close = k + 1 < nc && fabs(theta[k + 1] - theta[k]) < tol_cluster;
      bool in_hat = false;
      for (int q = 0; q < min(kCand, m - 1); ++q)
        if (fabs(theta_hat[q] - theta[k]) < tol_hat) in_hat = true;
      if (in_hat && !prev_close && !next_close) continue;  // spurious copy
      if (prev_close) continue;                            // keep one per cluster
      accepted[na++] = k;
    }
    *n_acc = na;
  }
  __syncthreads();
  const int na = *n_acc;
  for (int q = threadIdx.x; q < na; q += blockDim.x)
    tridiag_eigenvector(d, e, m, theta[accepted[q]], y + (int64_t)q * m, work + (int64_t)q * 5 * m);
}

}  // namespace

}  // namespace edg
