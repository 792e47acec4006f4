// Ritz selection shared by the single-sector and batched mixed-precision
// solvers, run on the host: T is at most a few hundred rows, and GB300's FP64
// rate makes a one-CTA bisection slower than one host core.
#pragma once
#include <algorithm>
#include <cmath>
#include <vector>

#include "tridiag.cuh"

namespace edg {

constexpr int kMaxEv = 32;             // Ritz pairs returned
constexpr int kCand = 2 * kMaxEv + 8;  // eigenvalues of T examined when copies are many

struct RitzSel {
  std::vector<double> theta;  // lowest eigenvalues of T, ascending
  std::vector<int> acc;       // indices into theta of the accepted Ritz values
  std::vector<double> y;      // acc.size() x m: their eigenvectors of T
};

// Lowest n_cand eigenvalues of T (diag alpha[0..m-1], off-diagonal
// beta[1..m-1]) and of T-hat (first row and column removed); the first `want`
// that pass the copy test, with their eigenvectors.  Without
// reorthogonalisation FP32 vectors make many copies of each converged level,
// so n_cand must leave room for them (kCand); with full reorthogonalisation
// 2 want + 8 is plenty.
inline void ritz_select(const double* alpha, const double* beta, int m, int want, int n_cand, RitzSel& out) {
  std::vector<double> d(alpha, alpha + m), e(m, 0.0);
  for (int i = 1; i < m; ++i) e[i] = beta[i];
  const int nc = std::min(m, std::max(n_cand, want)), nh = std::min(m - 1, nc + 2);
  out.theta.resize(nc);
  std::vector<double> hat(std::max(nh, 0));
  for (int k = 0; k < nc; ++k) out.theta[k] = tridiag_eigenvalue(d.data(), e.data(), m, k);
  for (int k = 0; k < nh; ++k) hat[k] = tridiag_eigenvalue(d.data() + 1, e.data() + 1, m - 1, k);
  // Cullum-Willoughby: a simple eigenvalue of T that T-hat also has is a copy
  // made by lost orthogonality.  Copies of a converged level built from FP32
  // vectors agree only to about the FP32 backward error, ~1e-7 |T|; T and
  // T-hat share a spurious value to FP64 accuracy.
  double scale = 0;
  for (int i = 0; i < m; ++i) scale = std::max(scale, std::fabs(d[i]) + std::fabs(e[i]) + (i + 1 < m ? std::fabs(e[i + 1]) : 0.0));
  scale = std::max(scale, 1.0);
  const double tol_cluster = 1e-7 * scale, tol_hat = 1e-10 * scale;
  out.acc.clear();
  const std::vector<double>& th = out.theta;
  for (int k = 0; k < nc && (int)out.acc.size() < want; ++k) {
    const bool prev_close = k > 0 && std::fabs(th[k] - th[k - 1]) < tol_cluster;
    const bool next_close = k + 1 < nc && std::fabs(th[k + 1] - th[k]) < tol_cluster;
    bool in_hat = false;
    for (int q = 0; q < nh; ++q)
      if (std::fabs(hat[q] - th[k]) < tol_hat) in_hat = true;
    if (in_hat && !prev_close && !next_close) continue;  // spurious copy
    if (prev_close) continue;                            // keep one per cluster
    out.acc.push_back(k);
  }
  const int na = (int)out.acc.size();
  out.y.assign((size_t)na * m, 0.0);
  std::vector<double> work(5 * (size_t)m);
  for (int q = 0; q < na; ++q)
    tridiag_eigenvector(d.data(), e.data(), m, th[out.acc[q]], out.y.data() + (size_t)q * m, work.data());
}

}  // namespace edg
