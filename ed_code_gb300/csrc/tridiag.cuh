// Real symmetric tridiagonal eigenproblem for the Lanczos T matrix.
//
// The reference rebuilds T (diagonal Re(alpha_j), off-diagonal beta_{j+1})
// and diagonalises it completely with LAPACK zheev at every iteration
// (lanczos.cpp:271-286), but only ever uses the lowest eigenvalue and, at the
// end of a cycle, its eigenvector (lanczos.cpp:286-318).  Here:
//   * eigenvalues: bisection on the Sturm sequence count (Barth, Martin and
//     Wilkinson, Numer. Math. 9 (1967) 386), the k lowest one by one;
//   * eigenvector: inverse iteration with a tridiagonal LU factorisation with
//     partial pivoting (Wilkinson, "The Algebraic Eigenvalue Problem", 1965,
//     ch. 9), two sweeps from a fixed start vector.
// Host and device share the code; everything is FP64.
#pragma once
#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define TD_HD __host__ __device__ inline
#else
#define TD_HD inline
#endif

namespace edg {

// Number of eigenvalues of T strictly below x.  d[0..m-1] diagonal,
// e[1..m-1] off-diagonal (e[0] unused).
TD_HD int sturm_count(const double* d, const double* e, int m, double x, double pivmin) {
  int cnt = 0;
  double q = d[0] - x;
  if (fabs(q) < pivmin) q = -pivmin;
  if (q < 0) ++cnt;
  for (int i = 1; i < m; ++i) {
    q = d[i] - x - e[i] * e[i] / q;
    if (fabs(q) < pivmin) q = -pivmin;
    if (q < 0) ++cnt;
  }
  return cnt;
}

// The k-th smallest eigenvalue (k = 0 is the lowest) by bisection.
TD_HD double tridiag_eigenvalue(const double* d, const double* e, int m, int k) {
  double lo = d[0], hi = d[0], emax = 0.0;
  for (int i = 0; i < m; ++i) {
    const double r = (i > 0 ? fabs(e[i]) : 0.0) + (i + 1 < m ? fabs(e[i + 1]) : 0.0);
    lo = fmin(lo, d[i] - r);
    hi = fmax(hi, d[i] + r);
    if (i > 0) emax = fmax(emax, fabs(e[i]));
  }
  const double scale = fmax(fabs(lo), fabs(hi));
  const double pivmin = fmax(1e-300, 2.2250738585072014e-308 * fmax(1.0, emax * emax));
  lo -= 2.2e-16 * scale + pivmin;
  hi += 2.2e-16 * scale + pivmin;
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    if (mid <= lo || mid >= hi) break;
    if (hi - lo <= 2.0 * 2.2204460492503131e-16 * fmax(fabs(lo), fabs(hi))) break;
    if (sturm_count(d, e, m, mid, pivmin) > k) hi = mid;
    else lo = mid;
  }
  return 0.5 * (lo + hi);
}

#if defined(__CUDACC__)
// Multisection on the same Sturm counts by the 32 lanes of one warp: each
// round evaluates the count at 32 interior points of the bracket and keeps
// the sub-interval where it passes k, 33x narrower.  Same bracket, pivot
// threshold and stopping rule as tridiag_eigenvalue; all lanes return it.
__device__ inline double warp_eigenvalue(const double* d, const double* e, int m, int k) {
  const int lane = threadIdx.x & 31;
  double lo = d[0], hi = d[0], emax = 0.0;
  for (int i = 0; i < m; ++i) {
    const double r = (i > 0 ? fabs(e[i]) : 0.0) + (i + 1 < m ? fabs(e[i + 1]) : 0.0);
    lo = fmin(lo, d[i] - r);
    hi = fmax(hi, d[i] + r);
    if (i > 0) emax = fmax(emax, fabs(e[i]));
  }
  const double scale = fmax(fabs(lo), fabs(hi));
  const double pivmin = fmax(1e-300, 2.2250738585072014e-308 * fmax(1.0, emax * emax));
  lo -= 2.2e-16 * scale + pivmin;
  hi += 2.2e-16 * scale + pivmin;
  for (int round = 0; round < 64; ++round) {
    if (hi - lo <= 2.0 * 2.2204460492503131e-16 * fmax(fabs(lo), fabs(hi))) break;
    const double x = lo + (hi - lo) * ((double)(lane + 1) / 33.0);
    const bool inside = x > lo && x < hi;
    const bool above = inside && sturm_count(d, e, m, x, pivmin) > k;
    const unsigned a = __ballot_sync(0xffffffffu, above);
    const unsigned in = __ballot_sync(0xffffffffu, inside);
    if (in == 0u) break;  // the bracket has no interior point left
    const int first = a ? __ffs(a) - 1 : 32;  // counts are monotone in x
    const double xlo = __shfl_sync(0xffffffffu, x, first > 0 ? first - 1 : 0);
    const double xhi = __shfl_sync(0xffffffffu, x, first < 32 ? first : 31);
    if (first > 0 && ((in >> (first - 1)) & 1u)) lo = xlo;
    if (first < 32) hi = xhi;
  }
  return 0.5 * (lo + hi);
}
#endif

// Eigenvector of eigenvalue lam, normalised, written to x[0..m-1].  Work
// arrays: 5*m doubles in `wk`.  The sign is fixed so that the largest
// component is positive.  For a level of a cluster of (nearly) equal
// eigenvalues, `prev` holds the n_prev unit vectors already computed for the
// cluster (m doubles each, consecutive): each sweep's iterate is
// orthogonalised against them (modified Gram-Schmidt), and `seed` > 0 varies
// the start vector, so the cluster's vectors come out orthonormal (the
// approach of LAPACK's inverse iteration for clustered eigenvalues).
TD_HD void tridiag_eigenvector_ex(const double* d, const double* e, int m, double lam, double* x, double* wk,
                                  const double* prev, int n_prev, int seed);
TD_HD void tridiag_eigenvector(const double* d, const double* e, int m, double lam, double* x, double* wk) {
  tridiag_eigenvector_ex(d, e, m, lam, x, wk, nullptr, 0, 0);
}
TD_HD void tridiag_eigenvector_ex(const double* d, const double* e, int m, double lam, double* x, double* wk,
                                  const double* prev, int n_prev, int seed) {
  double* u0 = wk;          // main diagonal of U
  double* u1 = wk + m;      // first superdiagonal of U
  double* u2 = wk + 2 * m;  // second superdiagonal of U (fill-in from pivoting)
  double* l = wk + 3 * m;   // multipliers
  double* piv = wk + 4 * m; // 1 when rows k, k+1 were swapped
  double scale = 0.0;
  for (int i = 0; i < m; ++i) scale = fmax(scale, fabs(d[i]) + (i > 0 ? fabs(e[i]) : 0.0));
  const double tiny = fmax(scale, 1e-300) * 2.2204460492503131e-16;
  // LU with partial pivoting of (T - lam I)
  for (int i = 0; i < m; ++i) {
    u0[i] = d[i] - lam;
    u1[i] = (i + 1 < m) ? e[i + 1] : 0.0;
    u2[i] = 0.0;
  }
  for (int k = 0; k + 1 < m; ++k) {
    const double sub = e[k + 1];
    if (fabs(u0[k]) >= fabs(sub)) {
      piv[k] = 0.0;
      if (u0[k] == 0.0) u0[k] = tiny;
      l[k] = sub / u0[k];
      u0[k + 1] -= l[k] * u1[k];
      u1[k + 1] -= l[k] * u2[k];
    } else {
      piv[k] = 1.0;
      l[k] = u0[k] / sub;
      // swap row k (u0[k], u1[k], u2[k]) with row k+1 (sub, u0[k+1], u1[k+1])
      const double r0 = sub, r1 = u0[k + 1], r2 = u1[k + 1];
      const double o1 = u1[k], o2 = u2[k];
      u0[k] = r0;
      u1[k] = r1;
      u2[k] = r2;
      u0[k + 1] = o1 - l[k] * r1;
      u1[k + 1] = o2 - l[k] * r2;
    }
  }
  if (u0[m - 1] == 0.0) u0[m - 1] = tiny;
  for (int i = 0; i < m; ++i) x[i] = seed > 0 ? 1.0 + 0.25 * (double)((i * (2 * seed + 1) + seed) % 7) / 7.0 : 1.0;
  for (int sweep = 0; sweep < 3; ++sweep) {
    // forward: apply the row operations to the right-hand side
    for (int k = 0; k + 1 < m; ++k) {
      if (piv[k] != 0.0) {
        const double t = x[k];
        x[k] = x[k + 1];
        x[k + 1] = t;
      }
      x[k + 1] -= l[k] * x[k];
    }
    // back substitution with U
    for (int i = m - 1; i >= 0; --i) {
      double s = x[i];
      if (i + 1 < m) s -= u1[i] * x[i + 1];
      if (i + 2 < m) s -= u2[i] * x[i + 2];
      double p = u0[i];
      if (fabs(p) < tiny) p = p < 0 ? -tiny : tiny;
      x[i] = s / p;
    }
    for (int q = 0; q < n_prev; ++q) {
      const double* pq = prev + (int64_t)q * m;
      double dot = 0.0;
      for (int i = 0; i < m; ++i) dot += pq[i] * x[i];
      for (int i = 0; i < m; ++i) x[i] -= dot * pq[i];
    }
    double nrm = 0.0, big = 0.0;
    int arg = 0;
    for (int i = 0; i < m; ++i) {
      nrm += x[i] * x[i];
      if (fabs(x[i]) > big) { big = fabs(x[i]); arg = i; }
    }
    nrm = sqrt(nrm);
    const double sgn = x[arg] < 0 ? -1.0 : 1.0;
    for (int i = 0; i < m; ++i) x[i] = sgn * x[i] / nrm;
  }
}

}  // namespace edg
