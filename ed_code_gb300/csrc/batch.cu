// Batched mixed-precision Lanczos: many sectors of uneven dimension
// ("segments") advanced together, one captured CUDA graph per Lanczos step for
// all of them.
//
// Every segment is a sector with stored rows (targets.cu) and a request
// (eigenvalues wanted, maximum steps, tolerance, seed).  Per segment the batch
// keeps its FP32 Krylov vectors V_0..V_m, w, u = v/norm, its FP64 alpha/beta
// and its own step counter and status in device memory, so segments join and
// leave independently: a segment added while others are half way starts at
// step 0 with the next graph.  The rows of all live segments are cut into
// tiles of `tile_rows` rows, and each kernel below runs one CTA per tile that
// reads its segment's descriptor.  One step is nine kernels:
//
//   k_b_hv          u_j = V_j / norm was written by the previous step;
//                   w = H V_j (CSR rows, lanes_per_row lanes per row) and the
//                   tile's partial of alpha_j = Re<V_j|w>
//   k_b_step        w -= alpha_j V_j + beta_j V_{j-1} and the tile's |w|^2
//   k_b_cgs_dot     classical Gram-Schmidt: the tile's <V_k|w>, k <= j
//   k_b_cgs_finish  the segment's <V_k|w> summed over its tiles (FP64); on
//                   the first pass also whether a second pass is needed (the
//                   first removed more than 1e-4 of |w|^2)
//   k_b_cgs_sub     w -= sum_k <V_k|w> V_k; the second pass ends with the
//                   tile's |w|^2 for beta_{j+1}
//   (the three Gram-Schmidt kernels run twice; the second pass returns at
//   once for a segment that does not need it)
//   k_b_scale       V_{j+1} = w / beta_{j+1}, u_{j+1}; the segment's last CTA
//                   advances j and, every check_every steps, runs the
//                   convergence test: the wanted Ritz pairs of T_j
//                   (bisection and inverse iteration in FP64); a segment whose
//                   residual bounds beta_j |y_k[j-1]| are all below
//                   tol * max(1, |theta_k|) stops, as does one that reached
//                   its maximum number of steps.
//
// Each reduction over a segment's tiles (alpha, |w|^2, the Gram-Schmidt
// decision, beta, the step counter) is closed by the segment's last CTA to
// finish (a ticket counter, below), so no kernel exists only to reduce and
// no CTA waits for another.

// The vectors are reorthogonalised every step against all stored vectors
// (with FP32 vectors the copies of converged levels otherwise appear within a
// few steps), or, with opts.reorth = 1, against v_{j-1} and v_j every step and
// against all of them only on the steps where Simon's estimates of the lost
// orthogonality call for it (pro_update below).  A stopped segment
// is finished with the single-sector solver's code (MixedFinish): Ritz
// vectors in FP64, one FP64 H*v each for the Rayleigh quotient (the returned
// eigenvalue) and its residual.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/edgpu.h"
#include "blas1.cuh"
#include "csr_row.cuh"
#include "edg_sector.cuh"
#include "ff.cuh"
#include "lanczos_common.cuh"
#include "tridiag.cuh"

struct edg_sector {
  edg::Sector s;
};

namespace edg {

int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

namespace {

constexpr int kThreads = 256;
static_assert(kThreads == kProThreads, "pro_step runs on one CTA of the batch's kernels");
constexpr int kMaxSteps = 511;  // Krylov vectors per segment: kMaxSteps + 1
constexpr int kCgsY = 8;        // CTAs per tile over the Krylov index k
constexpr int kBatchMaxEv = 32;

enum { kRunning = 0, kConverged = 1, kMaxedOut = 2, kCancelled = 3 };

struct SegDev {
  const uint64_t* row_ptr;
  const uint32_t* col;
  const uint16_t* vid;
  const float2* vtab;
  const double* ezz;
  const uint8_t* lid;
  const double* nrm;      // 65-entry tables in the sector's device parameters
  const double* nrm_inv;
  float2* V;              // (m_max + 1) x n
  float2* w;
  float2* u;
  double* alpha;          // m_max + 1
  double* beta;           // m_max + 2
  double* q;              // 2 (m_max + 1): reorthogonalisation coefficients
  double* ywork;          // want x 6 m_max: Ritz coefficients + inverse-iteration work
  double* aux;            // [0]: |w|^2 before reorthogonalisation
  double* omega;          // partial reorthogonalisation: 2 x (m_max + 2) estimates (nullptr: every step)
  int64_t n;
  int m_max, want, check_every;
  int pack_cb;            // column bits of packed entries (vid == nullptr)
  double tol;
};

struct SegState {
  int j;       // steps taken
  int status;  // kRunning, kConverged, kMaxedOut, kCancelled (set on the host)
  int redo;    // this step's second Gram-Schmidt pass is needed
  int kf;      // this step's Gram-Schmidt runs over V_kf..V_j: 0 (full) or j-1 (local)
  int force;   // partial reorthogonalisation: the next step reorthogonalises fully too
  int n_orth;  // steps that reorthogonalised fully
};

struct TileDev {
  int seg;
  int rows;
  int64_t row0;
};

__device__ __forceinline__ void block_sum2(double& a, double& b) {
  __shared__ double sa[kThreads], sb[kThreads];
  sa[threadIdx.x] = a;
  sb[threadIdx.x] = b;
  __syncthreads();
  for (int h = kThreads / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) {
      sa[threadIdx.x] += sa[threadIdx.x + h];
      sb[threadIdx.x] += sb[threadIdx.x + h];
    }
    __syncthreads();
  }
  a = sa[0];
  b = sb[0];
  __syncthreads();
}

// The fused kernels close a segment's reduction in whichever of its CTAs
// finishes last: every CTA writes its partial, then takes a ticket; the CTA
// holding the last ticket sums all the segment's partials in tile order (the
// same order for any timing, so the result is deterministic) and resets the
// counter for the next step.  No CTA waits for another.
__device__ __forceinline__ bool last_cta(int* cnt, int total) {
  __shared__ int is_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const int t = atomicAdd(cnt, 1);
    is_last = t == total - 1;
    if (is_last) *cnt = 0;
  }
  __syncthreads();
  if (is_last) __threadfence();
  return is_last != 0;
}

// sum of the tile partials part[2k], part[2k+1], k in [k0, k1), in order
__device__ __forceinline__ void seg_sum(const double* part, int k0, int k1, double& a, double& b) {
  a = 0;
  b = 0;
  for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
    a += __ldcg(part + 2 * k);
    b += __ldcg(part + 2 * k + 1);
  }
  block_sum2(a, b);
}

// ticket counters of a segment, one per fused reduction
enum { kCntAlpha = 0, kCntNorm = 1, kCntDecide = 2, kCntBeta = 3, kCntAdvance = 4, kCnts = 8 };

// w = H V_j on the tile's rows: 32/LPR rows per warp, LPR lanes per row, each
// row summed by the single-sector kernel's routines (unrolled entry loads,
// streaming hint on the row data, L2 evict_last on u).  Pipelined like the
// single-sector kernel: a warp loads the head entries of its next rows (and
// the offsets of the rows after) before it gathers for the current ones.
//
// Then alpha_j = Re<V_j|w>: the tile's partial (exact products summed in
// float-float per thread, FP64 across the CTA), closed per segment by the
// last CTA.
template <int LPR>
__global__ void __launch_bounds__(kThreads) k_b_hv(const SegDev* __restrict__ segs, const SegState* __restrict__ ss,
                                                   const TileDev* __restrict__ tiles, const int* __restrict__ tb,
                                                   double* __restrict__ part, int* __restrict__ cnt) {
  const TileDev t = tiles[blockIdx.x];
  if (ss[t.seg].status != kRunning) return;
  const SegDev& S = segs[t.seg];
  constexpr int kRowsPerWarp = 32 / LPR;
  constexpr int kU = head_entries<LPR>();
  const int lane = threadIdx.x & 31, sl = lane % LPR, sub = lane / LPR, wid = threadIdx.x >> 5;
  const float2* v = S.V + (int64_t)ss[t.seg].j * S.n;
  const int rows_per_pass = (kThreads / 32) * kRowsPerWarp;
  const uint64_t pl = l2_evict_last();
  auto offsets = [&](int r, uint64_t& b, uint64_t& e) {
    b = e = 0;
    if (r < t.rows) {
      b = S.row_ptr[t.row0 + r];
      e = S.row_ptr[t.row0 + r + 1];
    }
  };
  int r = wid * kRowsPerWarp + sub;
  uint64_t beg, end, beg1, end1;
  offsets(r, beg, end);
  offsets(r + rows_per_pass, beg1, end1);
  uint32_t e[kU];
  uint16_t h[kU];
  csr_head<LPR, kByVid, 1>(beg, end, sl, S.col, S.vid, 0, e, h);
  for (int r0 = 0; r0 < t.rows; r0 += rows_per_pass) {
    uint64_t beg2, end2;
    offsets(r + 2 * rows_per_pass, beg2, end2);
    uint32_t en[kU];
    uint16_t hn[kU];
    csr_head<LPR, kByVid, 1>(beg1, end1, sl, S.col, S.vid, 0, en, hn);
    float ar, ai;
    csr_finish<float, LPR, false, 1, kByVid>(beg, end, sl, S.col, S.vid, S.pack_cb, S.vtab, S.u, 0, pl, e, h, ar,
                                             ai);
    if (r < t.rows && sl == 0) {
      const int64_t i = t.row0 + r;
      const float ni = (float)S.nrm[S.lid[i]];
      const float d = (float)S.ezz[i];
      S.w[i] = row_out(ar, ai, ni, d, v[i]);
    }
    r += rows_per_pass;
    beg = beg1;
    end = end1;
    beg1 = beg2;
    end1 = end2;
#pragma unroll
    for (int q = 0; q < kU; ++q) {
      e[q] = en[q];
      h[q] = hn[q];
    }
  }
  __syncthreads();  // the tile's w rows are written
  FFAcc sr, si;
  for (int rr = threadIdx.x; rr < t.rows; rr += blockDim.x) {
    const int64_t i = t.row0 + rr;
    const float2 y = S.w[i], x = v[i];
    sr.add_prod(x.x, y.x);
    sr.add_prod(x.y, y.y);
    si.add_prod(x.x, y.y);
    si.sub_prod(x.y, y.x);
  }
  double a = sr.value(), b = si.value();
  block_sum2(a, b);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
  }
  const int k0 = tb[t.seg], k1 = tb[t.seg + 1];
  if (last_cta(cnt + kCnts * t.seg + kCntAlpha, k1 - k0)) {
    seg_sum(part, k0, k1, a, b);
    if (threadIdx.x == 0) S.alpha[ss[t.seg].j] = a;
  }
}

// Partial reorthogonalisation: the segment's last CTA of k_b_step updates
// its estimates (pro_step, lanczos_common.cuh) and sets this step's range.
__device__ void pro_update(const SegDev& S, SegState& st, int j, double w2) {
  pro_step(S.alpha, S.beta, j, w2, S.omega, S.m_max + 2, &st.force, &st.kf, &st.n_orth);
}

// w -= alpha_j V_j + beta_j V_{j-1}, and |w|^2 (tile partials of the stored
// values, closed per segment by the last CTA into aux[0]); then whether this
// step reorthogonalises (every step, or by the partial-reorthogonalisation
// estimates)
__global__ void __launch_bounds__(kThreads) k_b_step(const SegDev* __restrict__ segs, SegState* __restrict__ ss,
                                                     const TileDev* __restrict__ tiles, const int* __restrict__ tb,
                                                     double* __restrict__ part, int* __restrict__ cnt) {
  const TileDev t = tiles[blockIdx.x];
  if (ss[t.seg].status != kRunning) return;
  const SegDev& S = segs[t.seg];
  const int j = ss[t.seg].j;
  const FFScalar a(S.alpha[j]), b(j > 0 ? S.beta[j] : 0.0);
  const float2* v = S.V + (int64_t)j * S.n;
  const float2* vp = j > 0 ? v - S.n : nullptr;
  FFAcc sr;
  for (int r = threadIdx.x; r < t.rows; r += blockDim.x) {
    const int64_t i = t.row0 + r;
    const float2 y = S.w[i], x = v[i];
    const float2 p = vp ? vp[i] : make_float2(0.f, 0.f);
    const float2 o = make_float2(ff_axpy2(y.x, a, x.x, b, p.x), ff_axpy2(y.y, a, x.y, b, p.y));
    S.w[i] = o;
    sr.add_prod(o.x, o.x);
    sr.add_prod(o.y, o.y);
  }
  double s2 = sr.value(), z = 0;
  block_sum2(s2, z);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s2;
    part[2 * blockIdx.x + 1] = 0.0;
  }
  const int k0 = tb[t.seg], k1 = tb[t.seg + 1];
  if (last_cta(cnt + kCnts * t.seg + kCntNorm, k1 - k0)) {
    seg_sum(part, k0, k1, s2, z);
    if (threadIdx.x == 0) S.aux[0] = s2;
    if (S.omega) {
      pro_update(S, ss[t.seg], j, s2);
    } else if (threadIdx.x == 0) {
      ss[t.seg].kf = 0;
      ++ss[t.seg].n_orth;
    }
  }
}

// Sum v[0..2*kQ-1] over the CTA; thread 0 returns the sums in v.
template <int kQ>
__device__ __forceinline__ void block_sum_n(double* v) {
  __shared__ double sm[kThreads / 32][2 * kQ];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 2 * kQ; ++q)
    for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_down_sync(0xffffffffu, v[q], o);
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < 2 * kQ; ++q) sm[wid][q] = v[q];
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int q = 0; q < 2 * kQ; ++q) {
      double s = 0;
      for (int w = 0; w < kThreads / 32; ++w) s += sm[w][q];
      v[q] = s;
    }
  __syncthreads();
}

// tile partials of <V_k|w> for k <= j: in CTA (tile, y) warp wid takes
// k = 8*y + wid, 8*(y + kCgsY) + wid, ..., and sums its vector over all the
// tile's rows (lanes over rows, w re-read from L1 by the CTA's warps), so a
// warp shuffle, not a block reduction, closes each partial.  Products are
// summed with Kahan's compensation (ff.cuh): the q_k only correct w's small
// components along the V_k.
__global__ void __launch_bounds__(kThreads) k_b_cgs_dot(const SegDev* __restrict__ segs,
                                                        const SegState* __restrict__ ss,
                                                        const TileDev* __restrict__ tiles, int n_tiles,
                                                        double* __restrict__ part, int pass) {
  constexpr int kWarps = kThreads / 32;
  const TileDev t = tiles[blockIdx.x];
  const SegDev& S = segs[t.seg];
  const bool run = ss[t.seg].status == kRunning && (pass == 0 || ss[t.seg].redo);
  const int K = run ? ss[t.seg].j + 1 : 0, kf = ss[t.seg].kf;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const float2* __restrict__ w = S.w + t.row0;
  for (int k = kf + blockIdx.y * kWarps + wid; k < K; k += kCgsY * kWarps) {
    const float2* __restrict__ x = S.V + (int64_t)k * S.n + t.row0;
    KahanAcc sr, si;
    int r = lane;
    for (; r + 96 < t.rows; r += 128) {
      float2 a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = __ldcs(x + r + 32 * q);
        b[q] = w[r + 32 * q];
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        sr.add_prod(a[q].x, b[q].x);
        sr.add_prod(a[q].y, b[q].y);
        si.add_prod(a[q].x, b[q].y);
        si.sub_prod(a[q].y, b[q].x);
      }
    }
    for (; r < t.rows; r += 32) {
      const float2 a = __ldcs(x + r), b = w[r];
      sr.add_prod(a.x, b.x);
      sr.add_prod(a.y, b.y);
      si.add_prod(a.x, b.y);
      si.sub_prod(a.y, b.x);
    }
    double re = sr.value(), im = si.value();
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      re += __shfl_down_sync(0xffffffffu, re, o);
      im += __shfl_down_sync(0xffffffffu, im, o);
    }
    if (lane == 0) {
      const int64_t o = ((int64_t)k * n_tiles + blockIdx.x) * 2;
      part[o] = re;
      part[o + 1] = im;
    }
  }
}

// CTA (segment, y): q_k = sum of the segment's tile partials, k = y, y + kCgsY, ...
// After the first pass the last of the segment's kCgsY CTAs also decides
// whether the second pass is needed (Daniel, Gragg, Kaufman and Stewart's
// test): the first pass removed sum |q_k|^2 from |w|^2; when that is below
// 1e-4 |w|^2 (the norm changed by less than 0.005%) w is already orthogonal
// to the working precision and the second pass is skipped.
__global__ void __launch_bounds__(kThreads) k_b_cgs_finish(const SegDev* __restrict__ segs,
                                                           SegState* __restrict__ ss,
                                                           const int* __restrict__ tb, int n_tiles,
                                                           const double* __restrict__ part, int pass,
                                                           int* __restrict__ cnt) {
  if (ss[blockIdx.x].status != kRunning || (pass == 1 && !ss[blockIdx.x].redo)) return;
  const SegDev& S = segs[blockIdx.x];
  const int K = ss[blockIdx.x].j + 1, kf = ss[blockIdx.x].kf;
  for (int k = kf + blockIdx.y; k < K; k += kCgsY) {
    double a = 0, b = 0;
    for (int t = tb[blockIdx.x] + threadIdx.x; t < tb[blockIdx.x + 1]; t += blockDim.x) {
      a += part[((int64_t)k * n_tiles + t) * 2];
      b += part[((int64_t)k * n_tiles + t) * 2 + 1];
    }
    block_sum2(a, b);
    if (threadIdx.x == 0) {
      S.q[2 * k] = a;
      S.q[2 * k + 1] = b;
    }
  }
  if (pass == 0 && last_cta(cnt + kCnts * blockIdx.x + kCntDecide, kCgsY)) {
    double a = 0, b = 0;
    for (int k = kf + threadIdx.x; k < K; k += blockDim.x) {
      const double qr = __ldcg(S.q + 2 * k), qi = __ldcg(S.q + 2 * k + 1);
      a += qr * qr + qi * qi;
    }
    block_sum2(a, b);
    if (threadIdx.x == 0) ss[blockIdx.x].redo = a > 1e-4 * S.aux[0] ? 1 : 0;
  }
}

// w -= sum_k q_k V_k (the first pass; the second only when decided), and
// after the second, beta_{j+1} = |w| (tile partials of the stored values,
// closed per segment by the last CTA)
__global__ void __launch_bounds__(kThreads) k_b_cgs_sub(const SegDev* __restrict__ segs,
                                                        const SegState* __restrict__ ss,
                                                        const TileDev* __restrict__ tiles, int pass,
                                                        const int* __restrict__ tb, double* __restrict__ part,
                                                        int* __restrict__ cnt) {
  const TileDev t = tiles[blockIdx.x];
  if (ss[t.seg].status != kRunning) return;
  const bool sub = pass == 0 || ss[t.seg].redo;
  const SegDev& S = segs[t.seg];
  __shared__ float sq[2 * (kMaxSteps + 1)];
  const int K = ss[t.seg].j + 1, kf = ss[t.seg].kf;
  if (sub) {
    for (int k = 2 * kf + threadIdx.x; k < 2 * K; k += blockDim.x) sq[k] = (float)S.q[k];
    __syncthreads();
  }
  // FP32: the q_k are tiny against |w| once the vectors are nearly orthogonal
  FFAcc sr;
  for (int r = threadIdx.x; r < t.rows; r += blockDim.x) {
    const int64_t i = t.row0 + r;
    const float2 y = S.w[i];
    float re = y.x, im = y.y;
    if (sub) {
      for (int k = kf; k < K; ++k) {
        const float2 x = S.V[(int64_t)k * S.n + i];
        re = fmaf(-sq[2 * k], x.x, fmaf(sq[2 * k + 1], x.y, re));
        im = fmaf(-sq[2 * k], x.y, fmaf(-sq[2 * k + 1], x.x, im));
      }
      S.w[i] = make_float2(re, im);
    }
    if (pass == 1) {
      sr.add_prod(re, re);
      sr.add_prod(im, im);
    }
  }
  if (pass == 0) return;
  double s2 = sr.value(), z = 0;
  block_sum2(s2, z);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = s2;
    part[2 * blockIdx.x + 1] = 0.0;
  }
  const int k0 = tb[t.seg], k1 = tb[t.seg + 1];
  if (last_cta(cnt + kCnts * t.seg + kCntBeta, k1 - k0)) {
    seg_sum(part, k0, k1, s2, z);
    if (threadIdx.x == 0) S.beta[ss[t.seg].j + 1] = sqrt(s2);
  }
}

// V_{j+1} = w / beta_{j+1} and u_{j+1} = V_{j+1} / norm for the next H*v;
// then the segment's last CTA advances j and, every check_every steps, tests
// convergence: the wanted lowest Ritz pairs of T_j (multisection by a warp
// each and inverse iteration, FP64) and their residual bounds beta_j |y_k[j-1]|.
__global__ void __launch_bounds__(kThreads) k_b_scale(const SegDev* __restrict__ segs, SegState* __restrict__ ss,
                                                      const TileDev* __restrict__ tiles, const int* __restrict__ tb,
                                                      int* __restrict__ cnt) {
  const TileDev t = tiles[blockIdx.x];
  if (ss[t.seg].status != kRunning) return;
  const SegDev& S = segs[t.seg];
  const int j = ss[t.seg].j;
  const FFScalar s(1.0 / S.beta[j + 1]);
  float2* vn = S.V + (int64_t)(j + 1) * S.n;
  for (int r = threadIdx.x; r < t.rows; r += blockDim.x) {
    const int64_t i = t.row0 + r;
    const float2 y = S.w[i];
    const float2 x = make_float2(fmaf(y.x, s.l, __fmul_rn(y.x, s.h)), fmaf(y.y, s.l, __fmul_rn(y.y, s.h)));
    vn[i] = x;
    const float ni = (float)S.nrm_inv[S.lid[i]];
    S.u[i] = make_float2(x.x * ni, x.y * ni);
  }
  if (!last_cta(cnt + kCnts * t.seg + kCntAdvance, tb[t.seg + 1] - tb[t.seg])) return;
  __shared__ int ok;
  __shared__ double d[kMaxSteps + 1], e[kMaxSteps + 1];
  const int jn = j + 1;
  if (threadIdx.x == 0) {
    ok = 1;
    ss[t.seg].j = jn;
    if (jn >= S.m_max) ss[t.seg].status = kMaxedOut;
  }
  __syncthreads();
  if (jn >= S.m_max || S.tol <= 0 || jn % S.check_every != 0 || jn < 2 * S.want + 2) return;
  for (int i = threadIdx.x; i < jn; i += blockDim.x) {
    d[i] = __ldcg(S.alpha + i);
    e[i] = i > 0 ? __ldcg(S.beta + i) : 0.0;
  }
  __syncthreads();
  // one warp per wanted eigenvalue (multisection), then its lane 0 runs the
  // inverse iteration
  for (int k = threadIdx.x >> 5; k < S.want; k += blockDim.x >> 5) {
    const double th = warp_eigenvalue(d, e, jn, k);
    if ((threadIdx.x & 31) == 0) {
      double* y = S.ywork + (int64_t)k * 6 * S.m_max;
      tridiag_eigenvector(d, e, jn, th, y, y + S.m_max);
      if (__ldcg(S.beta + jn) * fabs(y[jn - 1]) > S.tol * fmax(1.0, fabs(th))) ok = 0;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && ok) ss[t.seg].status = kConverged;
}

// start vector V_0 = x / |x| of one segment, and u_0 = V_0 / norm: the CTAs'
// partials of |x|^2 (exact products in float-float), closed by the last CTA
// in CTA order into *nrm2 (deterministic), then the scaling
constexpr int kStartCtas = 608;
__global__ void __launch_bounds__(kThreads) k_b_start_norm(const float2* __restrict__ x, int64_t n,
                                                           double* __restrict__ part, int* __restrict__ cnt,
                                                           double* __restrict__ nrm2) {
  FFAcc s;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    s.add_prod(x[i].x, x[i].x);
    s.add_prod(x[i].y, x[i].y);
  }
  double a = s.value(), b = 0;
  block_sum2(a, b);
  if (threadIdx.x == 0) part[blockIdx.x] = a;
  if (last_cta(cnt, gridDim.x)) {
    a = 0;
    b = 0;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) a += __ldcg(part + k);
    block_sum2(a, b);
    if (threadIdx.x == 0) *nrm2 = a;
  }
}
__global__ void __launch_bounds__(kThreads) k_b_start(float2* __restrict__ V0, const float2* __restrict__ x,
                                                      int64_t n, const double* __restrict__ nrm_inv,
                                                      const uint8_t* __restrict__ lid, float2* __restrict__ u,
                                                      const double* __restrict__ nrm2) {
  const FFScalar inv(1.0 / sqrt(*nrm2));
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 v = make_float2(fmaf(x[i].x, inv.l, __fmul_rn(x[i].x, inv.h)),
                                 fmaf(x[i].y, inv.l, __fmul_rn(x[i].y, inv.h)));
    V0[i] = v;
    const float ni = (float)nrm_inv[lid[i]];
    u[i] = make_float2(v.x * ni, v.y * ni);
  }
}

// The end of many small segments at once.  Each stopped segment's FP64 Ritz
// vectors need H x, the Rayleigh quotient <x|Hx>/|x|^2 and the residual
// |Hx - theta x| / |x| (MixedFinish::rayleigh_async: six launches a vector).
// Segments of up to kFinMaxN rows are finished together instead: all their
// vectors are cut into tiles of kFinRows rows, and three launches (one CTA
// per tile) cover them all -- u = x / norm; Hx from the stored rows in FP64
// with the partials of |x|^2 and <x|Hx>; the residual's partials.  Each
// vector's partials are summed in tile order by its last CTA (a ticket), so
// the results do not depend on the other vectors.
struct FinVec {
  const uint64_t* row_ptr;
  const uint32_t* col;
  const uint16_t* vid;
  const double2* vtab;  // FP64 value table
  const double* ezz;
  const uint8_t* lid;
  const double* nrm;
  const double* nrm_inv;
  const double2* x;
  double2* u;
  double2* hx;
  double* res;  // |x|^2, <x|Hx>, theta, residual
  int64_t n;
  int pack_cb;
  int t0, t1;  // its tiles
};
struct FinTile {
  int v;
  int rows;
  int64_t row0;
};
// Their Ritz vectors X_q = sum_k y_q[k] V_k, also one launch for all: a CTA
// per tile of a segment, the same per-row arithmetic as k_ritz_vectors (FP32
// vectors, float-float sums, up to 8 vectors per sweep of V).
struct RitzSeg {
  const float2* V;
  const double* y;  // na x m coefficients
  double2* X;       // na x n
  int64_t n;
  int m, na;
};
constexpr int kFinRitzChunk = 8;
constexpr int kFinRows = 1024;
constexpr int64_t kFinMaxN = 1 << 16;

__global__ void __launch_bounds__(kThreads) k_f_ritz(const RitzSeg* __restrict__ rs, const FinTile* __restrict__ ts) {
  extern __shared__ __align__(16) float2 sy2[];  // kFinRitzChunk x m (head, tail)
  const FinTile t = ts[blockIdx.x];
  const RitzSeg& R = rs[t.v];
  for (int q0 = 0; q0 < R.na; q0 += kFinRitzChunk) {
    const int qn = min(kFinRitzChunk, R.na - q0);
    __syncthreads();
    for (int k = threadIdx.x; k < qn * R.m; k += blockDim.x) {
      const FFScalar c(R.y[(int64_t)(q0 + k / R.m) * R.m + k % R.m]);
      sy2[k] = make_float2(c.h, c.l);
    }
    __syncthreads();
    for (int r = threadIdx.x; r < t.rows; r += blockDim.x) {
      const int64_t i = t.row0 + r;
      FFAcc ar[kFinRitzChunk], ai[kFinRitzChunk];
      for (int j = 0; j < R.m; ++j) {
        const float2 v = R.V[(int64_t)j * R.n + i];
#pragma unroll
        for (int q = 0; q < kFinRitzChunk; ++q)
          if (q < qn) {
            const float2 c = sy2[q * R.m + j];
            ar[q].add_prod(c.x, v.x);
            ar[q].lo = fmaf(c.y, v.x, ar[q].lo);
            ai[q].add_prod(c.x, v.y);
            ai[q].lo = fmaf(c.y, v.y, ai[q].lo);
          }
      }
#pragma unroll
      for (int q = 0; q < kFinRitzChunk; ++q)
        if (q < qn) R.X[(int64_t)(q0 + q) * R.n + i] = make_double2(ar[q].value(), ai[q].value());
    }
  }
}
constexpr int64_t kFinCap = 1 << 23;  // vector entries per group of finishing segments

__global__ void __launch_bounds__(kThreads) k_f_u(const FinVec* __restrict__ vs, const FinTile* __restrict__ ts) {
  const FinTile t = ts[blockIdx.x];
  const FinVec& V = vs[t.v];
  for (int r = threadIdx.x; r < t.rows; r += blockDim.x) {
    const int64_t i = t.row0 + r;
    const double s = V.nrm_inv[V.lid[i]];
    const double2 x = V.x[i];
    V.u[i] = make_double2(x.x * s, x.y * s);
  }
}

__global__ void __launch_bounds__(kThreads) k_f_hv(const FinVec* __restrict__ vs, const FinTile* __restrict__ ts,
                                                   double* __restrict__ part, int* __restrict__ cnt) {
  constexpr int LPR = 8, kRows = 32 / LPR, kPass = (kThreads / 32) * kRows;
  const FinTile t = ts[blockIdx.x];
  const FinVec& V = vs[t.v];
  const int lane = threadIdx.x & 31, sl = lane % LPR, sub = lane / LPR, wid = threadIdx.x >> 5;
  Acc s0, s1;
  for (int base = wid * kRows; base < t.rows; base += kPass) {  // uniform within the warp
    const int r = base + sub;
    uint64_t beg = 0, end = 0;
    if (r < t.rows) {
      beg = V.row_ptr[t.row0 + r];
      end = V.row_ptr[t.row0 + r + 1];
    }
    double ar, ai;
    csr_row<double, LPR, false, 1, kByVid>(beg, end, sl, V.col, V.vid, V.pack_cb, V.vtab, V.u, ar, ai);
    if (r < t.rows && sl == 0) {
      const int64_t i = t.row0 + r;
      const double2 xi = V.x[i];
      const double2 h = row_out(ar, ai, V.nrm[V.lid[i]], V.ezz[i], xi);
      V.hx[i] = h;
      s0.add(xi.x * xi.x + xi.y * xi.y);
      s1.add(xi.x * h.x + xi.y * h.y);
    }
  }
  double a = s0.value(), b = s1.value();
  block_sum2(a, b);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = b;
  }
  if (last_cta(cnt + t.v, V.t1 - V.t0)) {
    seg_sum(part, V.t0, V.t1, a, b);
    if (threadIdx.x == 0) {
      V.res[0] = a;
      V.res[1] = b;
      V.res[2] = b / a;
    }
  }
}

__global__ void __launch_bounds__(kThreads) k_f_res(const FinVec* __restrict__ vs, const FinTile* __restrict__ ts,
                                                    double* __restrict__ part, int* __restrict__ cnt) {
  const FinTile t = ts[blockIdx.x];
  const FinVec& V = vs[t.v];
  const double th = __ldcg(V.res + 2);
  Acc r2;
  for (int r = threadIdx.x; r < t.rows; r += blockDim.x) {
    const int64_t i = t.row0 + r;
    const double2 a = V.x[i], h = V.hx[i];
    const double dr = h.x - th * a.x, di = h.y - th * a.y;
    r2.add(dr * dr + di * di);
  }
  double a = r2.value(), b = 0;
  block_sum2(a, b);
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = a;
    part[2 * blockIdx.x + 1] = 0.0;
  }
  if (last_cta(cnt + t.v, V.t1 - V.t0)) {
    seg_sum(part, V.t0, V.t1, a, b);
    if (threadIdx.x == 0) V.res[3] = sqrt(a / __ldcg(V.res));
  }
}

struct Segment {
  edg_sector* sec = nullptr;
  edg_batch_request req{};
  SegDev d{};
  SegState st{};
  int64_t bytes = 0;
  bool cancelled = false;  // edg_batch_cancel: released at the next settle, no result values
};

void release(Segment& g) {
  void* p[] = {g.d.V, g.d.w, g.d.u, g.d.alpha, g.d.beta, g.d.q, g.d.ywork, g.d.aux, g.d.omega};
  for (void* x : p)
    if (x) cudaFree(x);
  g.d = SegDev{};
}

}  // namespace

struct Batch;
static cudaError_t start_vector(Batch& B, const SegDev& d);

struct Batch {
  edg_batch_opts opts{};
  std::vector<Segment> segs;  // the first n_dev are in the device tables, in order
  std::vector<edg_batch_result> done;
  cudaStream_t st = nullptr;
  SegDev* d_segs = nullptr;
  SegState* d_state = nullptr;
  int* d_cnt = nullptr;  // kCnts ticket counters per segment (fused reductions)
  TileDev* d_tiles = nullptr;
  int* d_tb = nullptr;
  double* d_part = nullptr;
  size_t part_cap = 0;
  int n_tiles = 0, n_dev = 0;
  bool dirty = true;
  cudaGraphExec_t graph = nullptr;
  int64_t device_bytes = 0, steps = 0;
  MixedFinish fin;
  TdScratch td;                // device Ritz selection of the stopped segments
  double* ybuf = nullptr;      // their Ritz coefficients
  size_t ybuf_n = 0;
  double* d_start = nullptr;   // start vectors: kStartCtas partials, |x|^2
  int* d_start_cnt = nullptr;  // their ticket counter
  // finishing small segments together (k_f_*): Ritz vectors, u, Hx; tables
  double2 *fx = nullptr, *fu = nullptr, *fhx = nullptr;
  FinVec* d_fv = nullptr;
  FinTile* d_ft = nullptr;
  RitzSeg* d_rs = nullptr;
  FinTile* d_rt = nullptr;
  size_t rs_cap = 0, rt_cap = 0;
  double* d_fpart = nullptr;
  int* d_fcnt = nullptr;
  size_t fv_cap = 0, ft_cap = 0;
  // host seconds: add, step (graph replays and waits), finish (T, Ritz
  // vectors, Rayleigh quotients), release, rebuild (tables and graph capture)
  double timers[5] = {0, 0, 0, 0, 0};

  ~Batch() {
    if (st) cudaStreamSynchronize(st);
    if (graph) cudaGraphExecDestroy(graph);
    for (Segment& g : segs) release(g);
    cudaFree(d_segs);
    cudaFree(d_state);
    cudaFree(d_cnt);
    cudaFree(d_tiles);
    cudaFree(d_tb);
    cudaFree(d_part);
    cudaFree(ybuf);
    cudaFree(d_start);
    cudaFree(d_start_cnt);
    void* f[] = {fx, fu, fhx, d_fv, d_ft, d_fpart, d_fcnt, d_rs, d_rt};
    for (void* q : f) cudaFree(q);
    if (st) cudaStreamDestroy(st);
  }
};

// the queued small-segment vectors: tables up, then the three k_f_* launches
static cudaError_t finish_group(Batch& B, std::vector<RitzSeg>& rs, std::vector<FinTile>& rt,
                                std::vector<FinVec>& fv, std::vector<FinTile>& ft) {
  if (fv.empty()) return cudaSuccess;
  cudaError_t e = cudaSuccess;
  // the Ritz vectors first
  if (rs.size() > B.rs_cap) {
    cudaFree(B.d_rs);
    B.d_rs = nullptr;
    B.rs_cap = 0;
    if ((e = cudaMalloc(&B.d_rs, sizeof(RitzSeg) * rs.size())) != cudaSuccess) return e;
    B.rs_cap = rs.size();
  }
  if (rt.size() > B.rt_cap) {
    cudaFree(B.d_rt);
    B.d_rt = nullptr;
    B.rt_cap = 0;
    if ((e = cudaMalloc(&B.d_rt, sizeof(FinTile) * rt.size())) != cudaSuccess) return e;
    B.rt_cap = rt.size();
  }
  int m_max = 1;
  for (const RitzSeg& r : rs) m_max = std::max(m_max, r.m);
  if ((e = cudaMemcpyAsync(B.d_rs, rs.data(), sizeof(RitzSeg) * rs.size(), cudaMemcpyHostToDevice, B.st)) != cudaSuccess)
    return e;
  if ((e = cudaMemcpyAsync(B.d_rt, rt.data(), sizeof(FinTile) * rt.size(), cudaMemcpyHostToDevice, B.st)) != cudaSuccess)
    return e;
  k_f_ritz<<<(int)rt.size(), kThreads, sizeof(float2) * kFinRitzChunk * m_max, B.st>>>(B.d_rs, B.d_rt);
  if (fv.size() > B.fv_cap) {
    cudaFree(B.d_fv);
    cudaFree(B.d_fcnt);
    B.d_fv = nullptr;
    B.d_fcnt = nullptr;
    B.fv_cap = 0;
    if ((e = cudaMalloc(&B.d_fv, sizeof(FinVec) * fv.size())) != cudaSuccess) return e;
    if ((e = cudaMalloc(&B.d_fcnt, sizeof(int) * fv.size())) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(B.d_fcnt, 0, sizeof(int) * fv.size(), B.st)) != cudaSuccess) return e;
    B.fv_cap = fv.size();
  }
  if (ft.size() > B.ft_cap) {
    cudaFree(B.d_ft);
    cudaFree(B.d_fpart);
    B.d_ft = nullptr;
    B.d_fpart = nullptr;
    B.ft_cap = 0;
    if ((e = cudaMalloc(&B.d_ft, sizeof(FinTile) * ft.size())) != cudaSuccess) return e;
    if ((e = cudaMalloc(&B.d_fpart, sizeof(double) * 2 * ft.size())) != cudaSuccess) return e;
    B.ft_cap = ft.size();
  }
  if ((e = cudaMemcpyAsync(B.d_fv, fv.data(), sizeof(FinVec) * fv.size(), cudaMemcpyHostToDevice, B.st)) != cudaSuccess)
    return e;
  if ((e = cudaMemcpyAsync(B.d_ft, ft.data(), sizeof(FinTile) * ft.size(), cudaMemcpyHostToDevice, B.st)) != cudaSuccess)
    return e;
  const int nt = (int)ft.size();
  k_f_u<<<nt, kThreads, 0, B.st>>>(B.d_fv, B.d_ft);
  k_f_hv<<<nt, kThreads, 0, B.st>>>(B.d_fv, B.d_ft, B.d_fpart, B.d_fcnt);
  k_f_res<<<nt, kThreads, 0, B.st>>>(B.d_fv, B.d_ft, B.d_fpart, B.d_fcnt);
  // the host tables are reused by the next group
  if ((e = cudaStreamSynchronize(B.st)) != cudaSuccess) return e;
  rs.clear();
  rt.clear();
  fv.clear();
  ft.clear();
  return cudaGetLastError();
}

// V_0, u_0 of a segment from the random vector in its w, on the batch's stream
static cudaError_t start_vector(Batch& B, const SegDev& d) {
  cudaError_t e = cudaSuccess;
  if (!B.d_start) {
    if ((e = cudaMalloc(&B.d_start, sizeof(double) * (kStartCtas + 1))) != cudaSuccess) return e;
    if ((e = cudaMalloc(&B.d_start_cnt, sizeof(int))) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(B.d_start_cnt, 0, sizeof(int), B.st)) != cudaSuccess) return e;
  }
  const int grid = (int)std::min<int64_t>(kStartCtas, (d.n + kThreads - 1) / kThreads);
  k_b_start_norm<<<grid, kThreads, 0, B.st>>>(d.w, d.n, B.d_start, B.d_start_cnt, B.d_start + kStartCtas);
  k_b_start<<<grid, kThreads, 0, B.st>>>(d.V, d.w, d.n, d.nrm_inv, d.lid, d.u, B.d_start + kStartCtas);
  return cudaGetLastError();
}

namespace {

// Rows per tile of a segment: the batch's tile_rows, raised for a larger
// segment -- to n/64 rows up to 4096, and beyond that so that no segment has
// more than kMaxSegTiles tiles.  A tuner that chose small tiles on the first
// small sectors must not cut a large one into tens of thousands: the
// Gram-Schmidt dots sum each Krylov vector over a tile with one warp, and on
// 256-row tiles that loop is two iterations long (on a 64-request serving
// stream the dots then took 2.3x the subtraction pass that reads the same
// vectors).  The rule depends on the segment alone, so a segment's arithmetic
// is the same in any mix.
constexpr int64_t kMaxSegTiles = 4096;
int64_t seg_tile_rows(int tile_rows, int64_t n) {
  const int64_t by_size = std::min<int64_t>(4096, (n + 63) / 64);
  const int64_t by_count = (n + kMaxSegTiles - 1) / kMaxSegTiles;
  const int64_t rows = std::max<int64_t>(tile_rows, std::max(by_size, by_count));
  return (rows + 31) / 32 * 32;
}

int64_t segment_bytes(int64_t n, int m, int want) {
  return (int64_t)sizeof(float2) * n * (m + 3) + (int64_t)sizeof(double) * (6 * (m + 2) + 6 * (int64_t)want * m);
}

// copy the device step counters and statuses into the host mirror
cudaError_t pull_state(Batch& B) {
  if (!B.n_dev) return cudaSuccess;
  std::vector<SegState> h(B.n_dev);
  cudaError_t e = cudaMemcpyAsync(h.data(), B.d_state, sizeof(SegState) * B.n_dev, cudaMemcpyDeviceToHost, B.st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(B.st);
  if (e != cudaSuccess) return e;
  for (int k = 0; k < B.n_dev; ++k) {
    B.segs[k].st = h[k];
    if (B.segs[k].cancelled) B.segs[k].st.status = kCancelled;
  }
  return cudaSuccess;
}

using Clock = std::chrono::steady_clock;
double since(Clock::time_point t0) { return std::chrono::duration<double>(Clock::now() - t0).count(); }

// Finish every stopped segment: the Ritz selection of every stopped
// segment's T runs on the device in one batched launch (tridiag_dev.cu) and
// its kept values come back in one wait, then each segment's FP64 Ritz
// vectors and Rayleigh quotients are queued and read back in one more wait.
void finish_stopped(Batch& B) {
  const auto tf = Clock::now();
  std::vector<int> idx;
  for (size_t k = 0; k < B.segs.size(); ++k)
    if (B.segs[k].st.status != kRunning) idx.push_back((int)k);
  if (idx.empty()) return;
  const int ns = (int)idx.size();
  std::vector<int> status(ns, EDG_OK);
  std::vector<TdProb> probs(ns);
  std::vector<size_t> y_at(ns, 0);
  int tm_max = 1, nv_max = 1, want_max = 1;
  size_t y_total = 0;
  for (int i = 0; i < ns; ++i) {
    const Segment& g = B.segs[idx[i]];
    const int m = g.st.j;
    if (g.cancelled) {
      status[i] = EDG_ERR_CANCELLED;
      continue;
    }
    if (m < 1) {
      status[i] = fail(EDG_ERR_INVALID, "batch: a segment stopped before its first step");
      continue;
    }
    // Ritz vectors finished: the wanted levels and two spares (a copy that
    // passes the test on T is dropped by its Rayleigh quotient)
    const int n_try = std::min(kMaxEv, std::min(g.req.n_ev + 2, m));
    // the batch reorthogonalises (every step or partially), so copies of
    // converged levels are rare and n_try + 4 eigenvalues of T (and two more
    // of T-hat for the copy test) suffice
    const int nc = std::min(m, n_try + 4), nh = std::max(0, std::min(m - 1, nc + 2));
    probs[i] = TdProb{g.d.alpha, 1, g.d.beta, m, nc, nh, n_try, 1, nullptr, nullptr, nullptr};
    y_at[i] = y_total;
    y_total += (size_t)n_try * m;
    tm_max = std::max(tm_max, m);
    nv_max = std::max(nv_max, nc + nh);
    want_max = std::max(want_max, n_try);
  }
  std::vector<TdOut> sel(ns);
  cudaError_t e = B.td.reserve(ns, tm_max, nv_max, want_max);
  if (e == cudaSuccess && y_total > B.ybuf_n) {
    cudaFree(B.ybuf);
    B.ybuf = nullptr;
    B.ybuf_n = 0;
    if ((e = cudaMalloc(&B.ybuf, sizeof(double) * y_total)) == cudaSuccess) B.ybuf_n = y_total;
  }
  if (e == cudaSuccess) {
    for (int i = 0; i < ns; ++i) {
      probs[i].vals = B.td.vals + (size_t)i * nv_max;
      probs[i].y = B.ybuf + y_at[i];
      probs[i].work = B.td.work + (size_t)i * 5 * tm_max * want_max;
      if (status[i] != EDG_OK) probs[i].m = 0, probs[i].nc = probs[i].nh = probs[i].want = 0;
    }
    e = cudaMemcpyAsync(B.td.probs, probs.data(), sizeof(TdProb) * ns, cudaMemcpyHostToDevice, B.st);
    if (e == cudaSuccess) e = td_select_async(B.td.probs, ns, tm_max, nv_max, B.td.out, true, B.st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(sel.data(), B.td.out, sizeof(TdOut) * ns, cudaMemcpyDeviceToHost, B.st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(B.st);
  }
  if (e != cudaSuccess) {
    const int rc = cuda_fail(e, "batch: Ritz selection");
    for (int& s : status)
      if (s == EDG_OK) s = rc;
  }
  int64_t n_max = 1, x_max = 1;
  int m_max = 1, total = 0;
  std::vector<int> off(ns, 0);
  for (int i = 0; i < ns; ++i) {
    const Segment& g = B.segs[idx[i]];
    const int na = status[i] == EDG_OK ? sel[i].na : 0;
    if (status[i] == EDG_OK && na == 0)
      status[i] = fail(EDG_ERR_NOT_CONVERGED, "batch: no Ritz value survived the copy test");
    n_max = std::max(n_max, g.d.n);
    x_max = std::max(x_max, g.d.n * na);
    m_max = std::max(m_max, g.st.j);
    off[i] = total;
    total += status[i] == EDG_OK ? na : 0;
  }
  if (B.fin.reserve(n_max, m_max, total) != cudaSuccess || B.fin.reserve_x(x_max, 1) != cudaSuccess) {
    cudaGetLastError();
    for (int& s : status)
      if (s == EDG_OK) s = fail(EDG_ERR_NOMEM, "batch: finishing scratch");
  }
  // small segments together (k_f_*), larger ones a vector at a time
  std::vector<RitzSeg> rs;
  std::vector<FinTile> rt;
  std::vector<FinVec> fv;
  std::vector<FinTile> ft;
  std::vector<int> group;  // the segments (indices into status) in fv
  int64_t fel = 0;
  auto flush = [&]() {
    const cudaError_t fe = finish_group(B, rs, rt, fv, ft);
    if (fe != cudaSuccess)
      for (int k : group)
        if (status[k] == EDG_OK) status[k] = cuda_fail(fe, "batch: FP64 H*v of the small segments");
    group.clear();
    fel = 0;
  };
  for (int i = 0; i < ns; ++i) {
    if (status[i] != EDG_OK) continue;
    Segment& g = B.segs[idx[i]];
    const int m = g.st.j, na = sel[i].na;
    const Sector& S = g.sec->s;
    if (g.d.n <= kFinMaxN && S.vtab64) {
      const int64_t need = g.d.n * na;
      if (fel + need > kFinCap) flush();
      if (!B.fx) {
        double2 *a = nullptr, *b = nullptr, *c = nullptr;
        if (cudaMalloc(&a, sizeof(double2) * kFinCap) != cudaSuccess ||
            cudaMalloc(&b, sizeof(double2) * kFinCap) != cudaSuccess ||
            cudaMalloc(&c, sizeof(double2) * kFinCap) != cudaSuccess) {
          cudaGetLastError();
          cudaFree(a);
          cudaFree(b);
          cudaFree(c);
          status[i] = fail(EDG_ERR_NOMEM, "batch: finishing scratch");
          continue;
        }
        B.fx = a;
        B.fu = b;
        B.fhx = c;
      }
      if (m > kMaxSteps) {
        status[i] = fail(EDG_ERR_INVALID, "batch: more steps than the finish holds");
        continue;
      }
      for (int64_t r0 = 0; r0 < g.d.n; r0 += kFinRows)
        rt.push_back(FinTile{(int)rs.size(), (int)std::min<int64_t>(kFinRows, g.d.n - r0), r0});
      rs.push_back(RitzSeg{g.d.V, B.ybuf + y_at[i], B.fx + fel, g.d.n, m, na});
      group.push_back(i);
      for (int q = 0; q < na; ++q) {
        FinVec v{};
        v.row_ptr = S.row_ptr;
        v.col = S.col;
        v.vid = S.vid;
        v.vtab = reinterpret_cast<const double2*>(S.vtab64);
        v.ezz = S.ezz;
        v.lid = S.lid;
        v.nrm = g.d.nrm;
        v.nrm_inv = g.d.nrm_inv;
        v.x = B.fx + fel + (int64_t)q * g.d.n;
        v.u = B.fu + fel + (int64_t)q * g.d.n;
        v.hx = B.fhx + fel + (int64_t)q * g.d.n;
        v.res = B.fin.res + 4 * (off[i] + q);
        v.n = g.d.n;
        v.pack_cb = S.pack_cb;
        v.t0 = (int)ft.size();
        for (int64_t r0 = 0; r0 < g.d.n; r0 += kFinRows)
          ft.push_back(FinTile{(int)fv.size(), (int)std::min<int64_t>(kFinRows, g.d.n - r0), r0});
        v.t1 = (int)ft.size();
        fv.push_back(v);
      }
      fel += need;
      continue;
    }
    status[i] = B.fin.ritz_stored(B.st, g.d.V, g.d.n, m, na, m, B.ybuf + y_at[i]);
    if (status[i] == EDG_OK && (e = B.fin.rayleigh_async(g.sec->s, B.st, g.d.n, na, B.fin.res + 4 * off[i])) != cudaSuccess)
      status[i] = cuda_fail(e, "batch: FP64 H*v");
  }
  flush();
  std::vector<double> rr(4 * (size_t)std::max(total, 1));
  cudaMemcpyAsync(rr.data(), B.fin.res, sizeof(double) * 4 * total, cudaMemcpyDeviceToHost, B.st);
  if ((e = cudaStreamSynchronize(B.st)) != cudaSuccess) {
    const int rc = cuda_fail(e, "batch: residuals");
    for (int& s : status) s = rc;
  }
  for (int i = 0; i < ns; ++i) {
    Segment& g = B.segs[idx[i]];
    edg_batch_result r{};
    r.tag = g.req.tag;
    r.iterations = g.st.j;
    r.converged = g.st.status == kConverged;
    r.reorth_steps = g.st.n_orth;
    r.status = status[i];
    if (status[i] == EDG_OK) {
      const int na = sel[i].na;
      std::vector<double> ri(rr.begin() + 4 * off[i], rr.begin() + 4 * (off[i] + na));
      std::vector<double> th(sel[i].theta, sel[i].theta + na);
      std::vector<int> acc(na), keep;
      for (int q = 0; q < na; ++q) acc[q] = q;
      pick_levels(ri, th, acc, na, g.req.n_ev, r.eigs, r.ritz, r.residuals, keep);
      r.n_found = (int)keep.size();
    }
    B.done.push_back(r);
  }
  B.timers[2] += since(tf);
  const auto tr = Clock::now();
  std::vector<Segment> keep;
  for (Segment& g : B.segs) {
    if (g.st.status == kRunning) {
      keep.push_back(g);
      continue;
    }
    B.device_bytes -= g.bytes;
    release(g);
  }
  B.segs.swap(keep);
  B.dirty = true;
  B.timers[3] += since(tr);
}

// upload the tables of the current segments and capture one step as a graph
int rebuild(Batch& B) {
  if (B.graph) {
    cudaGraphExecDestroy(B.graph);
    B.graph = nullptr;
  }
  std::vector<SegDev> sd;
  std::vector<SegState> ss;
  std::vector<TileDev> tiles;
  std::vector<int> tb;
  int m_cap = 1;
  for (size_t k = 0; k < B.segs.size(); ++k) {
    sd.push_back(B.segs[k].d);
    ss.push_back(B.segs[k].st);
    m_cap = std::max(m_cap, B.segs[k].d.m_max);
    tb.push_back((int)tiles.size());
    const int64_t rows = seg_tile_rows(B.opts.tile_rows, B.segs[k].d.n);
    for (int64_t r0 = 0; r0 < B.segs[k].d.n; r0 += rows)
      tiles.push_back(TileDev{(int)k, (int)std::min<int64_t>(rows, B.segs[k].d.n - r0), r0});
  }
  tb.push_back((int)tiles.size());
  cudaFree(B.d_segs);
  cudaFree(B.d_state);
  cudaFree(B.d_cnt);
  cudaFree(B.d_tiles);
  cudaFree(B.d_tb);
  B.d_segs = nullptr;
  B.d_state = nullptr;
  B.d_cnt = nullptr;
  B.d_tiles = nullptr;
  B.d_tb = nullptr;
  B.n_tiles = (int)tiles.size();
  B.n_dev = 0;
  B.dirty = false;
  if (sd.empty()) return EDG_OK;
  const size_t need_part = (size_t)2 * B.n_tiles * (m_cap + 1);
  if (need_part > B.part_cap) {
    cudaFree(B.d_part);
    B.d_part = nullptr;
    B.part_cap = 0;
    if (cudaMalloc(&B.d_part, sizeof(double) * need_part) != cudaSuccess) return EDG_ERR_NOMEM;
    B.part_cap = need_part;
  }
  if (cudaMalloc(&B.d_segs, sizeof(SegDev) * sd.size()) != cudaSuccess ||
      cudaMalloc(&B.d_state, sizeof(SegState) * ss.size()) != cudaSuccess ||
      cudaMalloc(&B.d_cnt, sizeof(int) * kCnts * sd.size()) != cudaSuccess ||
      cudaMalloc(&B.d_tiles, sizeof(TileDev) * tiles.size()) != cudaSuccess ||
      cudaMalloc(&B.d_tb, sizeof(int) * tb.size()) != cudaSuccess)
    return EDG_ERR_NOMEM;
  cudaMemcpyAsync(B.d_segs, sd.data(), sizeof(SegDev) * sd.size(), cudaMemcpyHostToDevice, B.st);
  cudaMemcpyAsync(B.d_state, ss.data(), sizeof(SegState) * ss.size(), cudaMemcpyHostToDevice, B.st);
  cudaMemcpyAsync(B.d_tiles, tiles.data(), sizeof(TileDev) * tiles.size(), cudaMemcpyHostToDevice, B.st);
  cudaMemcpyAsync(B.d_tb, tb.data(), sizeof(int) * tb.size(), cudaMemcpyHostToDevice, B.st);
  cudaMemsetAsync(B.d_cnt, 0, sizeof(int) * kCnts * sd.size(), B.st);
  if (cudaStreamSynchronize(B.st) != cudaSuccess) return EDG_ERR_CUDA;  // the host vectors go out of scope
  B.n_dev = (int)sd.size();
  const int nt = B.n_tiles, ns = B.n_dev, lpr = B.opts.lanes_per_row;
  cudaGraph_t g;
  if (cudaStreamBeginCapture(B.st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return EDG_ERR_CUDA;
  // one step, nine kernels: H*v and alpha; the three-term update and |w|^2;
  // two classical Gram-Schmidt passes (tile dots, per-segment sums with the
  // second-pass decision, subtraction; the second pass ends with beta);
  // V_{j+1}, u_{j+1}, the step counter and the convergence test
  int* cnt = B.d_cnt;
  if (lpr == 8) k_b_hv<8><<<nt, kThreads, 0, B.st>>>(B.d_segs, B.d_state, B.d_tiles, B.d_tb, B.d_part, cnt);
  else if (lpr == 32) k_b_hv<32><<<nt, kThreads, 0, B.st>>>(B.d_segs, B.d_state, B.d_tiles, B.d_tb, B.d_part, cnt);
  else k_b_hv<16><<<nt, kThreads, 0, B.st>>>(B.d_segs, B.d_state, B.d_tiles, B.d_tb, B.d_part, cnt);
  k_b_step<<<nt, kThreads, 0, B.st>>>(B.d_segs, B.d_state, B.d_tiles, B.d_tb, B.d_part, cnt);
  for (int pass = 0; pass < 2; ++pass) {
    k_b_cgs_dot<<<dim3(nt, kCgsY), kThreads, 0, B.st>>>(B.d_segs, B.d_state, B.d_tiles, nt, B.d_part, pass);
    k_b_cgs_finish<<<dim3(ns, kCgsY), kThreads, 0, B.st>>>(B.d_segs, B.d_state, B.d_tb, nt, B.d_part, pass, cnt);
    k_b_cgs_sub<<<nt, kThreads, 0, B.st>>>(B.d_segs, B.d_state, B.d_tiles, pass, B.d_tb, B.d_part, cnt);
  }
  k_b_scale<<<nt, kThreads, 0, B.st>>>(B.d_segs, B.d_state, B.d_tiles, B.d_tb, cnt);
  cudaError_t e = cudaStreamEndCapture(B.st, &g);
  if (e != cudaSuccess) return EDG_ERR_CUDA;
  e = cudaGraphInstantiate(&B.graph, g, 0);
  cudaGraphDestroy(g);
  return e == cudaSuccess ? EDG_OK : EDG_ERR_CUDA;
}

// statuses back from the device; stopped segments finished; tables rebuilt
int settle(Batch& B) {
  cudaError_t e = pull_state(B);
  if (e != cudaSuccess) return cuda_fail(e, "batch: step counters");
  for (int k = 0; k < B.n_dev; ++k)
    if (B.segs[k].st.status != kRunning) B.dirty = true;
  if (!B.dirty) return EDG_OK;
  finish_stopped(B);
  const auto t0 = Clock::now();
  const int rc = rebuild(B);
  B.timers[4] += since(t0);
  return rc == EDG_OK ? EDG_OK : fail(rc, "batch: rebuilding the step graph failed");
}

}  // namespace

}  // namespace edg

using namespace edg;

struct edg_batch {
  Batch b;
};

extern "C" {

int edg_batch_create(const edg_batch_opts* opts, edg_batch** out) {
  if (!out) return fail(EDG_ERR_INVALID, "NULL argument");
  edg_batch* h = new edg_batch();
  if (opts) h->b.opts = *opts;
  edg_batch_opts& o = h->b.opts;
  if (o.tile_rows <= 0) o.tile_rows = 1024;
  o.tile_rows = std::max(32, std::min(o.tile_rows, 1 << 20));
  if (o.lanes_per_row != 8 && o.lanes_per_row != 16 && o.lanes_per_row != 32) o.lanes_per_row = 8;
  if (o.check_every <= 0) o.check_every = 10;
  if (o.reorth != 0 && o.reorth != 1) {
    delete h;
    return fail(EDG_ERR_INVALID, "batch: reorth must be 0 (every step) or 1 (partial)");
  }
  if (cudaStreamCreateWithFlags(&h->b.st, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return fail(EDG_ERR_CUDA, "batch stream");
  }
  *out = h;
  return EDG_OK;
}

int edg_batch_destroy(edg_batch* b) {
  delete b;
  return EDG_OK;
}

int edg_batch_footprint(const edg_sector* s, const edg_batch_request* req, int64_t* bytes) {
  if (!s || !req || !bytes) return fail(EDG_ERR_INVALID, "NULL argument");
  const int m = (int)std::min<int64_t>(std::max(2, req->max_iterations), s->s.P.n_p);
  *bytes = segment_bytes(s->s.P.n_p, m, std::min(std::max(1, req->n_ev), m));
  return EDG_OK;
}

int edg_batch_add(edg_batch* bh, edg_sector* sec, const edg_batch_request* req) {
  if (!bh || !sec || !req) return fail(EDG_ERR_INVALID, "NULL argument");
  Batch& B = bh->b;
  const auto t_add = Clock::now();
  Sector& S = sec->s;
  if (!S.col) return fail(EDG_ERR_INVALID, "batch segments need stored rows (edg_sector_build_targets)");
  if (req->n_ev < 1 || req->n_ev > kBatchMaxEv) return fail(EDG_ERR_INVALID, "n_ev must be in [1, 32]");
  if (req->max_iterations < 2 || req->max_iterations > kMaxSteps)
    return fail(EDG_ERR_INVALID, "max_iterations must be in [2, 511]");
  const int64_t n = S.P.n_p;
  Segment g;
  g.sec = sec;
  g.req = *req;
  const int m = (int)std::min<int64_t>(req->max_iterations, n);
  if (m < 2) return fail(EDG_ERR_INVALID, "batch: the sector needs at least 2 states");
  g.req.max_iterations = m;
  SegDev& d = g.d;
  d.row_ptr = S.row_ptr;
  d.col = S.col;
  d.vid = S.vid;
  d.pack_cb = S.pack_cb;
  d.vtab = S.vtab32;
  d.ezz = S.ezz;
  d.lid = S.lid;
  d.nrm = reinterpret_cast<const double*>(reinterpret_cast<const char*>(S.dP) + offsetof(SectorParams, nrm));
  d.nrm_inv = reinterpret_cast<const double*>(reinterpret_cast<const char*>(S.dP) + offsetof(SectorParams, nrm_inv));
  d.n = n;
  d.m_max = m;
  d.want = std::min(req->n_ev, m);
  d.check_every = B.opts.check_every;
  d.tol = req->tol;
  cudaError_t e = cudaMalloc(&d.V, sizeof(float2) * n * (m + 1));
  if (e == cudaSuccess) e = cudaMalloc(&d.w, sizeof(float2) * n);
  if (e == cudaSuccess) e = cudaMalloc(&d.u, sizeof(float2) * n);
  if (e == cudaSuccess) e = cudaMalloc(&d.alpha, sizeof(double) * (m + 1));
  if (e == cudaSuccess) e = cudaMalloc(&d.beta, sizeof(double) * (m + 2));
  if (e == cudaSuccess) e = cudaMalloc(&d.q, sizeof(double) * 2 * (m + 1));
  if (e == cudaSuccess) e = cudaMalloc(&d.ywork, sizeof(double) * 6 * (size_t)d.want * m);
  if (e == cudaSuccess) e = cudaMalloc(&d.aux, sizeof(double) * 2);
  if (e == cudaSuccess && B.opts.reorth == 1) e = cudaMalloc(&d.omega, sizeof(double) * 2 * (m + 2));
  if (e != cudaSuccess) {
    cudaGetLastError();
    release(g);
    return fail(EDG_ERR_NOMEM, "batch: the segment's vectors do not fit");
  }
  g.bytes = segment_bytes(n, m, d.want);
  // start vector: the splitmix64 stream of edg_fill_random with this seed, normalised
  const int rc = edg_fill_random(d.w, n, EDG_C64, req->seed, B.st);
  if (rc != EDG_OK) {
    release(g);
    return rc;
  }
  e = start_vector(B, d);
  if (e == cudaSuccess) e = cudaMemsetAsync(d.beta, 0, sizeof(double) * (m + 2), B.st);
  if (e != cudaSuccess || (e = cudaGetLastError()) != cudaSuccess) {
    release(g);
    return cuda_fail(e, "batch: start vector");
  }
  B.segs.push_back(g);
  B.device_bytes += g.bytes;
  B.dirty = true;
  B.timers[0] += since(t_add);
  return EDG_OK;
}

int edg_batch_step(edg_batch* bh, int n_steps) {
  if (!bh) return fail(EDG_ERR_INVALID, "NULL batch");
  Batch& B = bh->b;
  int rc = EDG_OK;
  for (int s = 0; s < n_steps && rc == EDG_OK; ++s) {
    if (B.dirty && (rc = settle(B)) != EDG_OK) break;
    if (B.n_dev == 0) break;
    const auto t0 = Clock::now();
    const cudaError_t e = cudaGraphLaunch(B.graph, B.st);
    if (e != cudaSuccess) return cuda_fail(e, "batch step");
    ++B.steps;
    if (B.steps % B.opts.check_every == 0) {
      const cudaError_t es = cudaStreamSynchronize(B.st);
      if (es != cudaSuccess) return cuda_fail(es, "batch step");
      B.timers[1] += since(t0);
      rc = settle(B);
    } else {
      B.timers[1] += since(t0);
    }
  }
  if (rc == EDG_OK) rc = settle(B);
  return rc;
}

int edg_batch_tune(edg_batch* bh, int steps, int* tile_rows, int* lanes_per_row, double* ms) {
  if (!bh || steps < 1) return fail(EDG_ERR_INVALID, "edg_batch_tune: NULL batch or steps < 1");
  Batch& B = bh->b;
  if (B.segs.empty()) return fail(EDG_ERR_INVALID, "edg_batch_tune: add the segments first");
  for (const Segment& g : B.segs)
    if (g.st.j != 0 || g.st.status != kRunning || g.cancelled)
      return fail(EDG_ERR_INVALID, "edg_batch_tune: tune before the first step");
  static const int kTiles[4] = {256, 1024, 4096, 16384}, kLanes[2] = {8, 16};
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const edg_batch_opts keep = B.opts;
  float best = 1e30f;
  int bt = keep.tile_rows, bl = keep.lanes_per_row, rc = EDG_OK;
  for (int ti = 0; ti < 4 && rc == EDG_OK; ++ti)
    for (int li = 0; li < 2 && rc == EDG_OK; ++li) {
      B.opts.tile_rows = kTiles[ti];
      B.opts.lanes_per_row = kLanes[li];
      if ((rc = rebuild(B)) != EDG_OK) break;
      cudaGraphLaunch(B.graph, B.st);  // warm-up step
      cudaEventRecord(e0, B.st);
      for (int k = 0; k < steps; ++k) cudaGraphLaunch(B.graph, B.st);
      cudaEventRecord(e1, B.st);
      const cudaError_t ce = cudaEventSynchronize(e1);
      float t = 0;
      cudaEventElapsedTime(&t, e0, e1);
      if (ce != cudaSuccess) rc = cuda_fail(ce, "edg_batch_tune");
      if (ms) ms[ti * 2 + li] = t / steps;
      if (t < best) {
        best = t;
        bt = kTiles[ti];
        bl = kLanes[li];
      }
      // back to the segments' start: seeded start vectors, step 0
      for (Segment& g : B.segs) {
        if (rc == EDG_OK) rc = edg_fill_random(g.d.w, g.d.n, EDG_C64, g.req.seed, B.st);
        if (rc == EDG_OK && start_vector(B, g.d) != cudaSuccess) rc = cuda_fail(cudaGetLastError(), "batch: start vector");
        cudaMemsetAsync(g.d.beta, 0, sizeof(double) * (g.d.m_max + 2), B.st);
        g.st = SegState{};
        g.st.status = kRunning;
      }
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  B.opts = keep;
  if (rc == EDG_OK) {
    B.opts.tile_rows = bt;
    B.opts.lanes_per_row = bl;
  }
  const cudaError_t ce = cudaStreamSynchronize(B.st);
  if (rc == EDG_OK && ce != cudaSuccess) rc = cuda_fail(ce, "edg_batch_tune");
  // the device tables and step counters from the reset host states
  if (rc == EDG_OK && (rc = rebuild(B)) != EDG_OK) rc = fail(rc, "edg_batch_tune: rebuilding the step graph");
  if (rc != EDG_OK) return rc;
  if (tile_rows) *tile_rows = bt;
  if (lanes_per_row) *lanes_per_row = bl;
  return EDG_OK;
}

int edg_batch_cancel(edg_batch* bh, int64_t tag) {
  if (!bh) return fail(EDG_ERR_INVALID, "NULL batch");
  Batch& B = bh->b;
  Segment* g = nullptr;
  for (Segment& x : B.segs)
    if (x.req.tag == tag && !x.cancelled) g = &x;
  if (!g) return fail(EDG_ERR_INVALID, "batch: no live segment with tag " + std::to_string(tag));
  g->cancelled = true;
  g->st.status = kCancelled;
  B.dirty = true;
  return settle(B);
}

int edg_batch_poll(edg_batch* bh, edg_batch_result* out, int cap, int* n_out) {
  if (!bh || !n_out || (cap > 0 && !out)) return fail(EDG_ERR_INVALID, "NULL argument");
  Batch& B = bh->b;
  const int n = std::max(0, std::min<int>(cap, (int)B.done.size()));
  for (int k = 0; k < n; ++k) out[k] = B.done[k];
  B.done.erase(B.done.begin(), B.done.begin() + n);
  *n_out = n;
  return EDG_OK;
}

int edg_batch_timers(const edg_batch* bh, double* seconds) {
  if (!bh || !seconds) return fail(EDG_ERR_INVALID, "NULL argument");
  for (int k = 0; k < 5; ++k) seconds[k] = bh->b.timers[k];
  return EDG_OK;
}

int edg_batch_info(const edg_batch* bh, int* n_active, int64_t* device_bytes, int64_t* steps) {
  if (!bh) return fail(EDG_ERR_INVALID, "NULL batch");
  if (n_active) *n_active = (int)bh->b.segs.size();
  if (device_bytes) *device_bytes = bh->b.device_bytes;
  if (steps) *steps = bh->b.steps;
  return EDG_OK;
}

}  // extern "C"
