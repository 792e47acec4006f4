// Stored targets: the orbit search of H*v done once per sector.
//
// For every row i and every anti-aligned flip group of its state (in the
// fixed order of the groups), one 32-bit word is kept in HBM:
//     entry = j | cls << jbits      (j: position of the flipped state's
//                                    representative, cls: its phase class)
// or 0xFFFFFFFF when the representative is not an allowed state.  Row i's
// words start at row_ptr[i]; their count is the number of anti-aligned
// groups of reps[i], which the H*v recomputes from the state.
//
// H*v then streams these words (coalesced: one warp per row, lane k handles
// the row's k-th word) and computes everything else on the fly from the state
// bits -- the bond and chirality coefficients (H_v.cpp:219-303), the diagonal
// Ezz, the phase from a per-class table -- exactly as the matrix-free kernel
// does.  The norm ratio norm_i/norm_j is split: u_j = v_j / norm_j is formed
// by a streaming pass before the row loop, norm_i multiplies the row sum.
//
// Memory: 4 bytes per (row, anti-aligned pair), 56 GB for the 36-site Sz=0
// sector, plus 8 bytes per row for row_ptr.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <iterator>
#include <numeric>
#include <string>
#include <vector>

#include "hv_common.cuh"

namespace edg {

namespace {

constexpr int kWarpsPerBlock = 8;
constexpr int kTgtThreads = 32 * kWarpsPerBlock;

// anti-aligned groups of state s, 32 at a time: bit l of word r is group 32r+l
template <typename Real, int NW>
__device__ __forceinline__ void anti_words(uint64_t s, const HvSmem<Real>& H, int ng, uint32_t (&words)[NW],
                                           Real& fac_lane) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int r = 0; r < NW; ++r) {
    const int g = 32 * r + lane;
    bool a = false;
    if (g < ng) {
      a = popc64(s & H.groups[g].mask) == 1;
      if (a) fac_lane += H.groups[g].fac;
    }
    words[r] = __ballot_sync(0xffffffffu, a);
  }
}

// group of the k-th anti-aligned pair
template <int NW>
__device__ __forceinline__ int select_group(const uint32_t (&words)[NW], int k) {
  uint32_t wsel = 0;
  int qsel = 0, before = 0, acc = 0;
#pragma unroll
  for (int q = 0; q < NW; ++q) {
    const int c = __popc(words[q]);
    if (k >= acc && k < acc + c) {
      wsel = words[q];
      qsel = q;
      before = acc;
    }
    acc += c;
  }
  return 32 * qsel + (int)__fns(wsel, 0u, k - before + 1);
}

template <int NW>
__device__ __forceinline__ int total(const uint32_t (&words)[NW]) {
  int n = 0;
#pragma unroll
  for (int q = 0; q < NW; ++q) n += __popc(words[q]);
  return n;
}

// number of anti-aligned groups per row
__global__ void __launch_bounds__(kTgtThreads) k_tgt_count(SectorView V, uint32_t* __restrict__ counts) {
  __shared__ SectorParams P;
  __shared__ uint64_t masks[kMaxGroups];
  for (int i = threadIdx.x; i < (int)(sizeof(SectorParams) / 8); i += blockDim.x)
    reinterpret_cast<uint64_t*>(&P)[i] = reinterpret_cast<const uint64_t*>(V.params)[i];
  __syncthreads();
  for (int g = threadIdx.x; g < P.n_groups; g += blockDim.x) masks[g] = V.groups[g].mask;
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < P.n_p; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t s = V.reps[i];
    uint32_t c = 0;
    for (int g = 0; g < P.n_groups; ++g) c += (popc64(s & masks[g]) == 1);
    counts[i] = c;
  }
}

// 64-bit exclusive scan: chunk sums, one CTA over the chunk sums, apply
constexpr int kScan = 256, kScanPer = 16, kChunk = kScan * kScanPer;

__device__ __forceinline__ unsigned long long block_scan64(unsigned long long x, unsigned long long* tot) {
  __shared__ unsigned long long ws[kScan / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned long long inc = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) ws[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    const unsigned long long v = lane < kScan / 32 ? ws[lane] : 0ull;
    unsigned long long vi = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, vi, o);
      if (lane >= o) vi += y;
    }
    if (lane < kScan / 32) ws[lane] = vi - v;
    if (lane == kScan / 32 - 1) *tot = vi;
  }
  __syncthreads();
  const unsigned long long r = inc - x + ws[wid];
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(kScan) k_scan64_chunks(const uint32_t* __restrict__ in, int64_t n,
                                                          unsigned long long* __restrict__ sums) {
  const int64_t b = (int64_t)blockIdx.x * kChunk + (int64_t)threadIdx.x * kScanPer;
  unsigned long long s = 0;
  for (int k = 0; k < kScanPer; ++k)
    if (b + k < n) s += in[b + k];
  __shared__ unsigned long long tot;
  block_scan64(s, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kScan) k_scan64_sums(unsigned long long* __restrict__ sums, int64_t n,
                                                        unsigned long long* __restrict__ total) {
  __shared__ unsigned long long tot;
  unsigned long long carry = 0;
  for (int64_t b0 = 0; b0 < n; b0 += kScan) {
    const int64_t i = b0 + threadIdx.x;
    const unsigned long long x = i < n ? sums[i] : 0ull;
    const unsigned long long e = block_scan64(x, &tot);
    if (i < n) sums[i] = carry + e;
    __syncthreads();
    carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(kScan) k_scan64_apply(const uint32_t* __restrict__ in, int64_t n,
                                                         const unsigned long long* __restrict__ offs,
                                                         uint64_t* __restrict__ out) {
  const int64_t b = (int64_t)blockIdx.x * kChunk + (int64_t)threadIdx.x * kScanPer;
  unsigned long long s = 0;
  for (int k = 0; k < kScanPer; ++k)
    if (b + k < n) s += in[b + k];
  __shared__ unsigned long long tot;
  unsigned long long run = block_scan64(s, &tot) + offs[blockIdx.x];
  for (int k = 0; k < kScanPer; ++k)
    if (b + k < n) {
      out[b + k] = run;
      run += in[b + k];
    }
}

// one warp per row: search every anti-aligned target once, store its word
template <bool kTorus, int NW>
__global__ void __launch_bounds__(kTgtThreads) k_tgt_fill(SectorView V, const uint64_t* __restrict__ row_ptr,
                                                          uint32_t* __restrict__ tgt) {
  __shared__ SectorParams P;
  extern __shared__ __align__(16) uint8_t sm[];
  for (int i = threadIdx.x; i < (int)(sizeof(SectorParams) / 8); i += blockDim.x)
    reinterpret_cast<uint64_t*>(&P)[i] = reinterpret_cast<const uint64_t*>(V.params)[i];
  __syncthreads();
  const HvSmem<float> H = stage_hv<float, kTorus>(V, P, sm);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = warp; i < P.n_p; i += n_warps) {
    const uint64_t s = V.reps[i];
    uint32_t words[NW];
    float fac = 0.f;
    anti_words<float, NW>(s, H, P.n_groups, words, fac);
    const int nt = total(words);
    const uint64_t base = row_ptr[i];
    for (int k = lane; k < nt; k += 32) {
      const int g = select_group(words, k);
      Orbit o;
      const int64_t j = locate<float, kTorus>(s ^ H.groups[g].mask, V, P, H, o);
      tgt[base + k] = j < 0 ? 0xFFFFFFFFu : (uint32_t)j | ((uint32_t)P.g2cls[o.g] << P.jbits);
    }
  }
}

template <typename Real>
struct CT2;
template <>
struct CT2<float> { using T = float2; };
template <>
struct CT2<double> { using T = double2; };

// u_j = v_j / norm_j
template <typename Real>
__global__ void k_u_scale(const typename CT2<Real>::T* __restrict__ v, const uint8_t* __restrict__ lid,
                          const double* __restrict__ nrm_inv_tab, int64_t n, typename CT2<Real>::T* __restrict__ u) {
  __shared__ Real tab[65];
  for (int k = threadIdx.x; k < 65; k += blockDim.x) tab[k] = (Real)nrm_inv_tab[k];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    typename CT2<Real>::T x = v[i];
    const Real s = tab[lid[i]];
    x.x *= s;
    x.y *= s;
    u[i] = x;
  }
}

// H*v from the stored targets: one warp per row
template <typename Real, int NW>
__global__ void __launch_bounds__(kTgtThreads) k_hv_stored(SectorView V, const uint64_t* __restrict__ row_ptr,
                                                           const uint32_t* __restrict__ tgt,
                                                           const typename CT2<Real>::T* __restrict__ v,
                                                           const typename CT2<Real>::T* __restrict__ u,
                                                           typename CT2<Real>::T* __restrict__ w) {
  using CT = typename CT2<Real>::T;
  __shared__ SectorParams P;
  __shared__ Real cph_re[64], cph_im[64];
  extern __shared__ __align__(16) uint8_t sm[];
  for (int i = threadIdx.x; i < (int)(sizeof(SectorParams) / 8); i += blockDim.x)
    reinterpret_cast<uint64_t*>(&P)[i] = reinterpret_cast<const uint64_t*>(V.params)[i];
  __syncthreads();
  for (int k = threadIdx.x; k < 64; k += blockDim.x) {
    cph_re[k] = (Real)P.cph_re[k];
    cph_im[k] = (Real)P.cph_im[k];
  }
  // only the group and chirality tables are needed here (no search)
  const HvSmem<Real> H = stage_hv<Real, true>(V, P, sm);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const uint32_t jmask = (P.jbits >= 32) ? 0xFFFFFFFFu : ((1u << P.jbits) - 1u);
  const bool use_ch = P.use_ch != 0;
  for (int64_t i = warp; i < P.n_p; i += n_warps) {
    const uint64_t s = __ldg(reinterpret_cast<const unsigned long long*>(V.reps) + i);
    uint32_t words[NW];
    Real anti = 0;
    anti_words<Real, NW>(s, H, P.n_groups, words, anti);
    const int nt = total(words);
    const uint64_t base = __ldg(reinterpret_cast<const unsigned long long*>(row_ptr) + i);
    Real accr = 0, acci = 0;
    for (int k = lane; k < nt; k += 32) {
      const uint32_t e = __ldg(tgt + base + k);
      if (e == 0xFFFFFFFFu) continue;
      const int g = select_group(words, k);
      const SmemGroup<Real>& gr = H.groups[g];
      const int cs = (int)((s >> gr.a) & 1u);
      Real cr = gr.Bre[cs], ci = gr.Bim[cs];
      if (use_ch) {
        for (int m = gr.ch_begin; m < gr.ch_end; ++m) {
          const SmemCh<Real>& c = H.ch[m];
          const Real sg = ((s >> c.z) & 1u) ? Real(1) : Real(-1);
          cr += sg * c.Are[cs];
          ci += sg * c.Aim[cs];
        }
      }
      const uint32_t cls = e >> P.jbits;
      const Real pr = cph_re[cls], pi = cph_im[cls];
      const Real er = cr * pr - ci * pi, ei = cr * pi + ci * pr;
      const CT uj = u[e & jmask];
      accr += er * uj.x - ei * uj.y;
      acci += er * uj.y + ei * uj.x;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      accr += __shfl_down_sync(0xffffffffu, accr, o);
      acci += __shfl_down_sync(0xffffffffu, acci, o);
      anti += __shfl_down_sync(0xffffffffu, anti, o);
    }
    if (lane == 0) {
      const CT vi = v[i];
      const Real ni = H.nrm[__ldg(V.lid + i)];
      const Real ezz = (Real)P.total_fac - Real(2) * anti;
      CT out;
      out.x = accr * ni + ezz * vi.x;
      out.y = acci * ni + ezz * vi.y;
      w[i] = out;
    }
  }
}

int n_words(int n_groups) { return n_groups <= 128 ? 4 : 8; }

template <typename K>
int grid_for(K kernel, size_t smem, int64_t work, int threads) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
  if (per_sm < 1) per_sm = 1;
  const int64_t want = (work + threads - 1) / threads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms * per_sm));
}

template <typename Real, int NW>
cudaError_t launch_stored_t(const Sector& S, const void* v, void* w, cudaStream_t st) {
  using CT = typename CT2<Real>::T;
  const int64_t n = S.P.n_p;
  const size_t smem = hv_smem_bytes<Real>(S.P.n_groups, S.P.n_ch, true, S.V.row_bits, S.V.n_chunks);
  const double* nrm_inv_dev =
      reinterpret_cast<const double*>(reinterpret_cast<const char*>(S.dP) + offsetof(SectorParams, nrm_inv));
  k_u_scale<Real><<<(int)std::min<int64_t>((n + 255) / 256, 152 * 32), 256, 0, st>>>(
      reinterpret_cast<const CT*>(v), S.lid, nrm_inv_dev, n, reinterpret_cast<CT*>(S.ubuf.ptr));
  auto kern = k_hv_stored<Real, NW>;
  const int grid = grid_for(kern, smem, n * 32, kTgtThreads);
  kern<<<grid, kTgtThreads, smem, st>>>(S.V, S.row_ptr, S.tgt, reinterpret_cast<const CT*>(v),
                                        reinterpret_cast<const CT*>(S.ubuf.ptr), reinterpret_cast<CT*>(w));
  return cudaGetLastError();
}

int64_t gcd64(int64_t a, int64_t b) {
  while (b) {
    const int64_t t = a % b;
    a = b;
    b = t;
  }
  return a < 0 ? -a : a;
}

}  // namespace

void free_targets(Sector& S) {
  if (S.tgt) cudaFree(S.tgt);
  if (S.row_ptr) cudaFree(S.row_ptr);
  if (S.ubuf.ptr) cudaFree(S.ubuf.ptr);
  S.tgt = nullptr;
  S.row_ptr = nullptr;
  S.ubuf = DeviceBuffer{};
  S.P.n_targets = 0;
}

// Returns EDG_OK, or a reason (EDG_ERR_NOMEM / EDG_ERR_UNSUPPORTED) with the
// sector left on the matrix-free kernels.
int build_targets(Sector& S, int64_t max_bytes, std::string& err) {
  SectorParams& P = S.P;
  if (S.tgt) return EDG_OK;
  if (P.use_chch) {
    err = "stored targets do not cover ChCh terms";
    return EDG_ERR_UNSUPPORTED;
  }
  if (P.n_groups > 256) {
    err = "stored targets need at most 256 flip groups";
    return EDG_ERR_UNSUPPORTED;
  }
  // phase classes: translation (a, b) has phase index (kx a L2 + ky b L1) mod G
  const int G = P.L1 * P.L2;
  const int64_t d = gcd64(gcd64((int64_t)P.kx * P.L2, (int64_t)P.ky * P.L1), G);
  const int n_cls = (int)(G / (d ? d : G));
  int cbits = 0;
  while ((1 << cbits) < n_cls) ++cbits;
  int jbits = 0;
  while (jbits < 63 && ((int64_t)1 << jbits) <= P.n_p) ++jbits;  // 2^jbits > n_p: room for the sentinel
  if (jbits + cbits > 32) {
    err = "position and phase class do not fit in 32 bits";
    return EDG_ERR_UNSUPPORTED;
  }
  std::fill(std::begin(P.cph_re), std::end(P.cph_re), 0.0);
  std::fill(std::begin(P.cph_im), std::end(P.cph_im), 0.0);
  std::vector<char> seen(64, 0);
  for (int b = 0; b < P.L2; ++b)
    for (int a = 0; a < P.L1; ++a) {
      const int g = a + P.L1 * b;
      const int64_t m = ((int64_t)P.kx * a * P.L2 + (int64_t)P.ky * b * P.L1) % G;
      const int c = (int)(m / (d ? d : G));
      P.g2cls[g] = (uint8_t)c;
      if (!seen[c]) {  // the first translation of a class gives its phase value
        seen[c] = 1;
        P.cph_re[c] = P.ph_re[g];
        P.cph_im[c] = P.ph_im[g];
      }
    }
  P.jbits = jbits;
  P.cbits = cbits;
  cudaStream_t st = S.stream;
  const int64_t n = P.n_p;
  uint32_t* counts = nullptr;
  unsigned long long *sums = nullptr, *tot = nullptr;
  const int64_t n_chunks = (n + kChunk - 1) / kChunk;
  cudaError_t e = cudaMemcpy(S.dP, &P, sizeof(P), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&counts, sizeof(uint32_t) * n);
  if (e == cudaSuccess) e = cudaMalloc(&sums, sizeof(unsigned long long) * n_chunks);
  if (e == cudaSuccess) e = cudaMalloc(&tot, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc(&S.row_ptr, sizeof(uint64_t) * n);
  auto cleanup = [&]() {
    cudaFree(counts);
    cudaFree(sums);
    cudaFree(tot);
  };
  if (e != cudaSuccess) {
    cleanup();
    free_targets(S);
    err = "stored targets: out of device memory for the row offsets";
    return EDG_ERR_NOMEM;
  }
  k_tgt_count<<<grid_for(k_tgt_count, 0, n, kTgtThreads), kTgtThreads, 0, st>>>(S.V, counts);
  k_scan64_chunks<<<(unsigned)n_chunks, kScan, 0, st>>>(counts, n, sums);
  k_scan64_sums<<<1, kScan, 0, st>>>(sums, n_chunks, tot);
  k_scan64_apply<<<(unsigned)n_chunks, kScan, 0, st>>>(counts, n, sums, S.row_ptr);
  unsigned long long n_tgt = 0;
  e = cudaMemcpyAsync(&n_tgt, tot, sizeof(n_tgt), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cleanup();
  const int64_t elem = P.n_p * 16;  // u scratch, sized for FP64
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  const double need = 4.0 * (double)n_tgt + (double)elem;
  if (e != cudaSuccess || need > (double)max_bytes || need > 0.9 * (double)free_b) {
    free_targets(S);
    err = e != cudaSuccess ? std::string("stored targets: ") + cudaGetErrorString(e)
                           : "stored targets do not fit in the allowed device memory";
    return e != cudaSuccess ? EDG_ERR_CUDA : EDG_ERR_NOMEM;
  }
  e = cudaMalloc(&S.tgt, sizeof(uint32_t) * std::max<unsigned long long>(1, n_tgt));
  if (e == cudaSuccess) e = cudaMalloc(&S.ubuf.ptr, (size_t)elem);
  if (e != cudaSuccess) {
    free_targets(S);
    err = "stored targets: out of device memory";
    return EDG_ERR_NOMEM;
  }
  S.ubuf.bytes = (size_t)elem;
  const bool torus = P.torus != 0;
  const size_t smem = hv_smem_bytes<float>(P.n_groups, P.n_ch, torus, S.V.row_bits, S.V.n_chunks);
  const int nw = n_words(P.n_groups);
  auto fill = [&](auto kern) {
    kern<<<grid_for(kern, smem, n * 32, kTgtThreads), kTgtThreads, smem, st>>>(S.V, S.row_ptr, S.tgt);
  };
  if (torus) {
    if (nw == 4) fill(k_tgt_fill<true, 4>);
    else fill(k_tgt_fill<true, 8>);
  } else {
    if (nw == 4) fill(k_tgt_fill<false, 4>);
    else fill(k_tgt_fill<false, 8>);
  }
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    free_targets(S);
    err = std::string("stored targets: ") + cudaGetErrorString(e);
    return EDG_ERR_CUDA;
  }
  P.n_targets = (int64_t)n_tgt;
  S.device_bytes += sizeof(uint32_t) * n_tgt + sizeof(uint64_t) * n + elem;
  e = cudaMemcpy(S.dP, &P, sizeof(P), cudaMemcpyHostToDevice);
  return e == cudaSuccess ? EDG_OK : EDG_ERR_CUDA;
}

cudaError_t launch_hv_stored(const Sector& S, const void* v, void* w, bool fp64, cudaStream_t st) {
  const int nw = n_words(S.P.n_groups);
  if (fp64) return nw == 4 ? launch_stored_t<double, 4>(S, v, w, st) : launch_stored_t<double, 8>(S, v, w, st);
  return nw == 4 ? launch_stored_t<float, 4>(S, v, w, st) : launch_stored_t<float, 8>(S, v, w, st);
}

}  // namespace edg
