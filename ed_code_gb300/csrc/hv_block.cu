// H applied to NV vectors at once (NV = 2 or 4) on the stored rows.
//
// The 36-site H*v moves about 1.5x its algorithmic bytes: the targets that a
// flip sends to another orbit member land at random positions of u, and each
// such gather moves a whole line from HBM for one 8-byte entry.  With NV
// vectors interleaved by row (element i of vector q at [i * NV + q]) one
// gather brings the entry of every vector -- 16 bytes (NV = 2) or 32 bytes
// (NV = 4) in FP32, still inside the line the single-vector gather already
// moves -- and the row's entries are read once for all NV vectors.
//
// Same row formula and summation order as the single-vector kernel
// (targets.cu): vector q of the block gets, bit for bit, the sums the
// single-vector kernel gives with the same lanes per row, because each lane
// visits the same entries in the same order and the segmented reduction has
// the same tree.  Consumers: block solvers, and the FP64 Rayleigh quotients of
// several Ritz vectors (one pass instead of one H*v each).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <string>

#include "../../include/edgpu.h"
#include "csr_row.cuh"
#include "hv_common.cuh"

struct edg_sector {
  edg::Sector s;
};

namespace edg {

int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);

namespace {

constexpr int kBlkThreads = 256;

// u[i*NV + q] = v[i*NV + q] / norm_i
template <typename Real, int NV>
__global__ void k_u_scale_blk(const typename CT2<Real>::T* __restrict__ v, const uint8_t* __restrict__ lid,
                              const double* __restrict__ nrm_inv_tab, int64_t n,
                              typename CT2<Real>::T* __restrict__ u) {
  __shared__ Real tab[65];
  for (int k = threadIdx.x; k < 65; k += blockDim.x) tab[k] = (Real)nrm_inv_tab[k];
  __syncthreads();
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * NV; e += (int64_t)gridDim.x * blockDim.x) {
    typename CT2<Real>::T x = v[e];
    const Real s = tab[lid[e / NV]];
    x.x *= s;
    x.y *= s;
    u[e] = x;
  }
}

template <int kFmt>
__device__ __forceinline__ bool is_packed(const uint16_t* vid) {
  return kFmt == kPacked || (kFmt == kByVid && vid == nullptr);
}

// The head of a row (as csr_head) and its gathers for the NV vectors.
template <typename Real, int NV, int LPR, int kFmt, int kPol>
__device__ __forceinline__ void blk_gather(const uint16_t* vid, int cb, const typename CT2<Real>::T* __restrict__ u,
                                           uint64_t pl, const uint32_t (&e)[head_entries<LPR>()],
                                           typename CT2<Real>::T (&x)[head_entries<LPR>()][NV]) {
  constexpr int kU = head_entries<LPR>();
  const uint32_t cmask = is_packed<kFmt>(vid) ? (1u << cb) - 1u : 0xFFFFFFFFu;
#pragma unroll
  for (int q = 0; q < kU; ++q)
    if (e[q] != 0xFFFFFFFFu) {
      const typename CT2<Real>::T* p = u + (int64_t)(e[q] & cmask) * NV;
#pragma unroll
      for (int k = 0; k < NV; ++k) x[q][k] = ld_keep(p + k, pl);
    }
}

template <typename Real, int NV, int LPR, int kPol, int kFmt>
__global__ void __launch_bounds__(kBlkThreads) k_hv_blk(const uint64_t* __restrict__ row_ptr,
                                                        const uint32_t* __restrict__ col,
                                                        const uint16_t* __restrict__ vid, int cb,
                                                        const typename CT2<Real>::T* __restrict__ vtab, int n_vals,
                                                        const double* __restrict__ ezz,
                                                        const uint8_t* __restrict__ lid,
                                                        const double* __restrict__ nrm_tab, int64_t n_p,
                                                        const typename CT2<Real>::T* __restrict__ v,
                                                        const typename CT2<Real>::T* __restrict__ u,
                                                        typename CT2<Real>::T* __restrict__ w) {
  using CT = typename CT2<Real>::T;
  constexpr int kRows = 32 / LPR;
  constexpr int kU = head_entries<LPR>();
  extern __shared__ __align__(16) uint8_t sm[];
  __shared__ Real nrm[65];
  CT* tab = reinterpret_cast<CT*>(sm);
  for (int k = threadIdx.x; k < 65; k += blockDim.x) nrm[k] = (Real)nrm_tab[k];
  for (int k = threadIdx.x; k < n_vals; k += blockDim.x) tab[k] = vtab[k];
  __syncthreads();
  const bool packed = is_packed<kFmt>(vid);
  const int lane = threadIdx.x & 31, sl = lane % LPR, sub = lane / LPR;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t stride = n_warps * kRows;
  const unsigned long long* rp = reinterpret_cast<const unsigned long long*>(row_ptr);
  const uint64_t pf = kPol == 2 ? l2_evict_first() : 0, pl = l2_evict_last();
  auto offsets = [&](int64_t r, uint64_t& b, uint64_t& e) {
    b = e = 0;
    if (r < n_p) {
      b = __ldg(rp + r);
      e = __ldg(rp + r + 1);
    }
  };
  int64_t i = warp * kRows + sub;
  uint64_t beg, end, beg1, end1;
  offsets(i, beg, end);
  offsets(i + stride, beg1, end1);
  uint32_t e[kU];
  uint16_t h[kU];
  csr_head<LPR, kFmt, kPol>(beg, end, sl, col, vid, pf, e, h);
  for (int64_t base = warp * kRows; base < n_p; base += stride) {
    uint64_t beg2, end2;
    offsets(i + 2 * stride, beg2, end2);
    uint32_t en[kU];
    uint16_t hn[kU];
    csr_head<LPR, kFmt, kPol>(beg1, end1, sl, col, vid, pf, en, hn);
    CT x[kU][NV];
    blk_gather<Real, NV, LPR, kFmt, kPol>(vid, cb, u, pl, e, x);
    Real ar[NV], ai[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) ar[k] = ai[k] = 0;
#pragma unroll
    for (int q = 0; q < kU; ++q) {
      if (e[q] == 0xFFFFFFFFu) continue;
      const int id = packed ? (int)(e[q] >> cb) : (int)h[q];
      const CT c = tab[id];
#pragma unroll
      for (int k = 0; k < NV; ++k) cmac(ar[k], ai[k], c, x[q][k]);
    }
    for (uint64_t t = beg + sl + LPR * kU; t < end; t += LPR) {
      uint32_t jt;
      int idt;
      ld_entry<kFmt, kPol>(col, vid, t, cb, pf, jt, idt);
      const CT c = tab[idt];
#pragma unroll
      for (int k = 0; k < NV; ++k) cmac(ar[k], ai[k], c, ld_keep(u + (int64_t)jt * NV + k, pl));
    }
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1)
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        ar[k] += __shfl_down_sync(0xffffffffu, ar[k], o, LPR);
        ai[k] += __shfl_down_sync(0xffffffffu, ai[k], o, LPR);
      }
    if (sl == 0 && i < n_p) {
      const Real ni = nrm[lid[i]];
      const Real d = (Real)ezz[i];
#pragma unroll
      for (int k = 0; k < NV; ++k) w[i * NV + k] = row_out(ar[k], ai[k], ni, d, v[i * NV + k]);
    }
    i += stride;
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
}

template <typename K>
int grid_for_blk(K kernel, size_t smem, int64_t work, int cap) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlkThreads, smem);
  if (cap > 0 && per_sm > cap) per_sm = cap;
  if (per_sm < 1) per_sm = 1;
  const int64_t want = (work + kBlkThreads - 1) / kBlkThreads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms * per_sm));
}

template <typename Real, int NV, int LPR, int kPol, int kFmt>
cudaError_t launch_blk4(const Sector& S, const void* v, void* w, void* u, cudaStream_t st) {
  using CT = typename CT2<Real>::T;
  const int64_t n = S.P.n_p;
  const double* nrm = reinterpret_cast<const double*>(reinterpret_cast<const char*>(S.dP) +
                                                      offsetof(SectorParams, nrm));
  const double* nrm_inv = reinterpret_cast<const double*>(reinterpret_cast<const char*>(S.dP) +
                                                          offsetof(SectorParams, nrm_inv));
  k_u_scale_blk<Real, NV><<<(int)std::min<int64_t>((n * NV + 255) / 256, 152 * 32), 256, 0, st>>>(
      reinterpret_cast<const CT*>(v), S.lid, nrm_inv, n, reinterpret_cast<CT*>(u));
  const CT* tab = reinterpret_cast<const CT*>(sizeof(Real) == 8 ? (const void*)S.vtab64 : (const void*)S.vtab32);
  const size_t tab_bytes = sizeof(CT) * S.n_vals;
  auto kern = k_hv_blk<Real, NV, LPR, kPol, kFmt>;
  const int grid = grid_for_blk(kern, tab_bytes, (n * LPR + 31) / 32 * 32, S.csr_cps);
  kern<<<grid, kBlkThreads, tab_bytes, st>>>(S.row_ptr, S.col, S.vid, S.pack_cb, tab, S.n_vals, S.ezz, S.lid, nrm, n,
                                             reinterpret_cast<const CT*>(v), reinterpret_cast<const CT*>(u),
                                             reinterpret_cast<CT*>(w));
  return cudaGetLastError();
}

template <typename Real, int NV, int LPR>
cudaError_t launch_blk3(const Sector& S, const void* v, void* w, void* u, cudaStream_t st) {
  if (S.pack_cb)
    return S.csr_pol == 2 ? launch_blk4<Real, NV, LPR, 2, kPacked>(S, v, w, u, st)
                          : launch_blk4<Real, NV, LPR, 1, kPacked>(S, v, w, u, st);
  return S.csr_pol == 2 ? launch_blk4<Real, NV, LPR, 2, kSplit>(S, v, w, u, st)
                        : launch_blk4<Real, NV, LPR, 1, kSplit>(S, v, w, u, st);
}

template <typename Real, int NV>
cudaError_t launch_blk2(const Sector& S, const void* v, void* w, void* u, cudaStream_t st) {
  switch (S.csr_lpr) {
    case 8: return launch_blk3<Real, NV, 8>(S, v, w, u, st);
    case 16: return launch_blk3<Real, NV, 16>(S, v, w, u, st);
    default: return launch_blk3<Real, NV, 32>(S, v, w, u, st);
  }
}

}  // namespace

// W = H V for nv = 2 or 4 interleaved vectors on the stored rows; u is the
// caller's n_p * nv scratch.  The value table must fit in shared memory.
cudaError_t launch_hv_block(const Sector& S, const void* v, void* w, int nv, bool fp64, void* u, cudaStream_t st) {
  if (fp64) return nv == 2 ? launch_blk2<double, 2>(S, v, w, u, st) : launch_blk2<double, 4>(S, v, w, u, st);
  return nv == 2 ? launch_blk2<float, 2>(S, v, w, u, st) : launch_blk2<float, 4>(S, v, w, u, st);
}

}  // namespace edg

extern "C" int edg_hv_block(edg_sector* s, const void* v, void* w, int n_vectors, int dtype, void* stream) {
  using namespace edg;
  if (!s || !v || !w) return fail(EDG_ERR_INVALID, "NULL argument");
  if (dtype != EDG_C128 && dtype != EDG_C64) return fail(EDG_ERR_INVALID, "dtype must be EDG_C128 or EDG_C64");
  if (n_vectors != 2 && n_vectors != 4) return fail(EDG_ERR_INVALID, "edg_hv_block: n_vectors must be 2 or 4");
  if (v == w) return fail(EDG_ERR_INVALID, "v and w must not alias");
  Sector& S = s->s;
  if (!S.col) return fail(EDG_ERR_INVALID, "edg_hv_block needs stored rows (edg_sector_build_targets)");
  const bool fp64 = dtype == EDG_C128;
  if ((size_t)S.n_vals * (fp64 ? 16 : 8) > 96 * 1024)
    return fail(EDG_ERR_UNSUPPORTED, "edg_hv_block: value table larger than 96 KB");
  const size_t bytes = (size_t)S.P.n_p * n_vectors * (fp64 ? 16 : 8);
  if (S.ublk.bytes < bytes) {
    if (S.ublk.ptr) cudaFree(S.ublk.ptr);
    S.ublk = DeviceBuffer{};
    if (cudaMalloc(&S.ublk.ptr, bytes) != cudaSuccess) {
      cudaGetLastError();
      return fail(EDG_ERR_NOMEM, "edg_hv_block: scratch of n_p x n_vectors entries");
    }
    S.ublk.bytes = bytes;
    S.device_bytes += bytes;
  }
  const cudaError_t e = launch_hv_block(S, v, w, n_vectors, fp64, S.ublk.ptr, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "edg_hv_block launch");
  return EDG_OK;
}
