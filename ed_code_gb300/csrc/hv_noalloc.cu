// edg_hv_noalloc: the stored-row H*v of targets.cu for callers that must not
// allocate device memory.
//
// The stored-row H*v runs in two kernels: the first writes u = v / norm into a
// scratch vector of n_p entries, the second streams the CSR rows and gathers
// from u.  edg_hv keeps that scratch in a buffer that edg_sector_build_targets
// allocates with cudaMalloc.  Some callers cannot have the library allocate or
// free device memory while they run: applications whose own allocator already
// owns the device's free memory (a framework's caching allocator, an arena
// sized at start-up), so that an extra cudaMalloc fails or fragments it, and
// latency-bound loops, where cudaMalloc/cudaFree would synchronise the device.
// This file gives them a variant whose scratch is a fixed array in the
// library's own device image, so the call itself allocates nothing.
//
// Limits and sharing:
//  * the array holds kScratchBytes = 16 MiB on every GPU that loads this
//    library's device code, until the process exits; hence at most 1,048,576
//    entries for complex128 and 2,097,152 for complex64 -- larger sectors are
//    rejected with EDG_ERR_INVALID;
//  * every call on a device uses the same array.  Nothing in it has to start
//    at zero (the first kernel writes entries 0..n_p-1 before the second one
//    reads them), but calls that overlap on the GPU -- on two streams, from
//    two threads, for two sectors -- overwrite each other's u and race.
//    Order them on one stream or with events.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <mutex>
#include <string>

#include "../../include/edgpu.h"
#include "csr_row.cuh"
#include "edg_sector.cuh"

struct edg_sector {
  edg::Sector s;
};

namespace edg {
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
}  // namespace edg

namespace {

constexpr size_t kScratchBytes = size_t(16) << 20;
constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

}  // namespace

// The scratch vector u.  In host code this name is only a host-side handle:
// kernels are given the device address that cudaGetSymbolAddress returns.
static __device__ __align__(256) double2 g_hv_scratch[kScratchBytes / sizeof(double2)];

namespace {

std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_hv_scratch on `dev`, looked up once per device (with
// that device current) and cached.
cudaError_t scratch_address(int dev, void** out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_hv_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return cudaSuccess;
}

template <typename Real>
struct Cplx;
template <>
struct Cplx<float> { using T = float2; };
template <>
struct Cplx<double> { using T = double2; };

// u_i = v_i / norm_i
template <typename Real>
__global__ void __launch_bounds__(kThreads) k_na_scale(const typename Cplx<Real>::T* __restrict__ v,
                                                       const uint8_t* __restrict__ lid,
                                                       const double* __restrict__ nrm_inv_tab, int64_t n,
                                                       typename Cplx<Real>::T* __restrict__ u) {
  __shared__ Real tab[65];
  for (int k = threadIdx.x; k < 65; k += blockDim.x) tab[k] = (Real)nrm_inv_tab[k];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    typename Cplx<Real>::T x = v[i];
    const Real s = tab[lid[i]];
    x.x *= s;
    x.y *= s;
    u[i] = x;
  }
}

// w_i = norm_i * sum_e vtab[vid_e] * u[col_e] + ezz_i * v_i, LPR lanes per row.
template <typename Real, int LPR>
__global__ void __launch_bounds__(kThreads) k_na_rows(const uint64_t* __restrict__ row_ptr,
                                                      const uint32_t* __restrict__ col,
                                                      const uint16_t* __restrict__ vid, int cb,
                                                      const typename Cplx<Real>::T* __restrict__ vtab,
                                                      const double* __restrict__ ezz, const uint8_t* __restrict__ lid,
                                                      const double* __restrict__ nrm_tab, int64_t n,
                                                      const typename Cplx<Real>::T* __restrict__ v,
                                                      const typename Cplx<Real>::T* __restrict__ u,
                                                      typename Cplx<Real>::T* __restrict__ w) {
  using CT = typename Cplx<Real>::T;
  __shared__ Real nrm[65];
  for (int k = threadIdx.x; k < 65; k += blockDim.x) nrm[k] = (Real)nrm_tab[k];
  __syncthreads();
  constexpr int kRows = 32 / LPR;
  const int lane = threadIdx.x & 31, sl = lane % LPR, sub = lane / LPR;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t n_warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  // every lane of the warp runs the same number of passes (shuffles below)
  for (int64_t base = warp * kRows; base < n; base += n_warps * kRows) {
    const int64_t i = base + sub;
    uint64_t beg = 0, end = 0;
    if (i < n) {
      beg = __ldg(reinterpret_cast<const unsigned long long*>(row_ptr) + i);
      end = __ldg(reinterpret_cast<const unsigned long long*>(row_ptr) + i + 1);
    }
    Real ar = 0, ai = 0;
    for (uint64_t t = beg + sl; t < end; t += LPR) {
      // split entries: column and value id in two arrays; packed: the id
      // above the low cb column bits of one u32
      const uint32_t e = __ldg(col + t);
      const CT c = __ldg(vtab + (vid ? (uint32_t)__ldg(vid + t) : e >> cb));
      const CT x = u[vid ? e : e & ((1u << cb) - 1u)];
      edg::cmac(ar, ai, c, x);
    }
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) {
      ar += __shfl_down_sync(0xffffffffu, ar, o, LPR);
      ai += __shfl_down_sync(0xffffffffu, ai, o, LPR);
    }
    if (sl == 0 && i < n) w[i] = edg::row_out(ar, ai, nrm[lid[i]], (Real)ezz[i], v[i]);
  }
}

template <typename K>
int grid_size(K kernel, int64_t threads_needed, int dev) {
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, 0);
  if (per_sm < 1) per_sm = 1;
  const int64_t want = (threads_needed + kThreads - 1) / kThreads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms * per_sm));
}

template <typename Real, int LPR>
cudaError_t launch_rows(const edg::Sector& S, const void* v, void* w, void* u, int dev, cudaStream_t st) {
  using CT = typename Cplx<Real>::T;
  const int64_t n = S.P.n_p;
  const char* params = reinterpret_cast<const char*>(S.dP);
  const double* nrm_inv = reinterpret_cast<const double*>(params + offsetof(edg::SectorParams, nrm_inv));
  const double* nrm = reinterpret_cast<const double*>(params + offsetof(edg::SectorParams, nrm));
  const CT* tab = reinterpret_cast<const CT*>(sizeof(Real) == 8 ? (const void*)S.vtab64 : (const void*)S.vtab32);
  auto scale = k_na_scale<Real>;
  scale<<<grid_size(scale, n, dev), kThreads, 0, st>>>(reinterpret_cast<const CT*>(v), S.lid, nrm_inv, n,
                                                       reinterpret_cast<CT*>(u));
  auto rows = k_na_rows<Real, LPR>;
  rows<<<grid_size(rows, n * LPR, dev), kThreads, 0, st>>>(S.row_ptr, S.col, S.vid, S.pack_cb, tab, S.ezz, S.lid, nrm, n,
                                                          reinterpret_cast<const CT*>(v),
                                                          reinterpret_cast<const CT*>(u), reinterpret_cast<CT*>(w));
  return cudaGetLastError();
}

template <typename Real>
cudaError_t launch(const edg::Sector& S, const void* v, void* w, void* u, int dev, cudaStream_t st) {
  switch (S.csr_lpr) {
    case 8: return launch_rows<Real, 8>(S, v, w, u, dev, st);
    case 16: return launch_rows<Real, 16>(S, v, w, u, dev, st);
    default: return launch_rows<Real, 32>(S, v, w, u, dev, st);
  }
}

}  // namespace

extern "C" int edg_hv_noalloc(edg_sector* s, const void* v, void* w, int dtype, void* stream) {
  using namespace edg;
  if (!s || !v || !w) return fail(EDG_ERR_INVALID, "NULL argument");
  if (dtype != EDG_C128 && dtype != EDG_C64) return fail(EDG_ERR_INVALID, "dtype must be EDG_C128 or EDG_C64");
  if (v == w) return fail(EDG_ERR_INVALID, "v and w must not alias");
  const Sector& S = s->s;
  const size_t elem = dtype == EDG_C128 ? 16 : 8;
  const int64_t max_n = (int64_t)(kScratchBytes / elem);
  if (S.P.n_p > max_n)
    return fail(EDG_ERR_INVALID, "edg_hv_noalloc: sector has " + std::to_string(S.P.n_p) +
                                     " states; its fixed 16 MiB scratch holds at most " + std::to_string(max_n) +
                                     (dtype == EDG_C128 ? " complex128" : " complex64") + " entries (use edg_hv)");
  if (!S.col) return fail(EDG_ERR_INVALID, "edg_hv_noalloc needs stored rows (edg_sector_build_targets)");
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "edg_hv_noalloc: cudaGetDevice");
  if (dev != S.device) return fail(EDG_ERR_INVALID, "edg_hv_noalloc: make the sector's device current first");
  if (dev < 0 || dev >= kMaxDevices) return fail(EDG_ERR_INVALID, "edg_hv_noalloc: device index out of range");
  void* u = nullptr;
  e = scratch_address(dev, &u);
  if (e != cudaSuccess) return cuda_fail(e, "edg_hv_noalloc: cudaGetSymbolAddress of the scratch array");
  const cudaStream_t st = (cudaStream_t)stream;
  e = dtype == EDG_C128 ? launch<double>(S, v, w, u, dev, st) : launch<float>(S, v, w, u, dev, st);
  if (e != cudaSuccess) return cuda_fail(e, "edg_hv_noalloc launch");
  return EDG_OK;
}
