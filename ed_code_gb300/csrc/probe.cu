// edg_probe_gather: the random-gather rate of this GPU, the ceiling of the
// stored-row H*v's far gathers.
//
// About half of the targets of a 36-site row land far from the row in the
// representative order, so the H*v reads them as independent random 8- or
// 16-byte entries of a vector far larger than L2; each miss moves a whole
// 32-byte sector.  A streaming copy's bandwidth is not the bound for that
// traffic.  This kernel measures it: `count` loads from a vector of n
// entries at splitmix64-hashed positions (no index array is read), eight
// independent loads in flight per thread, on a grid that fills every SM.
// The sum of the loaded values goes to *out only in a case that does not
// occur (a NaN sum), which keeps the loads from being optimised away.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>

#include "../../include/edgpu.h"

namespace edg {
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
}  // namespace edg

namespace {

constexpr int kThreads = 256;
constexpr int kLoads = 8;

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ float2 ld_hint(const float2* a, uint64_t pol) {
  float2 r;
  asm volatile("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(r.x), "=f"(r.y) : "l"(a), "l"(pol));
  return r;
}
__device__ __forceinline__ double2 ld_hint(const double2* a, uint64_t pol) {
  double2 r;
  asm volatile("ld.global.nc.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;" : "=d"(r.x), "=d"(r.y) : "l"(a), "l"(pol));
  return r;
}

// kHint: 0 plain non-coherent loads, 1 with the L2 evict_last policy of the
// H*v's gathers
template <typename T, int kHint>
__global__ void __launch_bounds__(kThreads) k_probe_gather(const T* __restrict__ u, uint64_t n, uint64_t count,
                                                          uint64_t seed, float* out) {
  uint64_t pol = 0;
  if (kHint) asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t nt = (uint64_t)gridDim.x * blockDim.x;
  float acc = 0.f;
  for (uint64_t k0 = tid * kLoads; k0 < count; k0 += nt * kLoads) {
    T x[kLoads];
#pragma unroll
    for (int q = 0; q < kLoads; ++q) {
      const uint64_t j = __umul64hi(mix64(seed + k0 + q), n);  // uniform in [0, n)
      if (k0 + q < count) x[q] = kHint ? ld_hint(u + j, pol) : __ldg(u + j);
    }
#pragma unroll
    for (int q = 0; q < kLoads; ++q)
      if (k0 + q < count) acc += (float)x[q].x;
  }
  if (acc != acc) out[0] = acc;
}

template <typename T, int kHint>
void launch_probe(const void* u, int64_t n, int64_t count, uint64_t seed, float* out, cudaStream_t st) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_probe_gather<T, kHint>, kThreads, 0);
  const int64_t want = std::max<int64_t>(1, (count + (int64_t)kThreads * kLoads - 1) / ((int64_t)kThreads * kLoads));
  const int grid = (int)std::min<int64_t>(want, (int64_t)sms * std::max(per_sm, 1));
  k_probe_gather<T, kHint><<<grid, kThreads, 0, st>>>(static_cast<const T*>(u), (uint64_t)n, (uint64_t)count, seed,
                                                      out);
}

}  // namespace

extern "C" {

int edg_probe_gather(const void* u, int64_t n, int dtype, int hint, int64_t count, uint64_t seed, float* out,
                     void* stream) {
  using namespace edg;
  if (!u || !out || n <= 0 || count < 0) return fail(EDG_ERR_INVALID, "bad argument");
  if (dtype != EDG_C128 && dtype != EDG_C64) return fail(EDG_ERR_INVALID, "dtype must be EDG_C128 or EDG_C64");
  if (hint != 0 && hint != 1) return fail(EDG_ERR_INVALID, "hint must be 0 or 1");
  cudaStream_t st = (cudaStream_t)stream;
  if (dtype == EDG_C64)
    hint ? launch_probe<float2, 1>(u, n, count, seed, out, st) : launch_probe<float2, 0>(u, n, count, seed, out, st);
  else
    hint ? launch_probe<double2, 1>(u, n, count, seed, out, st) : launch_probe<double2, 0>(u, n, count, seed, out, st);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "probe_gather");
  return EDG_OK;
}

}  // extern "C"
