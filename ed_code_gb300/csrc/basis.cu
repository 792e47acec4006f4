// Momentum-basis construction on the GPU: the role of pConstruct_States
// (Momentum_Basis.cpp:645-778) without its per-configuration tables.
//
// The C(N, n_up) configurations are split into records of 96 consecutive Lin
// indices (increasing-integer order, which is the reference's enumeration
// order).  Pass 1 (one thread per record) unranks the record's first
// configuration, steps through the rest with the same-popcount successor, and
// marks the allowed representatives (orbit minimum with p_id, Momentum_Basis.cpp
// :756-770).  A scan turns the per-record counts into positions, and pass 2
// writes the representatives, which come out already sorted ascending like the
// reference's pblock_states, with their stabiliser counts.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>

#include "edg_sector.cuh"

namespace edg {

namespace {

constexpr int kBuildThreads = 256;

// Stage the search tables into shared memory; returns pointers into `sm`.
struct BuildTables {
  const uint8_t* nk;
  const uint16_t* rots;
  const uint64_t* p1;
  const uint64_t* p2;
  const uint64_t* p3;  // T3 (3-D tori only)
};

template <bool kTorus>
__device__ BuildTables stage_build_tables(const SectorView& V, uint8_t* sm) {
  BuildTables T{};
  if (kTorus) {
    const int n = 1 << V.row_bits;
    uint16_t* rots = reinterpret_cast<uint16_t*>(sm);
    uint8_t* nk = sm + 2 * n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      rots[i] = V.rots[i];
      nk[i] = V.nk[i];
    }
    T.nk = nk;
    T.rots = rots;
  } else {
    const int n = V.n_perm * V.n_chunks * 256;
    uint64_t* p = reinterpret_cast<uint64_t*>(sm);
    for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = V.perms[i];
    T.p1 = p;
    T.p2 = p + V.n_chunks * 256;
    T.p3 = p + 2 * V.n_chunks * 256;
  }
  return T;
}

template <bool kTorus>
__device__ __forceinline__ int allowed(uint64_t t, const SectorParams& P, const BuildTables& T, int n_chunks) {
  if (kTorus) return torus_allowed(t, P, T.nk, T.rots);
  return walk_allowed(t, P, T.p1, T.p2, T.p3, n_chunks);
}

template <bool kTorus>
__global__ void __launch_bounds__(kBuildThreads) k_basis_count(SectorView V, uint32_t* __restrict__ counts) {
  __shared__ SectorParams P;
  extern __shared__ __align__(16) uint8_t sm[];
  for (int i = threadIdx.x; i < (int)(sizeof(SectorParams) / 8); i += blockDim.x)
    reinterpret_cast<uint64_t*>(&P)[i] = reinterpret_cast<const uint64_t*>(V.params)[i];
  BuildTables T = stage_build_tables<kTorus>(V, sm);
  __syncthreads();
  const int64_t n_recs = P.n_recs;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n_recs; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t lin0 = r * kRecBits;
    const int64_t rem = P.n_configs - lin0;
    const int n = rem < kRecBits ? (int)rem : kRecBits;
    uint64_t t = unrank_config((uint64_t)lin0, P.n_sites, P.n_ones, V.binom);
    uint32_t b[3] = {0u, 0u, 0u};
    uint32_t cnt = 0;
#pragma unroll
    for (int w = 0; w < 3; ++w) {
      for (int k = 0; k < 32; ++k) {
        const int idx = w * 32 + k;
        if (idx >= n) break;
        if (allowed<kTorus>(t, P, T, V.n_chunks)) {
          b[w] |= 1u << k;
          ++cnt;
        }
        if (idx + 1 < n) t = next_same_popcount(t);
      }
    }
    RankRec rec;
    rec.base = 0;
    rec.bits[0] = b[0];
    rec.bits[1] = b[1];
    rec.bits[2] = b[2];
    V.recs[r] = rec;
    counts[r] = cnt;
  }
}

template <bool kTorus>
__global__ void __launch_bounds__(kBuildThreads) k_basis_emit(SectorView V, const uint32_t* __restrict__ counts,
                                                              uint64_t* __restrict__ reps, uint8_t* __restrict__ lid) {
  __shared__ SectorParams P;
  extern __shared__ __align__(16) uint8_t sm[];
  for (int i = threadIdx.x; i < (int)(sizeof(SectorParams) / 8); i += blockDim.x)
    reinterpret_cast<uint64_t*>(&P)[i] = reinterpret_cast<const uint64_t*>(V.params)[i];
  BuildTables T = stage_build_tables<kTorus>(V, sm);
  __syncthreads();
  const int64_t n_recs = P.n_recs;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n_recs; r += (int64_t)gridDim.x * blockDim.x) {
    if (counts[r] == 0) continue;
    const RankRec rec = V.recs[r];
    const int64_t lin0 = r * kRecBits;
    const int64_t rem = P.n_configs - lin0;
    const int n = rem < kRecBits ? (int)rem : kRecBits;
    uint64_t t = unrank_config((uint64_t)lin0, P.n_sites, P.n_ones, V.binom);
    uint32_t q = rec.base;
    for (int idx = 0; idx < n; ++idx) {
      if ((rec.bits[idx >> 5] >> (idx & 31)) & 1u) {
        reps[q] = t;
        lid[q] = (uint8_t)allowed<kTorus>(t, P, T, V.n_chunks);
        ++q;
      }
      if (idx + 1 < n) t = next_same_popcount(t);
    }
  }
}

// ---- exclusive scan of the per-record counts into RankRec::base -----------
constexpr int kScanThreads = 256;
constexpr int kScanPerThread = 16;
constexpr int kScanChunk = kScanThreads * kScanPerThread;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t x, uint32_t* total) {
  __shared__ uint32_t warp_sums[kScanThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t incl = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_sums[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    uint32_t s = lane < kScanThreads / 32 ? warp_sums[lane] : 0u;
    uint32_t si = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, si, o);
      if (lane >= o) si += y;
    }
    if (lane < kScanThreads / 32) warp_sums[lane] = si - s;
    if (lane == kScanThreads / 32 - 1) *total = si;
  }
  __syncthreads();
  uint32_t r = incl - x + warp_sums[wid];
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_chunks(const uint32_t* __restrict__ in, int64_t n,
                                                               uint32_t* __restrict__ chunk_sums) {
  const int64_t base = (int64_t)blockIdx.x * kScanChunk + (int64_t)threadIdx.x * kScanPerThread;
  uint32_t s = 0;
  for (int k = 0; k < kScanPerThread; ++k)
    if (base + k < n) s += in[base + k];
  __shared__ uint32_t tot;
  block_exclusive_scan(s, &tot);
  if (threadIdx.x == 0) chunk_sums[blockIdx.x] = tot;
}

// One CTA scans the chunk sums in place (exclusive) and writes the total.
__global__ void __launch_bounds__(kScanThreads) k_scan_sums(uint32_t* __restrict__ sums, int64_t n,
                                                             unsigned long long* __restrict__ total_out) {
  __shared__ uint32_t tot;
  unsigned long long carry = 0;
  for (int64_t b0 = 0; b0 < n; b0 += kScanThreads) {
    int64_t i = b0 + threadIdx.x;
    uint32_t x = i < n ? sums[i] : 0u;
    uint32_t e = block_exclusive_scan(x, &tot);
    if (i < n) sums[i] = (uint32_t)(carry + e);
    __syncthreads();
    carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total_out = carry;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const uint32_t* __restrict__ in, int64_t n,
                                                              const uint32_t* __restrict__ chunk_offsets,
                                                              RankRec* __restrict__ recs) {
  const int64_t base = (int64_t)blockIdx.x * kScanChunk + (int64_t)threadIdx.x * kScanPerThread;
  uint32_t s = 0;
  for (int k = 0; k < kScanPerThread; ++k)
    if (base + k < n) s += in[base + k];
  __shared__ uint32_t tot;
  uint32_t run = block_exclusive_scan(s, &tot) + chunk_offsets[blockIdx.x];
  for (int k = 0; k < kScanPerThread; ++k) {
    if (base + k < n) {
      recs[base + k].base = run;
      run += in[base + k];
    }
  }
}

// Reference-order walk over every configuration: representative position and
// translation index for the parity export (rep_loc / state_ph).
__global__ void __launch_bounds__(kBuildThreads) k_walk_tables(SectorView V, int64_t* __restrict__ rep_loc,
                                                               int32_t* __restrict__ gidx) {
  __shared__ SectorParams P;
  extern __shared__ __align__(16) uint8_t sm[];
  for (int i = threadIdx.x; i < (int)(sizeof(SectorParams) / 8); i += blockDim.x)
    reinterpret_cast<uint64_t*>(&P)[i] = reinterpret_cast<const uint64_t*>(V.params)[i];
  BuildTables T = stage_build_tables<false>(V, sm);
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < P.n_configs;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t t = unrank_config((uint64_t)i, P.n_sites, P.n_ones, V.binom);
    Orbit o = orbit_walk(t, P, T.p1, T.p2, T.p3, V.n_chunks);
    int bit;
    const uint32_t q = vrec_of(o.rep, &bit);
    rep_loc[i] = (int64_t)q < P.n_vrecs ? rank_lookup_bit(bit, V.vrecs[q]) : -1;
    gidx[i] = o.g;
  }
}

// Value-indexed rank records: set the bit of every representative, then
// count per record (the scan kernels turn counts into bases).
__global__ void k_vrank_mark(const uint64_t* __restrict__ reps, int64_t n_p, RankRec* __restrict__ vrecs) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_p; i += (int64_t)gridDim.x * blockDim.x) {
    int bit;
    const uint32_t q = vrec_of(reps[i], &bit);
    atomicOr(&vrecs[q].bits[bit >> 5], 1u << (bit & 31));
  }
}
__global__ void k_vrank_count(const RankRec* __restrict__ vrecs, int64_t n, uint32_t* __restrict__ counts) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const RankRec r = vrecs[i];
    counts[i] = (uint32_t)(__popc(r.bits[0]) + __popc(r.bits[1]) + __popc(r.bits[2]));
  }
}

size_t build_smem_bytes(const SectorView& V, bool torus) {
  if (torus) return (size_t)3 << V.row_bits;
  return (size_t)V.n_perm * V.n_chunks * 256 * sizeof(uint64_t);
}

int grid_for(const void* kernel, size_t smem, int64_t work_items) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBuildThreads, smem);
  if (per_sm < 1) per_sm = 1;
  int64_t want = (work_items + kBuildThreads - 1) / kBuildThreads;
  int64_t cap = (int64_t)sms * per_sm * 8;
  return (int)std::max<int64_t>(1, std::min(want, cap));
}

}  // namespace

cudaError_t build_basis(Sector& S, std::string& err) {
  cudaStream_t st = S.stream;
  const bool torus = S.P.torus != 0;
  const int64_t n_recs = S.P.n_recs;
  uint32_t* counts = nullptr;
  uint32_t* chunk = nullptr;
  unsigned long long* total = nullptr;
  const int64_t n_chunks = (n_recs + kScanChunk - 1) / kScanChunk;
  cudaError_t e = cudaMalloc(&counts, sizeof(uint32_t) * std::max<int64_t>(1, n_recs));
  if (e == cudaSuccess) e = cudaMalloc(&chunk, sizeof(uint32_t) * std::max<int64_t>(1, n_chunks));
  if (e == cudaSuccess) e = cudaMalloc(&total, sizeof(unsigned long long));
  if (e != cudaSuccess) {
    err = "basis build: scratch allocation failed";
    cudaFree(counts); cudaFree(chunk); cudaFree(total);
    return e;
  }
  const size_t smem = build_smem_bytes(S.V, torus);
  if (torus) {
    cudaFuncSetAttribute(k_basis_count<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_basis_count<true><<<grid_for((const void*)k_basis_count<true>, smem, n_recs), kBuildThreads, smem, st>>>(S.V, counts);
  } else {
    cudaFuncSetAttribute(k_basis_count<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_basis_count<false><<<grid_for((const void*)k_basis_count<false>, smem, n_recs), kBuildThreads, smem, st>>>(S.V, counts);
  }
  k_scan_chunks<<<(unsigned)n_chunks, kScanThreads, 0, st>>>(counts, n_recs, chunk);
  k_scan_sums<<<1, kScanThreads, 0, st>>>(chunk, n_chunks, total);
  k_scan_apply<<<(unsigned)n_chunks, kScanThreads, 0, st>>>(counts, n_recs, chunk, S.recs);
  unsigned long long n_p = 0;
  e = cudaMemcpyAsync(&n_p, total, sizeof(n_p), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    err = std::string("basis build: ") + cudaGetErrorString(e);
    cudaFree(counts); cudaFree(chunk); cudaFree(total);
    return e;
  }
  S.P.n_p = (int64_t)n_p;
  if (n_p > 0) {
    e = cudaMalloc(&S.reps, sizeof(uint64_t) * n_p);
    if (e == cudaSuccess) e = cudaMalloc(&S.lid, n_p);
    if (e != cudaSuccess) {
      err = "basis build: representative allocation failed";
      cudaFree(counts); cudaFree(chunk); cudaFree(total);
      return e;
    }
    S.device_bytes += sizeof(uint64_t) * n_p + n_p;
    if (torus) {
      cudaFuncSetAttribute(k_basis_emit<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k_basis_emit<true><<<grid_for((const void*)k_basis_emit<true>, smem, n_recs), kBuildThreads, smem, st>>>(
          S.V, counts, S.reps, S.lid);
    } else {
      cudaFuncSetAttribute(k_basis_emit<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k_basis_emit<false><<<grid_for((const void*)k_basis_emit<false>, smem, n_recs), kBuildThreads, smem, st>>>(
          S.V, counts, S.reps, S.lid);
    }
  }
  e = cudaStreamSynchronize(st);
  // The Lin-indexed records are not needed past this point.
  cudaFree(S.recs);
  S.device_bytes -= sizeof(RankRec) * std::max<int64_t>(1, n_recs);
  S.recs = nullptr;
  S.V.recs = nullptr;
  if (e == cudaSuccess && n_p > 0) {
    uint64_t max_rep = 0;
    e = cudaMemcpy(&max_rep, S.reps + (n_p - 1), sizeof(uint64_t), cudaMemcpyDeviceToHost);
    const int64_t nv = (int64_t)(max_rep / kRecBits) + 1;
    const int64_t nv_chunks = (nv + kScanChunk - 1) / kScanChunk;
    S.P.n_vrecs = nv;
    uint32_t* vcounts = nullptr;
    uint32_t* vchunk = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&S.vrecs, sizeof(RankRec) * nv);
    if (e == cudaSuccess) e = cudaMalloc(&vcounts, sizeof(uint32_t) * nv);
    if (e == cudaSuccess) e = cudaMalloc(&vchunk, sizeof(uint32_t) * nv_chunks);
    if (e == cudaSuccess) {
      S.device_bytes += sizeof(RankRec) * nv;
      cudaMemsetAsync(S.vrecs, 0, sizeof(RankRec) * nv, st);
      const int blocks = (int)std::min<int64_t>((n_p + 255) / 256, 152 * 64);
      k_vrank_mark<<<blocks, 256, 0, st>>>(S.reps, (int64_t)n_p, S.vrecs);
      const int cblocks = (int)std::min<int64_t>((nv + 255) / 256, 152 * 64);
      k_vrank_count<<<cblocks, 256, 0, st>>>(S.vrecs, nv, vcounts);
      k_scan_chunks<<<(unsigned)nv_chunks, kScanThreads, 0, st>>>(vcounts, nv, vchunk);
      k_scan_sums<<<1, kScanThreads, 0, st>>>(vchunk, nv_chunks, total);
      k_scan_apply<<<(unsigned)nv_chunks, kScanThreads, 0, st>>>(vcounts, nv, vchunk, S.vrecs);
      unsigned long long check = 0;
      e = cudaMemcpyAsync(&check, total, sizeof(check), cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e == cudaSuccess && check != n_p) {
        err = "basis build: value rank records disagree with the representative count";
        e = cudaErrorUnknown;
      }
    } else if (err.empty()) {
      err = "basis build: value rank records: out of device memory";
    }
    cudaFree(vcounts);
    cudaFree(vchunk);
    S.V.vrecs = S.vrecs;
  }
  cudaFree(counts);
  cudaFree(chunk);
  cudaFree(total);
  if (e != cudaSuccess && err.empty()) err = std::string("basis build: ") + cudaGetErrorString(e);
  return e;
}

cudaError_t export_walk_tables(const Sector& S, int64_t* rep_loc_dev, int32_t* g_dev, cudaStream_t st) {
  const size_t smem = (size_t)S.V.n_perm * S.V.n_chunks * 256 * sizeof(uint64_t);
  cudaFuncSetAttribute(k_walk_tables, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_walk_tables<<<grid_for((const void*)k_walk_tables, smem, S.P.n_configs), kBuildThreads, smem, st>>>(S.V, rep_loc_dev,
                                                                                                  g_dev);
  return cudaGetLastError();
}

}  // namespace edg
