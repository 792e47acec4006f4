// Pieces of the stored-row H*v shared by the single-sector kernel
// (targets.cu) and the batch (batch.cu): the complex type of a precision, the
// L2 cache policies of the loads, and one CSR row's sum over LPR lanes.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace edg {
namespace {

template <typename Real>
struct CT2;
template <>
struct CT2<float> { using T = float2; };
template <>
struct CT2<double> { using T = double2; };

// Cache policy of the CSR loads (tuned per sector with the lanes per row).
// The row data (col, vid) are read once per H*v; the gathered u entries are
// reused by other rows while they stay in L2.  Policy 1 reads the row data
// with the streaming hint (ld.global.cs); policy 2 gives them the L2
// evict_first priority instead.  Both give the u gathers L2 evict_last.  At
// 36 sites (a 2 GB u against a 129 MB L2) policy 2 measured 68 ms against
// 84 ms; at 30-32 sites policy 1 is the faster one.
__device__ __forceinline__ uint64_t l2_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
template <int kPol>
__device__ __forceinline__ uint32_t ld_row(const uint32_t* a, uint64_t pol) {
  if (kPol == 1) return __ldcs(a);
  uint32_t r;
  asm volatile("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(r) : "l"(a), "l"(pol));
  return r;
}
template <int kPol>
__device__ __forceinline__ int ld_row(const uint16_t* a, uint64_t pol) {
  if (kPol == 1) return __ldcs(a);
  uint16_t r;
  asm volatile("ld.global.nc.L2::cache_hint.u16 %0, [%1], %2;" : "=h"(r) : "l"(a), "l"(pol));
  return r;
}
__device__ __forceinline__ float2 ld_keep(const float2* a, uint64_t pol) {
  float2 r;
  asm volatile("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(r.x), "=f"(r.y) : "l"(a), "l"(pol));
  return r;
}
__device__ __forceinline__ double2 ld_keep(const double2* a, uint64_t pol) {
  double2 r;
  asm volatile("ld.global.nc.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;" : "=d"(r.x), "=d"(r.y) : "l"(a), "l"(pol));
  return r;
}

// acc += c * x for complex c, x, as explicit FMAs in a fixed order, so every
// kernel that sums rows (single vector, block, batch) rounds the same way
// whatever the compiler would have contracted.
__device__ __forceinline__ float fmaR(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmaR(double a, double b, double c) { return fma(a, b, c); }
template <typename Real, typename CT>
__device__ __forceinline__ void cmac(Real& ar, Real& ai, const CT& c, const CT& x) {
  ar = fmaR(c.x, x.x, fmaR(-c.y, x.y, ar));
  ai = fmaR(c.x, x.y, fmaR(c.y, x.x, ai));
}
// a row's result: norm_i * sum + Ezz_i * v_i
template <typename Real, typename CT>
__device__ __forceinline__ CT row_out(Real ar, Real ai, Real ni, Real d, const CT& vi) {
  CT out;
  out.x = fmaR(ar, ni, d * vi.x);
  out.y = fmaR(ai, ni, d * vi.y);
  return out;
}

// Entry formats of the stored rows.  kSplit: a u32 column array and a u16
// value-id array (6 bytes an entry).  kPacked: one u32 an entry, the column
// in the low cb bits and the value id above them (4 bytes), used when the
// deduplicated value table and the sector size leave room (cb < 32 and
// n_p < 2^cb, so no entry is all ones).  kByVid: either, chosen per segment
// by vid == nullptr (the batch, whose segments may differ).
constexpr int kSplit = 0, kPacked = 1, kByVid = 2;

template <int kFmt, int kPol>
__device__ __forceinline__ void ld_entry(const uint32_t* col, const uint16_t* vid, uint64_t t, int cb, uint64_t pf,
                                         uint32_t& j, int& id) {
  const bool packed = kFmt == kPacked || (kFmt == kByVid && vid == nullptr);
  const uint32_t e = ld_row<kPol>(col + t, pf);
  if (packed) {
    j = e & ((1u << cb) - 1u);
    id = (int)(e >> cb);
  } else {
    j = e;
    id = ld_row<kPol>(vid + t, pf);
  }
}

// Entries a lane resolves in the unrolled head of a row (LPR lanes a row).
template <int LPR>
__host__ __device__ constexpr int head_entries() {
  return 64 / LPR < 2 ? 2 : 64 / LPR;
}

// The head of one CSR row: lane sl loads entries beg + sl + LPR*q (q < kU) as
// stored (e: the u32 word, h: the u16 value id of split rows), all ones past
// the row's end.  No valid entry is all ones (a column is below n_p < 2^32 - 1,
// and below 2^cb when packed).
template <int LPR, int kFmt, int kPol>
__device__ __forceinline__ void csr_head(uint64_t beg, uint64_t end, int sl, const uint32_t* __restrict__ col,
                                         const uint16_t* __restrict__ vid, uint64_t pf,
                                         uint32_t (&e)[head_entries<LPR>()], uint16_t (&h)[head_entries<LPR>()]) {
  constexpr int kU = head_entries<LPR>();
  const bool packed = kFmt == kPacked || (kFmt == kByVid && vid == nullptr);
#pragma unroll
  for (int q = 0; q < kU; ++q) {
    const uint64_t t = beg + sl + LPR * q;
    e[q] = 0xFFFFFFFFu;
    h[q] = 0;
    if (t < end) {
      e[q] = ld_row<kPol>(col + t, pf);
      if (!packed) h[q] = (uint16_t)ld_row<kPol>(vid + t, pf);
    }
  }
}

// The head's gathers: x[q] = u[column of e[q]] for the valid entries.
template <typename Real, int LPR, int kFmt>
__device__ __forceinline__ void csr_gather(const uint16_t* vid, int cb, const typename CT2<Real>::T* __restrict__ u,
                                           uint64_t pl, const uint32_t (&e)[head_entries<LPR>()],
                                           typename CT2<Real>::T (&x)[head_entries<LPR>()]) {
  constexpr int kU = head_entries<LPR>();
  const bool packed = kFmt == kPacked || (kFmt == kByVid && vid == nullptr);
  const uint32_t cmask = packed ? (1u << cb) - 1u : 0xFFFFFFFFu;
#pragma unroll
  for (int q = 0; q < kU; ++q)
    if (e[q] != 0xFFFFFFFFu) x[q] = ld_keep(u + (e[q] & cmask), pl);
}

// The row sum once the head's gathers are issued: the head's products, then
// the entries past the head in a loop, then a segmented reduction that
// leaves the row sum in lane sl == 0.
template <typename Real, int LPR, bool kSmemTab, int kPol, int kFmt>
__device__ __forceinline__ void csr_consume(uint64_t beg, uint64_t end, int sl, const uint32_t* __restrict__ col,
                                            const uint16_t* __restrict__ vid, int cb,
                                            const typename CT2<Real>::T* vtab,
                                            const typename CT2<Real>::T* __restrict__ u, uint64_t pf, uint64_t pl,
                                            const uint32_t (&e)[head_entries<LPR>()],
                                            const uint16_t (&h)[head_entries<LPR>()],
                                            const typename CT2<Real>::T (&x)[head_entries<LPR>()], Real& ar,
                                            Real& ai) {
  using CT = typename CT2<Real>::T;
  constexpr int kU = head_entries<LPR>();
  const bool packed = kFmt == kPacked || (kFmt == kByVid && vid == nullptr);
  ar = 0;
  ai = 0;
#pragma unroll
  for (int q = 0; q < kU; ++q) {
    if (e[q] == 0xFFFFFFFFu) continue;
    const int id = packed ? (int)(e[q] >> cb) : (int)h[q];
    const CT c = kSmemTab ? vtab[id] : __ldg(vtab + id);
    cmac(ar, ai, c, x[q]);
  }
  for (uint64_t t = beg + sl + LPR * kU; t < end; t += LPR) {
    uint32_t jt;
    int idt;
    ld_entry<kFmt, kPol>(col, vid, t, cb, pf, jt, idt);
    const CT c = kSmemTab ? vtab[idt] : __ldg(vtab + idt);
    const CT y = ld_keep(u + jt, pl);
    cmac(ar, ai, c, y);
  }
#pragma unroll
  for (int o = LPR / 2; o > 0; o >>= 1) {
    ar += __shfl_down_sync(0xffffffffu, ar, o, LPR);
    ai += __shfl_down_sync(0xffffffffu, ai, o, LPR);
  }
}

// Gathers and row sum of a row whose head is loaded.
template <typename Real, int LPR, bool kSmemTab, int kPol, int kFmt>
__device__ __forceinline__ void csr_finish(uint64_t beg, uint64_t end, int sl, const uint32_t* __restrict__ col,
                                           const uint16_t* __restrict__ vid, int cb,
                                           const typename CT2<Real>::T* vtab,
                                           const typename CT2<Real>::T* __restrict__ u, uint64_t pf, uint64_t pl,
                                           const uint32_t (&e)[head_entries<LPR>()],
                                           const uint16_t (&h)[head_entries<LPR>()], Real& ar, Real& ai) {
  typename CT2<Real>::T x[head_entries<LPR>()];
  csr_gather<Real, LPR, kFmt>(vid, cb, u, pl, e, x);
  csr_consume<Real, LPR, kSmemTab, kPol, kFmt>(beg, end, sl, col, vid, cb, vtab, u, pf, pl, e, h, x, ar, ai);
}

// One CSR row, handled by LPR lanes of a warp (sl = lane within the row).
// The row's first LPR*kU entries are resolved in one unrolled step -- all
// entry loads, then all gathers -- longer rows finish in a loop.
// Returns the row sum in lane sl == 0 after a segmented reduction.
template <typename Real, int LPR, bool kSmemTab, int kPol, int kFmt>
__device__ __forceinline__ void csr_row(uint64_t beg, uint64_t end, int sl, const uint32_t* __restrict__ col,
                                        const uint16_t* __restrict__ vid, int cb, const typename CT2<Real>::T* vtab,
                                        const typename CT2<Real>::T* __restrict__ u, Real& ar, Real& ai) {
  constexpr int kU = head_entries<LPR>();
  const uint64_t pf = kPol == 2 ? l2_evict_first() : 0, pl = l2_evict_last();
  uint32_t e[kU];
  uint16_t h[kU];
  csr_head<LPR, kFmt, kPol>(beg, end, sl, col, vid, pf, e, h);
  csr_finish<Real, LPR, kSmemTab, kPol, kFmt>(beg, end, sl, col, vid, cb, vtab, u, pf, pl, e, h, ar, ai);
}

}  // namespace
}  // namespace edg
