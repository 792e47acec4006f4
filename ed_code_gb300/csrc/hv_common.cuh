// Device helpers shared by the H*v kernels (hv.cu) and the stored-target
// build (targets.cu): shared-memory staging of the term tables, the orbit
// search dispatch and the position lookup.
#pragma once
#include <cuda_runtime.h>

#include "edg_sector.cuh"

namespace edg {

constexpr int kHvThreads = 256;

template <typename Real>
struct C2;
template <>
struct C2<float> { using T = float2; };
template <>
struct C2<double> { using T = double2; };

template <typename Real>
struct HvSmem {
  SmemGroup<Real>* groups;
  SmemCh<Real>* ch;
  Real* ph_re;
  Real* ph_im;
  Real* nrm;
  Real* nrm_inv;
  const uint8_t* nk;
  const uint16_t* rots;
  const uint64_t* p1;
  const uint64_t* p2;
  const uint64_t* p3;  // T3 (3-D tori only)
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

template <typename Real>
__host__ __device__ inline size_t hv_smem_bytes(int n_groups, int n_ch, bool torus, int row_bits, int n_chunks,
                                                int n_perm) {
  size_t b = align16(sizeof(SmemGroup<Real>) * n_groups);
  b += align16(sizeof(SmemCh<Real>) * n_ch);
  b += align16(sizeof(Real) * (64 + 64 + 65 + 65));
  if (torus) b += align16((size_t)3 << row_bits);
  else b += (size_t)n_perm * n_chunks * 256 * sizeof(uint64_t);
  return b;
}

template <typename Real, bool kTorus>
__device__ HvSmem<Real> stage_hv(const SectorView& V, const SectorParams& P, uint8_t* sm) {
  HvSmem<Real> H{};
  size_t off = 0;
  H.groups = reinterpret_cast<SmemGroup<Real>*>(sm + off);
  off += align16(sizeof(SmemGroup<Real>) * P.n_groups);
  H.ch = reinterpret_cast<SmemCh<Real>*>(sm + off);
  off += align16(sizeof(SmemCh<Real>) * P.n_ch);
  Real* tab = reinterpret_cast<Real*>(sm + off);
  H.ph_re = tab;
  H.ph_im = tab + 64;
  H.nrm = tab + 128;
  H.nrm_inv = tab + 193;
  off += align16(sizeof(Real) * (64 + 64 + 65 + 65));
  for (int g = threadIdx.x; g < P.n_groups; g += blockDim.x) {
    const TermGroup src = V.groups[g];
    SmemGroup<Real> d;
    d.mask = src.mask;
    d.fac = (Real)src.fac;
    d.Bre[0] = (Real)src.Bre[0];
    d.Bre[1] = (Real)src.Bre[1];
    d.Bim[0] = (Real)src.Bim[0];
    d.Bim[1] = (Real)src.Bim[1];
    d.a = (int16_t)src.a;
    d.ch_begin = (int16_t)src.ch_begin;
    d.ch_end = (int16_t)src.ch_end;
    d.ya = (int8_t)(kTorus ? src.a / P.L1 : -1);
    d.yb = (int8_t)(kTorus ? src.b / P.L1 : -1);
    H.groups[g] = d;
  }
  for (int m = threadIdx.x; m < P.n_ch; m += blockDim.x) {
    const ChTerm src = V.ch[m];
    SmemCh<Real> d;
    d.Are[0] = (Real)src.Are[0];
    d.Are[1] = (Real)src.Are[1];
    d.Aim[0] = (Real)src.Aim[0];
    d.Aim[1] = (Real)src.Aim[1];
    d.z = src.z;
    H.ch[m] = d;
  }
  for (int k = threadIdx.x; k < 64; k += blockDim.x) {
    H.ph_re[k] = (Real)P.ph_re[k];
    H.ph_im[k] = (Real)P.ph_im[k];
  }
  for (int k = threadIdx.x; k < 65; k += blockDim.x) {
    H.nrm[k] = (Real)P.nrm[k];
    H.nrm_inv[k] = (Real)P.nrm_inv[k];
  }
  if (kTorus) {
    const int n = 1 << V.row_bits;
    uint16_t* rots = reinterpret_cast<uint16_t*>(sm + off);
    uint8_t* nk = sm + off + 2 * n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      rots[i] = V.rots[i];
      nk[i] = V.nk[i];
    }
    H.nk = nk;
    H.rots = rots;
  } else {
    const int n = V.n_perm * V.n_chunks * 256;
    uint64_t* p = reinterpret_cast<uint64_t*>(sm + off);
    for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = V.perms[i];
    H.p1 = p;
    H.p2 = p + V.n_chunks * 256;
    H.p3 = p + 2 * V.n_chunks * 256;
  }
  return H;
}

template <typename Real, bool kTorus>
__device__ __forceinline__ Orbit search(uint64_t t, const SectorParams& P, const HvSmem<Real>& H, int n_chunks) {
  if (kTorus) return orbit_torus(t, P, H.nk, H.rots);
  return orbit_walk(t, P, H.p1, H.p2, H.p3, n_chunks);
}

// Position j of the representative o.rep; j < 0 when it is not an allowed
// state (the reference's rep_loc < 0).
static __device__ __forceinline__ int64_t position(const Orbit& o, const SectorView& V, const SectorParams& P) {
  // A translate of t is an n_sites-bit word; anything else means the search
  // found no candidate, and is treated as "no allowed representative" rather
  // than used as a table index.
  if (o.rep & ~P.full_mask) return -1;
  if ((unsigned)o.g >= 64u || (unsigned)o.stab > 64u) return -1;
  int bit;
  const uint32_t q = vrec_of(o.rep, &bit);
  if ((int64_t)q >= P.n_vrecs) return -1;  // larger than every representative
  const uint4 raw = __ldg(reinterpret_cast<const uint4*>(V.vrecs) + q);
  RankRec rec;
  rec.base = raw.x;
  rec.bits[0] = raw.y;
  rec.bits[1] = raw.z;
  rec.bits[2] = raw.w;
  return rank_lookup_bit(bit, rec);
}

template <typename Real, bool kTorus>
__device__ __forceinline__ int64_t locate(uint64_t t, const SectorView& V, const SectorParams& P,
                                          const HvSmem<Real>& H, Orbit& o) {
  o = search<Real, kTorus>(t, P, H, V.n_chunks);
  return position(o, V, P);
}

// Row-level facts for the torus fast path.  s is a representative, so its top
// row is at its rotation minimum and no row has a smaller one.  When the top
// row is the only row reaching that minimum and it is aperiodic, the identity
// is the only candidate translation of s -- and of every flip of s that leaves
// the top row alone and gives no other row a rotation minimum <= mstar.  Such
// a flipped state is its own representative with stabiliser 1.
struct RowInfo {
  int mstar;
  bool uniq;
};
template <typename Real>
__device__ __forceinline__ RowInfo torus_row_info(uint64_t s, const SectorParams& P, const HvSmem<Real>& H) {
  const int Lx = P.L1, Ly = P.L2;
  const uint64_t rmask = (1ull << Lx) - 1ull;
  const int rtop = (int)((s >> (Lx * (Ly - 1))) & rmask);
  RowInfo r;
  r.mstar = H.nk[rtop];
  int cnt = 0;
  for (int y = 0; y < Ly; ++y) cnt += (H.nk[(int)((s >> (Lx * y)) & rmask)] == r.mstar);
  r.uniq = (cnt == 1) && (H.rots[rtop] == 1u);
  return r;
}


}  // namespace edg
