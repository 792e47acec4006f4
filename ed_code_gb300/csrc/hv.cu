// Matrix-free H*v in the momentum basis: the role of sHv (H_v.cpp:192-357).
//
// One thread owns one basis row i (coalesced loads of reps/lid/v and a
// coalesced store of w).  Per row:
//   * the anti-aligned flip groups are found 64 at a time as a bit mask
//     (groups merge every bond and chirality term that flips the same pair);
//   * each one is flipped with one XOR, its representative and translation
//     come from the orbit search (row-rotation candidates on row-major tori,
//     the reference's walk otherwise), its position j from the value-indexed
//     rank records, its phase and norm ratio from shared-memory tables;
//   * w_i = sum_targets c(s)*phase*norm_i/norm_j*v_j + Ezz(s)*v_i, with
//     Ezz(s) = sum_bonds lambda*J/4 - 2*sum_{anti-aligned} lambda*J/4.
// ChCh bowtie terms (H_v.cpp:305-353) run as a separate per-row loop, only
// when |ChCh| > 1e-16 as in the reference.
//
// The grid is persistent (a fixed number of CTAs per SM striding over rows),
// so the per-CTA shared-memory staging of the term tables is paid once per
// CTA, not once per 256 rows.
#include <cuda_runtime.h>

#include <algorithm>

#include "edg_sector.cuh"

namespace edg {

namespace {

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
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

template <typename Real>
__host__ __device__ inline size_t hv_smem_bytes(int n_groups, int n_ch, bool torus, int row_bits, int n_chunks) {
  size_t b = align16(sizeof(SmemGroup<Real>) * n_groups);
  b += align16(sizeof(SmemCh<Real>) * n_ch);
  b += align16(sizeof(Real) * (64 + 64 + 65 + 65));
  if (torus) b += align16((size_t)3 << row_bits);
  else b += (size_t)2 * n_chunks * 256 * sizeof(uint64_t);
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
    const int n = 2 * V.n_chunks * 256;
    uint64_t* p = reinterpret_cast<uint64_t*>(sm + off);
    for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = V.perms[i];
    H.p1 = p;
    H.p2 = p + V.n_chunks * 256;
  }
  return H;
}

template <typename Real, bool kTorus>
__device__ __forceinline__ Orbit search(uint64_t t, const SectorParams& P, const HvSmem<Real>& H, int n_chunks) {
  if (kTorus) return orbit_torus(t, P, H.nk, H.rots);
  return orbit_walk(t, P, H.p1, H.p2, n_chunks);
}

// Position j of the representative o.rep; j < 0 when it is not an allowed
// state (the reference's rep_loc < 0).
__device__ __forceinline__ int64_t position(const Orbit& o, const SectorView& V, const SectorParams& P) {
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

template <typename Real, bool kTorus, bool kChCh>
__global__ void __launch_bounds__(kHvThreads, 4) k_hv(SectorView V, const typename C2<Real>::T* __restrict__ v,
                                                   typename C2<Real>::T* __restrict__ w) {
  using CT = typename C2<Real>::T;
  __shared__ SectorParams P;
  extern __shared__ __align__(16) uint8_t sm[];
  for (int i = threadIdx.x; i < (int)(sizeof(SectorParams) / 8); i += blockDim.x)
    reinterpret_cast<uint64_t*>(&P)[i] = reinterpret_cast<const uint64_t*>(V.params)[i];
  __syncthreads();
  const HvSmem<Real> H = stage_hv<Real, kTorus>(V, P, sm);
  __syncthreads();

  const int64_t n_p = P.n_p;
  const int ng = P.n_groups;
  const bool use_ch = P.use_ch != 0;
  const Real total_fac = (Real)P.total_fac;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_p; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t s = __ldg(reinterpret_cast<const unsigned long long*>(V.reps) + i);
    const int li = __ldg(V.lid + i);
    const CT vi = v[i];
    const Real norm_i = H.nrm[li];
    Real accr = 0, acci = 0, anti = 0;
    RowInfo ri{0, false};
    if (kTorus) ri = torus_row_info(s, P, H);
    const int top = P.L2 - 1;
    const uint64_t rmask = (1ull << P.L1) - 1ull;
    for (int g0 = 0; g0 < ng; g0 += 64) {
      const int gn = min(64, ng - g0);
      uint64_t am = 0;
      for (int k = 0; k < gn; ++k) {
        const uint64_t m = H.groups[g0 + k].mask;
        am |= (uint64_t)(popc64(s & m) == 1) << k;
      }
      while (am) {
        const int g = g0 + ffs64(am);
        am &= am - 1;
        const SmemGroup<Real>& gr = H.groups[g];
        anti += gr.fac;
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
        const uint64_t t = s ^ gr.mask;
        Orbit o;
        bool fast = false;
        if (kTorus && ri.uniq && gr.ya != top && gr.yb != top) {
          const int na = H.nk[(int)((t >> (P.L1 * gr.ya)) & rmask)];
          const int nb = H.nk[(int)((t >> (P.L1 * gr.yb)) & rmask)];
          if (na > ri.mstar && nb > ri.mstar) {
            o.rep = t;
            o.g = 0;
            o.stab = 1;
            fast = true;
          }
        }
        if (!fast) o = search<Real, kTorus>(t, P, H, V.n_chunks);
        const int64_t j = position(o, V, P);
        if (j >= 0) {
          const Real sc = norm_i * H.nrm_inv[o.stab];
          const Real pr = H.ph_re[o.g], pi = H.ph_im[o.g];
          const Real er = (cr * pr - ci * pi) * sc;
          const Real ei = (cr * pi + ci * pr) * sc;
          const CT vj = v[j];
          accr += er * vj.x - ei * vj.y;
          acci += er * vj.y + ei * vj.x;
        }
      }
    }
    if (kChCh) {
      // ChCh (H_v.cpp:305-353): two successive pair flips, term by term.
      const Real chch = (Real)(P.ChCh * 0.25 * 0.25);
      for (int k = 0; k < P.n_bowties; ++k) {
        const Bowtie b = V.bows[k];
        const int tx = (int)((s >> b.x) & 1u), ty = (int)((s >> b.y) & 1u);
        if (tx == ty) continue;
        // ch_sgn1 = (ty ? i : -i), negated when bit z of the flipped state is 0
        Real s1 = ty ? Real(1) : Real(-1);
        const uint64_t tmp = s ^ ((1ull << b.x) | (1ull << b.y));
        if (!((tmp >> b.z) & 1u)) s1 = -s1;
        const int tp = (int)((tmp >> b.p) & 1u), tq = (int)((tmp >> b.q) & 1u);
        if (tp == tq) continue;
        Real s2 = tq ? Real(1) : Real(-1);
        const uint64_t tmp2 = tmp ^ ((1ull << b.p) | (1ull << b.q));
        if (!((tmp2 >> b.r) & 1u)) s2 = -s2;
        Orbit o;
        const int64_t j = locate<Real, kTorus>(tmp2, V, P, H, o);
        if (j >= 0) {
          // (i s1)(i s2) = -s1 s2
          const Real sc = -chch * s1 * s2 * norm_i * H.nrm_inv[o.stab];
          const Real er = H.ph_re[o.g] * sc, ei = H.ph_im[o.g] * sc;
          const CT vj = v[j];
          accr += er * vj.x - ei * vj.y;
          acci += er * vj.y + ei * vj.x;
        }
      }
    }
    const Real ezz = total_fac - Real(2) * anti;
    CT out;
    out.x = accr + ezz * vi.x;
    out.y = acci + ezz * vi.y;
    w[i] = out;
  }
}

template <bool kTorus>
__global__ void __launch_bounds__(kHvThreads) k_count_offdiag(SectorView V, unsigned long long* __restrict__ nnz) {
  __shared__ SectorParams P;
  extern __shared__ __align__(16) uint8_t sm[];
  for (int i = threadIdx.x; i < (int)(sizeof(SectorParams) / 8); i += blockDim.x)
    reinterpret_cast<uint64_t*>(&P)[i] = reinterpret_cast<const uint64_t*>(V.params)[i];
  __syncthreads();
  const HvSmem<float> H = stage_hv<float, kTorus>(V, P, sm);
  __syncthreads();
  unsigned long long cnt = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < P.n_p; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t s = V.reps[i];
    for (int g = 0; g < P.n_groups; ++g) {
      const uint64_t m = H.groups[g].mask;
      if (popc64(s & m) != 1) continue;
      Orbit o;
      if (locate<float, kTorus>(s ^ m, V, P, H, o) >= 0) ++cnt;
    }
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(nnz, cnt);
}

template <typename K>
int persistent_grid(K kernel, size_t smem, int64_t rows) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kHvThreads, smem);
  if (per_sm < 1) per_sm = 1;
  int64_t want = (rows + kHvThreads - 1) / kHvThreads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms * per_sm));
}

template <typename Real, bool kTorus, bool kChCh>
cudaError_t launch_t(const Sector& S, const void* v, void* w, cudaStream_t st) {
  using CT = typename C2<Real>::T;
  const size_t smem = hv_smem_bytes<Real>(S.P.n_groups, S.P.n_ch, kTorus, S.V.row_bits, S.V.n_chunks);
  auto kern = k_hv<Real, kTorus, kChCh>;
  const int grid = persistent_grid(kern, smem, S.P.n_p);
  kern<<<grid, kHvThreads, smem, st>>>(S.V, reinterpret_cast<const CT*>(v), reinterpret_cast<CT*>(w));
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_hv(const Sector& S, const void* v, void* w, bool fp64, cudaStream_t st) {
  if (S.tplan && S.hv_variant == 1) return launch_hv_torus(S, v, w, fp64, st);
  return launch_hv_generic(S, v, w, fp64, st);
}

cudaError_t launch_hv_generic(const Sector& S, const void* v, void* w, bool fp64, cudaStream_t st) {
  const bool torus = S.P.torus != 0, chch = S.P.use_chch != 0;
  if (fp64) {
    if (torus) return chch ? launch_t<double, true, true>(S, v, w, st) : launch_t<double, true, false>(S, v, w, st);
    return chch ? launch_t<double, false, true>(S, v, w, st) : launch_t<double, false, false>(S, v, w, st);
  }
  if (torus) return chch ? launch_t<float, true, true>(S, v, w, st) : launch_t<float, true, false>(S, v, w, st);
  return chch ? launch_t<float, false, true>(S, v, w, st) : launch_t<float, false, false>(S, v, w, st);
}

cudaError_t count_offdiag(const Sector& S, unsigned long long* nnz_dev, cudaStream_t st) {
  const bool torus = S.P.torus != 0;
  const size_t smem = hv_smem_bytes<float>(S.P.n_groups, S.P.n_ch, torus, S.V.row_bits, S.V.n_chunks);
  cudaMemsetAsync(nnz_dev, 0, sizeof(unsigned long long), st);
  if (torus) {
    const int grid = persistent_grid(k_count_offdiag<true>, smem, S.P.n_p);
    k_count_offdiag<true><<<grid, kHvThreads, smem, st>>>(S.V, nnz_dev);
  } else {
    const int grid = persistent_grid(k_count_offdiag<false>, smem, S.P.n_p);
    k_count_offdiag<false><<<grid, kHvThreads, smem, st>>>(S.V, nnz_dev);
  }
  return cudaGetLastError();
}

}  // namespace edg
