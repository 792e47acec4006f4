// H*v specialised for row-major tori (T1 = +x, T2 = +y, Lx, Ly <= 8): the
// same row formula as hv.cu (sHv, H_v.cpp:192-357), with the per-row and
// per-target integer work cut down:
//
//  * anti-aligned pairs: one XOR with the translated state per displacement
//    class (TorusPlan) instead of one test per pair;
//  * the row values of s and their rotation minima are packed into bytes once
//    per row; a flip changes at most two rows, so a target needs two table
//    lookups to decide between
//      - the fast case: s's top row is the only row at the minimum rotation
//        value and is aperiodic, the flip leaves the top row alone and gives no
//        other row a rotation minimum <= it.  Then the flipped state is its own
//        representative (translation 0, stabiliser 1);
//      - the search: candidates are the rows at the smallest rotation minimum,
//        rotated to it; the smallest full translate wins and the number of
//        ties is the stabiliser;
//  * the coefficient of a pair is its bond part plus at most two chirality
//    terms, signed by bits z1, z2 of s;
//  * the position of the representative comes from the value-indexed rank
//    records: one 16-byte load, no Lin index;
//  * each thread resolves two targets before it loads, so the rank-record and
//    v loads of both are in flight together;
//  * norm_i multiplies the row sum once.
#include <cuda_runtime.h>

#include <algorithm>

#include "edg_sector.cuh"

namespace edg {

namespace {

constexpr int kThreads = 256;

template <typename Real>
struct C2;
template <>
struct C2<float> { using T = float2; };
template <>
struct C2<double> { using T = double2; };

template <typename Real>
struct TG {  // shared-memory copy of a TorusGroup in the working precision
  uint64_t mask;
  Real B[4], A1[4], A2[4];
  Real fac;
  uint8_t a, z1, z2, ya, yb, da, db, same_row;
};

// Up to 8 byte-sized values in one 64-bit word (byte y = row y).
__device__ __forceinline__ int byte_at(uint64_t x, int y) {
  return (int)(__byte_perm((uint32_t)x, (uint32_t)(x >> 32), (unsigned)y) & 0xFFu);
}
__device__ __forceinline__ uint64_t with_byte(uint64_t x, int y, int v) {
  return x ^ ((uint64_t)(byte_at(x, y) ^ v) << (8 * y));
}

__device__ __forceinline__ uint64_t rot_rows(uint64_t t, int shift, int N, uint64_t full) {
  return shift ? (((t << shift) | (t >> (N - shift))) & full) : t;
}
__device__ __forceinline__ uint64_t rot_within(uint64_t u, int a, int Lx, const uint64_t* hi, const uint64_t* lo) {
  return a ? (((u << a) & hi[a]) | ((u >> (Lx - a)) & lo[a])) : u;
}

// One target of row s: representative, translation, stabiliser, coefficient.
template <typename Real>
struct Target {
  uint64_t rep;
  int g, stab;
  Real cr, ci;
};

template <typename Real>
__device__ __forceinline__ Target<Real> resolve(uint64_t s, const TG<Real>& gr, uint64_t rw, uint64_t nks, int mstar,
                                                bool uniq, int top, const SectorParams& P, const uint8_t* nk,
                                                const uint16_t* rots) {
  Target<Real> T;
  const int cs = (int)((s >> gr.a) & 1u);
  const Real s1 = ((s >> gr.z1) & 1u) ? Real(1) : Real(-1);
  const Real s2 = ((s >> gr.z2) & 1u) ? Real(1) : Real(-1);
  T.cr = gr.B[2 * cs] + s1 * gr.A1[2 * cs] + s2 * gr.A2[2 * cs];
  T.ci = gr.B[2 * cs + 1] + s1 * gr.A1[2 * cs + 1] + s2 * gr.A2[2 * cs + 1];
  const uint64_t t = s ^ gr.mask;
  // the rows of t that differ from s
  int Ra = byte_at(rw, gr.ya) ^ gr.da;
  int Rb = byte_at(rw, gr.yb) ^ gr.db;
  if (gr.same_row) Rb = Ra = Ra ^ gr.db;
  const int na = nk[Ra], nb = nk[Rb];
  if (uniq && gr.ya != top && gr.yb != top && na > mstar && nb > mstar) {
    T.rep = t;
    T.g = 0;
    T.stab = 1;
    return T;
  }
  const int Lx = P.L1, N = P.n_sites;
  uint64_t rt = with_byte(rw, gr.ya, Ra);
  rt = with_byte(rt, gr.yb, Rb);
  uint64_t nt = with_byte(nks, gr.ya, na);
  nt = with_byte(nt, gr.yb, nb);
  uint32_t mm = __vminu4((uint32_t)nt, (uint32_t)(nt >> 32));
  mm = __vminu4(mm, mm >> 16);
  mm = __vminu4(mm, mm >> 8);
  const uint32_t bc = (mm & 0xFFu) * 0x01010101u;
  // one set bit (bit 8y) per row y whose rotation minimum is the smallest
  uint64_t cand = ((uint64_t)(__vcmpeq4((uint32_t)(nt >> 32), bc) & 0x01010101u) << 32) |
                  (uint64_t)(__vcmpeq4((uint32_t)nt, bc) & 0x01010101u);
  if (top < 7) cand &= (1ull << (8 * (top + 1))) - 1ull;  // rows that exist
  T.rep = ~0ull;
  T.g = 0;
  T.stab = 0;
  while (cand) {
    const int y = ffs64(cand) >> 3;
    cand &= cand - 1;
    const int b = top - y;
    const uint64_t u2 = rot_rows(t, Lx * b, N, P.full_mask);
    uint32_t rs = rots[byte_at(rt, y)];
    while (rs) {
      const int a = __ffs(rs) - 1;
      rs &= rs - 1;
      const uint64_t Vt = rot_within(u2, a, Lx, P.rot_hi, P.rot_lo);
      if (Vt < T.rep) {
        T.rep = Vt;
        T.g = a + Lx * b;
        T.stab = 1;
      } else if (Vt == T.rep) {
        ++T.stab;
      }
    }
  }
  return T;
}

// Position of the representative by its value; -1 when not allowed.
__device__ __forceinline__ int64_t vrank(uint64_t rep, const RankRec* __restrict__ vrecs, int64_t n_vrecs) {
  int bit;
  const uint32_t q = vrec_of(rep, &bit);
  if ((int64_t)q >= n_vrecs) return -1;
  const uint4 raw = __ldg(reinterpret_cast<const uint4*>(vrecs) + q);
  RankRec rec;
  rec.base = raw.x;
  rec.bits[0] = raw.y;
  rec.bits[1] = raw.z;
  rec.bits[2] = raw.w;
  return rank_lookup_bit(bit, rec);
}

template <typename Real>
__global__ void __launch_bounds__(kThreads, 2) k_hv_torus(SectorView V, const TorusPlan* __restrict__ plan,
                                                          const TorusGroup* __restrict__ tgroups,
                                                          const typename C2<Real>::T* __restrict__ v,
                                                          typename C2<Real>::T* __restrict__ w) {
  using CT = typename C2<Real>::T;
  __shared__ SectorParams P;
  __shared__ TorusPlan TP;
  __shared__ uint8_t nk[256];
  __shared__ uint16_t rots[256];
  __shared__ Real ph_re[64], ph_im[64], nrm[65], nrm_inv[65];
  extern __shared__ __align__(16) uint8_t sm[];
  TG<Real>* G = reinterpret_cast<TG<Real>*>(sm);

  for (int i = threadIdx.x; i < (int)(sizeof(SectorParams) / 8); i += blockDim.x)
    reinterpret_cast<uint64_t*>(&P)[i] = reinterpret_cast<const uint64_t*>(V.params)[i];
  for (int i = threadIdx.x; i < (int)(sizeof(TorusPlan) / 8); i += blockDim.x)
    reinterpret_cast<uint64_t*>(&TP)[i] = reinterpret_cast<const uint64_t*>(plan)[i];
  for (int i = threadIdx.x; i < (1 << V.row_bits); i += blockDim.x) {
    nk[i] = V.nk[i];
    rots[i] = V.rots[i];
  }
  __syncthreads();
  for (int k = threadIdx.x; k < 64; k += blockDim.x) {
    ph_re[k] = (Real)P.ph_re[k];
    ph_im[k] = (Real)P.ph_im[k];
  }
  for (int k = threadIdx.x; k < 65; k += blockDim.x) {
    nrm[k] = (Real)P.nrm[k];
    nrm_inv[k] = (Real)P.nrm_inv[k];
  }
  for (int g = threadIdx.x; g < P.n_groups; g += blockDim.x) {
    const TorusGroup s = tgroups[g];
    TG<Real> d;
    d.mask = s.mask;
    for (int q = 0; q < 4; ++q) {
      d.B[q] = (Real)s.B[q];
      d.A1[q] = (Real)s.A1[q];
      d.A2[q] = (Real)s.A2[q];
    }
    d.fac = (Real)s.fac;
    d.a = s.a;
    d.z1 = s.z1;
    d.z2 = s.z2;
    d.ya = s.ya;
    d.yb = s.yb;
    d.da = s.da;
    d.db = s.db;
    d.same_row = s.same_row;
    G[g] = d;
  }
  __syncthreads();

  const int Lx = P.L1, Ly = P.L2, N = P.n_sites, top = Ly - 1;
  const uint64_t rmask = (1ull << Lx) - 1ull, full = P.full_mask;
  const Real total_fac = (Real)P.total_fac;
  const int n_classes = TP.n_classes;
  const int64_t n_vrecs = P.n_vrecs;
  const RankRec* __restrict__ vrecs = V.vrecs;

  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < P.n_p; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t s = __ldg(reinterpret_cast<const unsigned long long*>(V.reps) + i);
    const int li = __ldg(V.lid + i);
    const CT vi = v[i];
    // row values of s and their rotation minima, one byte per row; unused
    // bytes of the minima are 0xFF so they never win a minimum
    uint64_t rw = 0, nks = ~0ull;
    for (int y = 0; y < Ly; ++y) {
      const int r = (int)((s >> (Lx * y)) & rmask);
      rw |= (uint64_t)r << (8 * y);
      nks = with_byte(nks, y, nk[r]);
    }
    const int rtop = byte_at(rw, top);
    const int mstar = nk[rtop];
    int n_eq = 0;
    for (int y = 0; y < Ly; ++y) n_eq += (byte_at(nks, y) == mstar);
    const bool uniq = (n_eq == 1) && (rots[rtop] == 1u);

    // anti-aligned pairs, class by class: (s XOR T_{-d}(s)) & classmask
    int c = 0;
    uint64_t m = 0;
    {
      const TorusClass cl = TP.cls[0];
      m = (s ^ rot_within(rot_rows(s, Lx * cl.rot_b, N, full), cl.rot_a, Lx, P.rot_hi, P.rot_lo)) & cl.classmask;
    }
    auto next = [&](int& gidx) -> bool {
      while (!m) {
        if (++c >= n_classes) return false;
        const TorusClass cl = TP.cls[c];
        m = (s ^ rot_within(rot_rows(s, Lx * cl.rot_b, N, full), cl.rot_a, Lx, P.rot_hi, P.rot_lo)) & cl.classmask;
      }
      const int x0 = ffs64(m);
      m &= m - 1;
      gidx = TP.gid[c][x0];
      return true;
    };

    Real accr = 0, acci = 0, anti = 0;
    int ga = 0, gb = 0;
    bool ha = next(ga);
    bool hb = ha && next(gb);
    // two targets at a time: their rank-record and v loads overlap
    while (ha) {
      const TG<Real>& A = G[ga];
      anti += A.fac;
      const Target<Real> TA = resolve<Real>(s, A, rw, nks, mstar, uniq, top, P, nk, rots);
      Target<Real> TB;
      TB.rep = ~0ull;
      if (hb) {
        const TG<Real>& Bg = G[gb];
        anti += Bg.fac;
        TB = resolve<Real>(s, Bg, rw, nks, mstar, uniq, top, P, nk, rots);
      }
      const int64_t ja = (TA.rep & ~full) ? -1 : vrank(TA.rep, vrecs, n_vrecs);
      const int64_t jb = (TB.rep & ~full) ? -1 : vrank(TB.rep, vrecs, n_vrecs);
      CT va, vb;
      va.x = va.y = vb.x = vb.y = Real(0);
      if (ja >= 0) va = v[ja];
      if (jb >= 0) vb = v[jb];
      if (ja >= 0) {
        const Real sc = nrm_inv[TA.stab];
        const Real pr = ph_re[TA.g] * sc, pi = ph_im[TA.g] * sc;
        const Real er = TA.cr * pr - TA.ci * pi, ei = TA.cr * pi + TA.ci * pr;
        accr += er * va.x - ei * va.y;
        acci += er * va.y + ei * va.x;
      }
      if (jb >= 0) {
        const Real sc = nrm_inv[TB.stab];
        const Real pr = ph_re[TB.g] * sc, pi = ph_im[TB.g] * sc;
        const Real er = TB.cr * pr - TB.ci * pi, ei = TB.cr * pi + TB.ci * pr;
        accr += er * vb.x - ei * vb.y;
        acci += er * vb.y + ei * vb.x;
      }
      ha = hb && next(ga);
      hb = ha && next(gb);
    }
    const Real ni = nrm[li];
    const Real ezz = total_fac - Real(2) * anti;
    CT out;
    out.x = accr * ni + ezz * vi.x;
    out.y = acci * ni + ezz * vi.y;
    w[i] = out;
  }
}

template <typename Real>
cudaError_t launch_t(const Sector& S, const void* v, void* w, cudaStream_t st) {
  using CT = typename C2<Real>::T;
  const size_t smem = sizeof(TG<Real>) * std::max(1, S.P.n_groups);
  auto kern = k_hv_torus<Real>;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
  if (per_sm < 1) per_sm = 1;
  const int64_t want = (S.P.n_p + kThreads - 1) / kThreads;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms * per_sm));
  kern<<<grid, kThreads, smem, st>>>(S.V, S.tplan, S.tgroups, reinterpret_cast<const CT*>(v), reinterpret_cast<CT*>(w));
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_hv_torus(const Sector& S, const void* v, void* w, bool fp64, cudaStream_t st) {
  return fp64 ? launch_t<double>(S, v, w, st) : launch_t<float>(S, v, w, st);
}

}  // namespace edg
