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

#include "hv_common.cuh"

namespace edg {

namespace {


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
  const size_t smem = hv_smem_bytes<Real>(S.P.n_groups, S.P.n_ch, kTorus, S.V.row_bits, S.V.n_chunks, S.V.n_perm);
  auto kern = k_hv<Real, kTorus, kChCh>;
  const int grid = persistent_grid(kern, smem, S.P.n_p);
  kern<<<grid, kHvThreads, smem, st>>>(S.V, reinterpret_cast<const CT*>(v), reinterpret_cast<CT*>(w));
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_hv(const Sector& S, const void* v, void* w, bool fp64, cudaStream_t st) {
  if (S.col) return launch_hv_stored(S, v, w, fp64, st);
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
  const size_t smem = hv_smem_bytes<float>(S.P.n_groups, S.P.n_ch, torus, S.V.row_bits, S.V.n_chunks, S.V.n_perm);
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
