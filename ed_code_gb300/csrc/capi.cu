// C ABI of the GPU sector (include/edgpu.h) and the host-side sector set-up.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/edgpu.h"
#include "edg_sector.cuh"

struct edg_sector {
  edg::Sector s;
};

namespace edg {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char* what) {
  return fail(EDG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// M_PI as the reference defines it (global.h:17).
constexpr double kPi = 3.14159265358979323846;

static void free_sector(Sector& S) {
  free_targets(S);
  void* ptrs[] = {S.dP,   S.reps,    S.lid,         S.recs,         S.vrecs,       S.Ia,    S.Ib,
                  S.groups, S.ch,   S.bows,    S.nk,          S.rots,         S.perms,       S.binom, S.host_in.ptr,
                  S.host_out.ptr, S.lz_work.ptr, S.ublk.ptr};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (S.stream) cudaStreamDestroy(S.stream);
  if (S.copy_stream) cudaStreamDestroy(S.copy_stream);
  for (cudaEvent_t ev : S.chunk_done)
    if (ev) cudaEventDestroy(ev);
  S = Sector{};
}

template <class T>
static cudaError_t upload(T** dst, const T* src, size_t n, size_t& bytes) {
  cudaError_t e = cudaMalloc(dst, sizeof(T) * std::max<size_t>(n, 1));
  if (e != cudaSuccess) return e;
  bytes += sizeof(T) * std::max<size_t>(n, 1);
  if (n) e = cudaMemcpy(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice);
  return e;
}

static bool is_perm(const int* T, int n) {
  std::vector<char> seen(n, 0);
  for (int i = 0; i < n; ++i) {
    if (T[i] < 0 || T[i] >= n || seen[T[i]]) return false;
    seen[T[i]] = 1;
  }
  return true;
}

// LxLy (Momentum_Basis.cpp:19-36): cycle length of site 0 under T1 and T2.
static void lxly(const std::vector<int>& T1, const std::vector<int>& T2, int& L1, int& L2) {
  L1 = 0;
  int s = 0;
  do { s = T1[s]; ++L1; } while (s != 0);
  L2 = 0;
  s = 0;
  do { s = T2[s]; ++L2; } while (s != 0);
}

static uint64_t binomial(int n, int k) {
  if (k < 0 || k > n) return 0;
  if (k > n - k) k = n - k;
  uint64_t r = 1;
  for (int i = 1; i <= k; ++i) r = r * (uint64_t)(n - k + i) / (uint64_t)i;
  return r;
}

static int create_sector(const edg_model* m, int n_ones, int kx, int ky, int kz, Sector& S) {
  if (!m || !m->T1 || !m->T2) return fail(EDG_ERR_INVALID, "model or T1/T2 missing");
  const int N = m->n_sites;
  if (N < 2 || N > kMaxSites) return fail(EDG_ERR_UNSUPPORTED, "n_sites must be in [2, 40]");
  if (N % 2) return fail(EDG_ERR_UNSUPPORTED, "odd n_sites: the reference's split_id/bits_right disagree for odd N");
  if (n_ones < 0 || n_ones > N) return fail(EDG_ERR_INVALID, "n_ones out of range");
  if (!is_perm(m->T1, N) || !is_perm(m->T2, N)) return fail(EDG_ERR_INVALID, "T1/T2 must be permutations of the sites");
  if (m->T3 && !is_perm(m->T3, N)) return fail(EDG_ERR_INVALID, "T3 must be a permutation of the sites");
  S.T1.assign(m->T1, m->T1 + N);
  S.T2.assign(m->T2, m->T2 + N);
  if (m->T3) S.T3.assign(m->T3, m->T3 + N);
  S.lambda = m->lambda;
  S.Ch = m->Ch;
  S.ChCh = m->ChCh;
  int L1, L2, L3 = 1;
  lxly(S.T1, S.T2, L1, L2);
  if (m->T3) {  // LxLyLz (Momentum_Basis.cpp:38-63): the cycle length of site 0
    L3 = 0;
    int s = 0;
    do { s = S.T3[s]; ++L3; } while (s != 0);
  }
  // Lanczos_sector.cpp:50-55 (2-D), :234-238 (3-D)
  if (kx >= L1 || ky >= L2 || kz >= L3 || kx < 0 || ky < 0 || kz < 0)
    return fail(EDG_ERR_MOMENTUM, "Invalid kx or ky");
  if (L1 * L2 * L3 > 64) return fail(EDG_ERR_UNSUPPORTED, "L1*L2*L3 > 64 translations");

  SectorParams& P = S.P;
  std::memset(&P, 0, sizeof(P));
  P.n_sites = N;
  P.n_ones = n_ones;
  P.half = N / 2;
  P.L1 = L1;
  P.L2 = L2;
  P.kx = kx;
  P.ky = ky;
  P.L3 = L3;
  P.kz = kz;
  P.full_mask = (N == 64) ? ~0ull : ((1ull << N) - 1ull);
  P.right_mask = (1ull << P.half) - 1ull;
  P.n_configs = (int64_t)binomial(N, n_ones);
  P.n_recs = (P.n_configs + kRecBits - 1) / kRecBits;
  P.ChCh = m->ChCh;

  // Row-major torus test: T1 = +x, T2 = +y with Lx = L1, Ly = L2 (2-D only).
  {
    const int Lx = L1, Ly = L2;
    bool t = !m->T3 && (Lx * Ly == N) && Lx >= 2 && Lx <= kMaxTorusRow && Ly <= 16;
    for (int s = 0; t && s < N; ++s) {
      const int x = s % Lx, y = s / Lx;
      if (S.T1[s] != (x + 1) % Lx + Lx * y) t = false;
      if (S.T2[s] != x + Lx * ((y + 1) % Ly)) t = false;
    }
    P.torus = t ? 1 : 0;
  }

  // Phases exp(-i(px*lx + py*ly [+ pz*lz])) for the translation (a, b, c)
  // from a state to its representative, lx = (L1-a)%L1, ly = (L2-b)%L2,
  // lz = (L3-c)%L3, with the reference's expressions (Momentum_Basis.cpp:
  // 747-753 and :861-872; px, py, pz as Lanczos_sector.cpp:57 and :240).
  const double px = 2 * kx * kPi / L1, py = 2 * ky * kPi / L2, pz = 2 * kz * kPi / L3;
  for (int c = 0; c < L3; ++c)
    for (int b = 0; b < L2; ++b)
      for (int a = 0; a < L1; ++a) {
        const int lx = (L1 - a) % L1, ly = (L2 - b) % L2, lz = (L3 - c) % L3;
        const std::complex<double> ph =
            m->T3 ? std::exp(std::complex<double>(0.0, -px * lx - py * ly - pz * lz))
                  : std::exp(std::complex<double>(0.0, -px * lx - py * ly));
        P.ph_re[a + L1 * b + L1 * L2 * c] = ph.real();
        P.ph_im[a + L1 * b + L1 * L2 * c] = ph.imag();
      }
  const int G = L1 * L2 * L3;
  for (int lid = 1; lid <= 64; ++lid) {
    const int64_t n = (int64_t)G / lid;  // integer division as Momentum_Basis.cpp:764, :883
    P.nrm[lid] = n > 0 ? std::sqrt((double)n) : 0.0;
    P.nrm_inv[lid] = n > 0 ? 1 / std::sqrt((double)n) : 0.0;
  }
  for (int k = 0; k < G; ++k) {
    P.chi_re[k] = std::cos(2 * kPi * k / G);
    P.chi_im[k] = -std::sin(2 * kPi * k / G);
  }
  for (int a = 0; a < kMaxTorusRow && P.torus; ++a) {
    uint64_t hi = 0, lo = 0;
    for (int s = 0; s < N; ++s) {
      const int x = s % L1;
      if (x >= a) hi |= 1ull << s;
      else lo |= 1ull << s;
    }
    P.rot_hi[a] = hi;
    P.rot_lo[a] = lo;
  }

  // Flip groups: every bond (|J| >= 1e-16, H_v.cpp:230-231) and chirality
  // entry (|Ch| > 1e-16, H_v.cpp:263) is filed under its unordered pair.
  std::vector<TermGroup> groups;
  std::vector<std::vector<ChTerm>> group_ch;
  std::map<std::pair<int, int>, int> gid;
  auto group_of = [&](int x, int y) -> int {
    const int a = std::min(x, y), b = std::max(x, y);
    auto it = gid.find({a, b});
    if (it != gid.end()) return it->second;
    TermGroup g;
    std::memset(&g, 0, sizeof g);
    g.mask = (1ull << a) | (1ull << b);
    g.a = a;
    g.b = b;
    groups.push_back(g);
    group_ch.emplace_back();
    gid[{a, b}] = (int)groups.size() - 1;
    return (int)groups.size() - 1;
  };
  double total_fac = 0.0;
  for (int k = 0; k < m->n_bonds; ++k) {
    const edg_bond& bd = m->bonds[k];
    if (bd.x < 0 || bd.x >= N || bd.y < 0 || bd.y >= N) return fail(EDG_ERR_INVALID, "bond site out of range");
    if (std::abs(bd.J) < 1e-16) continue;
    const double fac = 0.25 * m->lambda * bd.J;
    total_fac += fac;
    if (bd.x == bd.y) continue;  // never anti-aligned: diagonal only
    const int g = group_of(bd.x, bd.y);
    TermGroup& gr = groups[g];
    gr.fac += fac;
    const std::complex<double> e(bd.re, bd.im);
    for (int cs = 0; cs < 2; ++cs) {
      // cs = bit a of the state; bit x is cs when x == a, else 1 - cs
      const int tx = (bd.x == gr.a) ? cs : 1 - cs;
      const std::complex<double> c = (tx == 1 ? std::conj(e) : e) * bd.J * 0.5;
      gr.Bre[cs] += c.real();
      gr.Bim[cs] += c.imag();
    }
  }
  P.total_fac = total_fac;
  P.use_ch = std::abs(m->Ch) > 1e-16 ? 1 : 0;
  if (P.use_ch) {
    for (int k = 0; k < m->n_triangles; ++k) {
      const edg_triangle& t = m->triangles[k];
      if (t.i < 0 || t.i >= N || t.j < 0 || t.j >= N || t.k < 0 || t.k >= N)
        return fail(EDG_ERR_INVALID, "triangle site out of range");
      if (t.i == t.j) continue;
      const int g = group_of(t.i, t.j);
      const TermGroup& gr = groups[g];
      ChTerm c;
      std::memset(&c, 0, sizeof c);
      c.z = t.k;
      const std::complex<double> ep(t.re, t.im), I(0, 1);
      for (int cs = 0; cs < 2; ++cs) {
        const int ty = (t.j == gr.a) ? cs : 1 - cs;
        const std::complex<double> sgn = ty == 1 ? I * ep : -I * std::conj(ep);  // H_v.cpp:287-290
        const std::complex<double> A = m->Ch * 0.25 * sgn;
        c.Are[cs] = A.real();
        c.Aim[cs] = A.imag();
      }
      group_ch[g].push_back(c);
    }
  }
  std::vector<ChTerm> ch;
  for (size_t g = 0; g < groups.size(); ++g) {
    groups[g].ch_begin = (int)ch.size();
    for (const ChTerm& c : group_ch[g]) ch.push_back(c);
    groups[g].ch_end = (int)ch.size();
  }
  if ((int)groups.size() > kMaxGroups || (int)ch.size() > kMaxChTerms)
    return fail(EDG_ERR_UNSUPPORTED, "more than 512 flipped pairs or 1024 chirality terms");
  P.n_groups = (int)groups.size();
  P.n_ch = (int)ch.size();
  P.use_chch = (std::abs(m->ChCh) > 1e-16 && m->n_bowties > 0) ? 1 : 0;
  std::vector<Bowtie> bows;
  if (P.use_chch) {
    if (m->n_bowties > kMaxBowties) return fail(EDG_ERR_UNSUPPORTED, "more than 65536 bowties");
    for (int k = 0; k < m->n_bowties; ++k) {
      const edg_bowtie& b = m->bowties[k];
      const int v[6] = {b.x, b.y, b.z, b.p, b.q, b.r};
      for (int q = 0; q < 6; ++q)
        if (v[q] < 0 || v[q] >= N) return fail(EDG_ERR_INVALID, "bowtie site out of range");
      bows.push_back(Bowtie{b.x, b.y, b.z, b.p, b.q, b.r});
    }
  }
  P.n_bowties = (int)bows.size();

  // Lin tables (Lin_Tables.cpp:57-78; Ib as Momentum_Basis.cpp:731-737):
  // Ia = 1-based rank among half-words of equal popcount; Ib[l] = Lin index
  // of the first configuration with left half l, or -1 when there is none.
  const int h = P.half;
  const int64_t nh = (int64_t)1 << h;
  std::vector<uint32_t> Ia(nh);
  std::vector<int64_t> Ib(nh, -1);
  {
    std::vector<int64_t> next_rank(h + 2, 1);
    for (int64_t w = 0; w < nh; ++w) Ia[w] = (uint32_t)next_rank[__builtin_popcountll(w)]++;
    int64_t lin = 0;
    for (int64_t l = 0; l < nh; ++l) {
      const int q = n_ones - __builtin_popcountll(l);
      if (q < 0 || q > h) continue;
      Ib[l] = lin;
      lin += (int64_t)binomial(h, q);
    }
    if (lin != P.n_configs) return fail(EDG_ERR_INVALID, "Lin table size mismatch");
  }
  std::vector<uint64_t> binom((kMaxSites + 1) * (kMaxSites + 1));
  for (int n = 0; n <= kMaxSites; ++n)
    for (int k = 0; k <= kMaxSites; ++k) binom[n * (kMaxSites + 1) + k] = binomial(n, k);
  // Orbit-search tables: row rotation minima (torus) and 8-bit permutation
  // chunks for T1, T2 (the reference's walk).
  int row_bits = P.torus ? L1 : 0;
  std::vector<uint8_t> nk(1u << row_bits);
  std::vector<uint16_t> rots(1u << row_bits);
  if (P.torus) {
    const int Lx = L1;
    const uint32_t rm = (1u << Lx) - 1u;
    for (uint32_t r = 0; r <= rm; ++r) {
      uint32_t best = r, set = 0;
      for (int a = 0; a < Lx; ++a) {
        const uint32_t v = a ? (((r << a) | (r >> (Lx - a))) & rm) : r;
        if (v < best) { best = v; set = 0; }
        if (v == best) set |= 1u << a;
      }
      nk[r] = (uint8_t)best;
      rots[r] = (uint16_t)set;
    }
  }
  const int n_chunks = (N + 7) / 8;
  const int n_perm = m->T3 ? 3 : 2;
  std::vector<uint64_t> perms((size_t)n_perm * n_chunks * 256, 0);
  for (int which = 0; which < n_perm; ++which) {
    const std::vector<int>& T = which == 0 ? S.T1 : (which == 1 ? S.T2 : S.T3);
    for (int c = 0; c < n_chunks; ++c)
      for (int byte = 0; byte < 256; ++byte) {
        uint64_t out = 0;
        for (int k = 0; k < 8; ++k) {
          const int site = 8 * c + k;
          if (site < N && ((byte >> k) & 1)) out |= 1ull << T[site];
        }
        perms[(which * n_chunks + c) * 256 + byte] = out;
      }
  }

  // Device memory: rank records dominate (16 B per 96 configurations).
  {
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const double need = (double)P.n_recs * 16 + (double)P.n_recs * 4 + (double)P.n_configs / 30.0 * 9.0;
    if (need > 0.95 * (double)free_b) return fail(EDG_ERR_NOMEM, "sector needs more device memory than is free");
  }
  cudaError_t e = cudaStreamCreateWithFlags(&S.stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_fail(e, "stream");
  size_t bytes = 0;
  if ((e = upload(&S.Ia, Ia.data(), Ia.size(), bytes)) != cudaSuccess) return cuda_fail(e, "Ia");
  if ((e = upload(&S.Ib, Ib.data(), Ib.size(), bytes)) != cudaSuccess) return cuda_fail(e, "Ib");
  if ((e = upload(&S.groups, groups.data(), groups.size(), bytes)) != cudaSuccess) return cuda_fail(e, "groups");
  if ((e = upload(&S.ch, ch.data(), ch.size(), bytes)) != cudaSuccess) return cuda_fail(e, "ch");
  if ((e = upload(&S.bows, bows.data(), bows.size(), bytes)) != cudaSuccess) return cuda_fail(e, "bowties");
  if ((e = upload(&S.nk, nk.data(), nk.size(), bytes)) != cudaSuccess) return cuda_fail(e, "nk");
  if ((e = upload(&S.rots, rots.data(), rots.size(), bytes)) != cudaSuccess) return cuda_fail(e, "rots");
  if ((e = upload(&S.perms, perms.data(), perms.size(), bytes)) != cudaSuccess) return cuda_fail(e, "perms");
  if ((e = upload(&S.binom, binom.data(), binom.size(), bytes)) != cudaSuccess) return cuda_fail(e, "binom");
  e = cudaMalloc(&S.recs, sizeof(RankRec) * std::max<int64_t>(1, P.n_recs));
  if (e != cudaSuccess) return fail(EDG_ERR_NOMEM, "rank records: out of device memory");
  bytes += sizeof(RankRec) * std::max<int64_t>(1, P.n_recs);
  if ((e = upload(&S.dP, &P, 1, bytes)) != cudaSuccess) return cuda_fail(e, "params");
  S.device_bytes = bytes;

  SectorView& V = S.V;
  V.params = S.dP;
  V.recs = S.recs;
  V.Ia = S.Ia;
  V.Ib = S.Ib;
  V.groups = S.groups;
  V.ch = S.ch;
  V.bows = S.bows;
  V.nk = S.nk;
  V.rots = S.rots;
  V.perms = S.perms;
  V.binom = S.binom;
  V.n_chunks = n_chunks;
  V.n_perm = n_perm;
  V.row_bits = row_bits;

  std::string err;
  e = build_basis(S, err);
  if (e != cudaSuccess) return fail(e == cudaErrorMemoryAllocation ? EDG_ERR_NOMEM : EDG_ERR_CUDA, err);
  V.reps = S.reps;
  V.lid = S.lid;
  // n_p is now known: refresh the device copy of the parameters.
  e = cudaMemcpy(S.dP, &P, sizeof(P), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "params");
  if (P.n_p == 0) return fail(EDG_ERR_EMPTY, "No states in psector");
  if (P.n_p >= (int64_t)0xFFFFFFFFll) return fail(EDG_ERR_UNSUPPORTED, "sector dimension exceeds 2^32-1");
  return EDG_OK;
}

// splitmix64 test vectors: entry i takes counters 2i (re) and 2i+1 (im).
__global__ void k_fill_random(void* dst, int64_t n, int dtype, uint64_t seed) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < 2 * n; i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t z = seed * 0x9E3779B97F4A7C15ull + (uint64_t)(i + 1) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z = z ^ (z >> 31);
    const double u = 2.0 * ((double)(z >> 11) * (1.0 / 9007199254740992.0)) - 1.0;
    if (dtype == EDG_C128) static_cast<double*>(dst)[i] = u;
    else static_cast<float*>(dst)[i] = (float)u;
  }
}

}  // namespace edg

using namespace edg;

extern "C" {

const char* edg_last_error(void) { return g_last_error.c_str(); }
int edg_abi_version(void) { return EDGPU_ABI_VERSION; }

int edg_sector_create3(const edg_model* model, int n_ones, int kx, int ky, int kz, edg_sector** out) {
  if (!out) return fail(EDG_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (!model || !model->T1 || !model->T2) return fail(EDG_ERR_INVALID, "model or T1/T2 missing");
  edg_sector* h = new edg_sector();
  cudaGetDevice(&h->s.device);
  int rc = create_sector(model, n_ones, kx, ky, kz, h->s);
  if (rc != EDG_OK) {
    free_sector(h->s);
    delete h;
    return rc;
  }
  *out = h;
  return EDG_OK;
}

int edg_sector_create(const edg_model* model, int n_ones, int kx, int ky, edg_sector** out) {
  if (model && model->T3) return fail(EDG_ERR_INVALID, "a model with T3 needs edg_sector_create3 (kz)");
  return edg_sector_create3(model, n_ones, kx, ky, 0, out);
}

int edg_sector_destroy(edg_sector* s) {
  if (!s) return EDG_OK;
  free_sector(s->s);
  delete s;
  return EDG_OK;
}

int edg_sector_get_info(const edg_sector* s, edg_sector_info* info) {
  if (!s || !info) return fail(EDG_ERR_INVALID, "NULL argument");
  const SectorParams& P = s->s.P;
  info->n_sites = P.n_sites;
  info->n_ones = P.n_ones;
  info->L1 = P.L1;
  info->L2 = P.L2;
  info->kx = P.kx;
  info->ky = P.ky;
  info->L3 = P.L3;
  info->kz = P.kz;
  info->torus = P.torus;
  info->n_groups = P.n_groups;
  info->n_p = P.n_p;
  info->n_configs = P.n_configs;
  info->device_bytes = (int64_t)s->s.device_bytes;
  info->n_targets = P.n_targets;
  info->lanes_per_row = s->s.col ? s->s.csr_lpr : 0;
  info->cache_policy = s->s.col ? s->s.csr_pol : 0;
  info->ctas_per_sm = s->s.col ? s->s.csr_cps : 0;
  info->pipelined = s->s.col ? s->s.csr_pipe : 0;
  info->entry_bytes = s->s.col ? (s->s.pack_cb ? 4 : 6) : 0;
  info->n_values = s->s.n_vals;
  return EDG_OK;
}

int edg_sector_copy_basis(const edg_sector* s, int64_t* states, double* norm, double* norm_inv) {
  if (!s) return fail(EDG_ERR_INVALID, "NULL sector");
  const Sector& S = s->s;
  const int64_t n = S.P.n_p;
  cudaError_t e;
  if (states) {
    e = cudaMemcpy(states, S.reps, sizeof(int64_t) * n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "copy states");
  }
  if (norm || norm_inv) {
    std::vector<uint8_t> lid(n);
    e = cudaMemcpy(lid.data(), S.lid, n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "copy lid");
    for (int64_t i = 0; i < n; ++i) {
      if (norm) norm[i] = S.P.nrm[lid[i]];
      if (norm_inv) norm_inv[i] = S.P.nrm_inv[lid[i]];
    }
  }
  return EDG_OK;
}

int edg_sector_copy_lin_tables(const edg_sector* s, int64_t* Ia, int64_t* Ib, int64_t* bits_right) {
  if (!s) return fail(EDG_ERR_INVALID, "NULL sector");
  const Sector& S = s->s;
  const int64_t nh = (int64_t)1 << S.P.half;
  cudaError_t e;
  if (Ia) {
    std::vector<uint32_t> tmp(nh);
    e = cudaMemcpy(tmp.data(), S.Ia, sizeof(uint32_t) * nh, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "copy Ia");
    for (int64_t i = 0; i < nh; ++i) Ia[i] = tmp[i];
  }
  if (Ib) {
    e = cudaMemcpy(Ib, S.Ib, sizeof(int64_t) * nh, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "copy Ib");
  }
  if (bits_right) *bits_right = (int64_t)S.P.right_mask;
  return EDG_OK;
}

int edg_sector_copy_config_tables(const edg_sector* s, int64_t max_configs, int64_t* rep_loc, double* state_ph,
                                  int32_t* lxly) {
  if (!s) return fail(EDG_ERR_INVALID, "NULL sector");
  const Sector& S = s->s;
  const int64_t nc = S.P.n_configs;
  if (nc > max_configs) return fail(EDG_ERR_INVALID, "sector has more configurations than max_configs");
  int64_t* d_loc = nullptr;
  int32_t* d_g = nullptr;
  cudaError_t e = cudaMalloc(&d_loc, sizeof(int64_t) * nc);
  if (e == cudaSuccess) e = cudaMalloc(&d_g, sizeof(int32_t) * nc);
  if (e != cudaSuccess) {
    cudaFree(d_loc);
    return cuda_fail(e, "config tables");
  }
  e = export_walk_tables(S, d_loc, d_g, S.stream);
  std::vector<int32_t> g(nc);
  if (e == cudaSuccess) e = cudaStreamSynchronize(S.stream);
  if (e == cudaSuccess && rep_loc) e = cudaMemcpy(rep_loc, d_loc, sizeof(int64_t) * nc, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(g.data(), d_g, sizeof(int32_t) * nc, cudaMemcpyDeviceToHost);
  cudaFree(d_loc);
  cudaFree(d_g);
  if (e != cudaSuccess) return cuda_fail(e, "config tables");
  const int L1 = S.P.L1, L2 = S.P.L2;
  for (int64_t i = 0; i < nc; ++i) {
    const int a = g[i] % L1, b = (g[i] / L1) % L2;
    if (state_ph) {
      state_ph[2 * i] = S.P.ph_re[g[i]];
      state_ph[2 * i + 1] = S.P.ph_im[g[i]];
    }
    if (lxly) {
      lxly[2 * i] = (L1 - a) % L1;
      lxly[2 * i + 1] = (L2 - b) % L2;
    }
  }
  return EDG_OK;
}

int edg_hv(edg_sector* s, const void* v, void* w, int dtype, void* stream) {
  if (!s || !v || !w) return fail(EDG_ERR_INVALID, "NULL argument");
  if (dtype != EDG_C128 && dtype != EDG_C64) return fail(EDG_ERR_INVALID, "dtype must be EDG_C128 or EDG_C64");
  if (v == w) return fail(EDG_ERR_INVALID, "v and w must not alias");
  cudaError_t e = launch_hv(s->s, v, w, dtype == EDG_C128, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "hv launch");
  return EDG_OK;
}

static cudaError_t ensure(DeviceBuffer& b, size_t bytes) {
  if (b.bytes >= bytes) return cudaSuccess;
  if (b.ptr) cudaFree(b.ptr);
  b.ptr = nullptr;
  b.bytes = 0;
  cudaError_t e = cudaMalloc(&b.ptr, bytes);
  if (e == cudaSuccess) b.bytes = bytes;
  return e;
}

int edg_hv_host(edg_sector* s, const void* v, void* w, int dtype) {
  if (!s || !v || !w) return fail(EDG_ERR_INVALID, "NULL argument");
  if (dtype != EDG_C128 && dtype != EDG_C64) return fail(EDG_ERR_INVALID, "dtype must be EDG_C128 or EDG_C64");
  Sector& S = s->s;
  const size_t bytes = (size_t)S.P.n_p * (dtype == EDG_C128 ? 16 : 8);
  cudaError_t e = ensure(S.host_in, bytes);
  if (e == cudaSuccess) e = ensure(S.host_out, bytes);
  if (e != cudaSuccess) return cuda_fail(e, "hv_host buffers");
  const bool fp64 = dtype == EDG_C128;
  const int64_t n = S.P.n_p;
  constexpr int kChunks = 8;
  // v in page-locked host memory that the device can address: with stored
  // rows, one kernel reads it in place and writes both the device copy of v
  // and u = v / norm, instead of a copy-engine copy and then the u pass
  cudaPointerAttributes va{};
  const void* v_dev = nullptr;
  if (cudaPointerGetAttributes(&va, v) != cudaSuccess)
    cudaGetLastError();
  else if (va.type == cudaMemoryTypeHost && va.devicePointer &&
           reinterpret_cast<uintptr_t>(va.devicePointer) % (fp64 ? 16 : 8) == 0)
    v_dev = va.devicePointer;
  const bool u_done = S.col && v_dev;
  e = u_done ? launch_u_in(S, v_dev, S.host_in.ptr, fp64, S.stream)
             : cudaMemcpyAsync(S.host_in.ptr, v, bytes, cudaMemcpyHostToDevice, S.stream);
  // w in page-locked host memory that the device can address (cudaHostAlloc,
  // cudaHostRegister): the kernel stores each w_i there itself, over the
  // host link while it runs, with no copy after it.
  cudaPointerAttributes wa{};
  void* w_dev = nullptr;
  if (cudaPointerGetAttributes(&wa, w) != cudaSuccess)
    cudaGetLastError();  // clear the failed query; w is then copied back
  else if (wa.type == cudaMemoryTypeHost)
    w_dev = wa.devicePointer;
  if (e == cudaSuccess && w_dev) {
    e = u_done ? launch_hv_rows(S, S.host_in.ptr, w_dev, fp64, 0, n, false, S.stream)
               : launch_hv(S, S.host_in.ptr, w_dev, fp64, S.stream);
  } else if (S.col && n >= (1 << 20)) {
    // rows in row order: the w rows of chunk c go back to the host while the
    // rows of chunk c + 1 are computed
    if (!S.copy_stream && e == cudaSuccess) e = cudaStreamCreateWithFlags(&S.copy_stream, cudaStreamNonBlocking);
    for (int c = 0; c < kChunks && e == cudaSuccess; ++c)
      if (!S.chunk_done[c]) e = cudaEventCreateWithFlags(&S.chunk_done[c], cudaEventDisableTiming);
    const size_t elem = fp64 ? 16 : 8;
    for (int c = 0; c < kChunks && e == cudaSuccess; ++c) {
      const int64_t r0 = n * c / kChunks, r1 = n * (c + 1) / kChunks;
      e = launch_hv_rows(S, S.host_in.ptr, S.host_out.ptr, fp64, r0, r1, c == 0 && !u_done, S.stream);
      if (e == cudaSuccess) e = cudaEventRecord(S.chunk_done[c], S.stream);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(S.copy_stream, S.chunk_done[c], 0);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(static_cast<char*>(w) + r0 * elem, static_cast<char*>(S.host_out.ptr) + r0 * elem,
                            (size_t)(r1 - r0) * elem, cudaMemcpyDeviceToHost, S.copy_stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(S.copy_stream);
  } else {
    if (e == cudaSuccess)
      e = u_done ? launch_hv_rows(S, S.host_in.ptr, S.host_out.ptr, fp64, 0, n, false, S.stream)
                 : launch_hv(S, S.host_in.ptr, S.host_out.ptr, fp64, S.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(w, S.host_out.ptr, bytes, cudaMemcpyDeviceToHost, S.stream);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(S.stream);
  if (e != cudaSuccess) return cuda_fail(e, "hv_host");
  return EDG_OK;
}

int edg_solve_plain(edg_sector* s, const edg_solver_opts* opts, double* eigs, int64_t eigs_capacity,
                    int64_t* n_eigs, double* evecs, int64_t evecs_capacity, edg_solver_stats* stats) {
  if (!s || !opts || !eigs || !n_eigs) return fail(EDG_ERR_INVALID, "NULL argument");
  *n_eigs = 0;
  return solve_plain(s->s, *opts, eigs, eigs_capacity, n_eigs, evecs, evecs_capacity, stats);
}

int edg_solve_mixed(edg_sector* s, const edg_mixed_opts* opts, double* eigs, double* ritz, double* residuals,
                    int64_t* n_eigs, double* evecs, edg_mixed_stats* stats) {
  if (!s || !opts || !eigs || !n_eigs) return fail(EDG_ERR_INVALID, "NULL argument");
  if (opts->iterations > 2000) return fail(EDG_ERR_UNSUPPORTED, "at most 2000 iterations");
  *n_eigs = 0;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  return solve_mixed(s->s, *opts, eigs, ritz, residuals, n_eigs, opts->want_vectors ? evecs : nullptr, stats);
}

int edg_sector_build_targets(edg_sector* s, int64_t max_bytes) {
  if (!s) return fail(EDG_ERR_INVALID, "NULL sector");
  std::string err;
  const int rc = build_targets(s->s, max_bytes > 0 ? max_bytes : INT64_MAX, err);
  if (rc != EDG_OK) return fail(rc, err);
  return EDG_OK;
}

int edg_sector_free_targets(edg_sector* s) {
  if (!s) return fail(EDG_ERR_INVALID, "NULL sector");
  free_targets(s->s);
  cudaMemcpy(s->s.dP, &s->s.P, sizeof(SectorParams), cudaMemcpyHostToDevice);
  return EDG_OK;
}

int edg_sector_tune(edg_sector* s, int lanes_per_row, int* chosen, double* ms) {
  if (!s) return fail(EDG_ERR_INVALID, "NULL sector");
  const int rc = tune_rows(s->s, lanes_per_row, chosen, ms);
  if (rc != EDG_OK) return fail(rc, "tuning the stored-row kernel failed");
  return EDG_OK;
}

int edg_sector_set_rows(edg_sector* s, int lanes_per_row, int cache_policy, int ctas_per_sm, int pipelined) {
  if (!s) return fail(EDG_ERR_INVALID, "NULL sector");
  if (lanes_per_row != 8 && lanes_per_row != 16 && lanes_per_row != 32)
    return fail(EDG_ERR_INVALID, "lanes_per_row must be 8, 16 or 32");
  if (cache_policy != 1 && cache_policy != 2) return fail(EDG_ERR_INVALID, "cache_policy must be 1 or 2");
  if (ctas_per_sm < 0 || ctas_per_sm > 32) return fail(EDG_ERR_INVALID, "ctas_per_sm must be 0 to 32");
  if (pipelined != 0 && pipelined != 1) return fail(EDG_ERR_INVALID, "pipelined must be 0 or 1");
  s->s.csr_lpr = lanes_per_row;
  s->s.csr_pol = cache_policy;
  s->s.csr_cps = ctas_per_sm;
  s->s.csr_pipe = pipelined;
  return EDG_OK;
}

int edg_count_offdiag(edg_sector* s, int64_t* nnz_off) {
  if (!s || !nnz_off) return fail(EDG_ERR_INVALID, "NULL argument");
  Sector& S = s->s;
  unsigned long long* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(unsigned long long));
  if (e != cudaSuccess) return cuda_fail(e, "count_offdiag");
  e = count_offdiag(S, d, S.stream);
  unsigned long long h = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, S.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(S.stream);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(e, "count_offdiag");
  *nnz_off = (int64_t)h;
  return EDG_OK;
}

int edg_fill_random(void* dst, int64_t n, int dtype, uint64_t seed, void* stream) {
  if (!dst || n < 0) return fail(EDG_ERR_INVALID, "bad argument");
  if (dtype != EDG_C128 && dtype != EDG_C64) return fail(EDG_ERR_INVALID, "dtype must be EDG_C128 or EDG_C64");
  const int64_t work = 2 * n;
  const int blocks = (int)std::min<int64_t>(std::max<int64_t>(1, (work + 255) / 256), 152 * 32);
  k_fill_random<<<blocks, 256, 0, (cudaStream_t)stream>>>(dst, n, dtype, seed);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "fill_random");
  return EDG_OK;
}

}  // extern "C"
