// Core integer and term logic of the momentum-sector H*v, shared by the
// basis-construction and H*v kernels.
//
// Reference path (hiteshjc/ED_Code, src/):
//   translateT / LxLy ............ Momentum_Basis.cpp:4-36
//   representative_p ............. Momentum_Basis.cpp:472-543 (2-D), :545-643 (3-D)
//   Lin_Tables / split_id ........ Lin_Tables.cpp:42-78, Momentum_Basis.cpp:731-737
//   sHv row formula .............. H_v.cpp:218-355
//
// Layout of one sector in HBM (all device arrays, owned by the sector):
//   reps[n_p]      u64   representatives in increasing order (pblock_states)
//   lid[n_p]       u8    stabiliser count of each representative; the norms
//                        sqrt(L1*L2/lid) come from a 65-entry table
//   vrecs[n_vrec]  16 B  {u32 base, u32 bits[3]}: one record per 96 consecutive
//                        values 0..max_rep; bit set <=> that value is an
//                        allowed representative; base = allowed ones before it.
//                        j(rep) = base + popcount of the bits below it.
//                        (While the basis is built the same records are indexed
//                        by Lin index over the C(N, n_up) configurations.)
//   Ia[2^h], Ib[2^h]     Lin tables (Ia as u32, Ib as i64), Lin = Ia[r] + Ib[l] - 1
//
// The representative of a flipped state is found on the fly, so no per-
// configuration table (the reference's rep_loc/state_ph, 24 B per
// configuration) is needed.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define EDG_HD __host__ __device__ __forceinline__
#else
#define EDG_HD inline
#endif

namespace edg {

constexpr int kMaxSites = 40;      // Lin tables hold 2^(N/2) entries
constexpr int kMaxGroups = 512;    // distinct flipped pairs
constexpr int kMaxChTerms = 1024;  // chirality terms
constexpr int kMaxBowties = 65536;
constexpr int kRecBits = 96;       // Lin indices per rank record
constexpr int kMaxTorusRow = 10;   // row-rotation search tables hold 2^Lx entries

EDG_HD int popc64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __popcll(x);
#else
  return __builtin_popcountll(x);
#endif
}
EDG_HD int popc32(uint32_t x) {
#if defined(__CUDA_ARCH__)
  return __popc(x);
#else
  return __builtin_popcount(x);
#endif
}
EDG_HD int ffs64(uint64_t x) {  // index of lowest set bit, x != 0
#if defined(__CUDA_ARCH__)
  return __ffsll((long long)x) - 1;
#else
  return __builtin_ctzll(x);
#endif
}

struct alignas(16) RankRec {
  uint32_t base;
  uint32_t bits[3];
};

// All terms whose off-diagonal part flips the same pair {a, b} (a < b).  For a
// state s with s_a != s_b the coefficient is
//   c(s) = B[s_a] + sum_{ch terms m} (s_{z_m} ? +A_m[s_a] : -A_m[s_a])
// where B collects the bond terms  J/2 * (s_x ? conj(e) : e)  (H_v.cpp:232-255)
// and A the chirality terms  Ch/4 * (s_y ? i*ep : -i*conj(ep))  (H_v.cpp:263-303).
struct TermGroup {
  uint64_t mask;
  int a, b;
  int ch_begin, ch_end;
  double fac;           // sum over bonds of 0.25*lambda*J (diagonal part)
  double Bre[2], Bim[2];
};
struct ChTerm {
  int z;
  int pad;
  double Are[2], Aim[2];
};
struct Bowtie {  // ChCh term, H_v.cpp:305-353
  int x, y, z, p, q, r;
};

// Everything a kernel needs to know about one sector, in one POD block that
// lives in device memory and is staged into shared memory per CTA.
struct SectorParams {
  int n_sites, n_ones, half;        // half = N/2 (even N only)
  int L1, L2;
  int kx, ky;
  int L3, kz;                       // third translation of a 3-D torus (L3 = 1, kz = 0 in 2-D)
  int torus;                        // 1: row-major torus T1=+x, T2=+y (Lx=L1, Ly=L2)
  int n_groups, n_ch, n_bowties;
  int use_ch, use_chch;
  int pad0, pad1;
  int64_t n_p, n_configs, n_recs;   // n_recs: Lin-indexed records used while building
  int64_t n_vrecs;                  // value-indexed rank records (see value_rank)
  uint64_t full_mask, right_mask;
  double total_fac;                 // sum over bonds of 0.25*lambda*J
  double ChCh;
  // Phase for translation g = a + L1 b + L1 L2 c (T1^a T2^b T3^c) from a
  // state to its representative: exp(-i(px*lx + py*ly + pz*lz)),
  // lx=(L1-a)%L1, ly=(L2-b)%L2, lz=(L3-c)%L3, evaluated on the host with the
  // reference's expression (Momentum_Basis.cpp:753, :872).
  double ph_re[64], ph_im[64];
  // Norm tables by stabiliser count: sqrt(G/lid) and its inverse, G = L1 L2 L3,
  // with the reference's integer division (Momentum_Basis.cpp:764-766, :883).
  double nrm[65], nrm_inv[65];
  // e^{-2 pi i m/G}: character values for the p_id test.
  double chi_re[64], chi_im[64];
  // Torus search tables (row length Lx = L1, Ly = L2 rows).
  uint64_t rot_hi[kMaxTorusRow], rot_lo[kMaxTorusRow];  // per-row masks of bits x >= a / x < a
  // Stored targets (targets.cu): phase class of each translation g, number
  // of classes, value-table offset of each group, number of stored targets.
  uint8_t g2cls[64];
  int n_cls, pad2;
  int64_t n_targets;
};

// --------------------------------------------------------------------------
// Lin index and representative position
// --------------------------------------------------------------------------
EDG_HD int64_t lin_index(uint64_t s, int half, uint64_t right_mask, const uint32_t* Ia, const int64_t* Ib) {
  return (int64_t)Ia[s & right_mask] + Ib[s >> half] - 1;
}

// Record holding Lin index `lin` and the bit inside it.  lin < 2^37 for
// N <= 40, so lin/96 = (lin>>5)/3 runs in 32-bit arithmetic.
EDG_HD uint32_t rec_of(int64_t lin, int* bit) {
  const uint32_t q = (uint32_t)((uint64_t)lin >> 5) / 3u;
  *bit = (int)(lin - (int64_t)q * kRecBits);
  return q;
}

// Position of representative `rep` among the allowed representatives, -1 if
// it is not one (the reference's rep_loc[...] < 0 case).
EDG_HD int64_t rank_lookup_bit(int bit, const RankRec& rec) {
  int w = bit >> 5, o = bit & 31;
  uint32_t word = rec.bits[w];
  if (!((word >> o) & 1u)) return -1;
  int below = popc32(word & ((1u << o) - 1u));
  if (w > 0) below += popc32(rec.bits[0]);
  if (w > 1) below += popc32(rec.bits[1]);
  return (int64_t)rec.base + below;
}
// Position of representative `rep` by its value: records cover the values
// 0..max_rep in blocks of 96 (representatives are orbit minima, so max_rep is
// far below 2^N and the table is about as small as a Lin-indexed one), and
// the lookup needs no Lin index.  -1 when rep is not an allowed state.
EDG_HD uint32_t vrec_of(uint64_t rep, int* bit) {
  uint64_t q;
  if ((rep >> 37) == 0) q = (uint32_t)(rep >> 5) / 3u;  // 32-bit division for rep < 2^37
  else q = (rep >> 5) / 3u;
  *bit = (int)(rep - q * kRecBits);
  return (uint32_t)q;
}
EDG_HD int64_t rank_lookup(int64_t lin, const RankRec& rec) {
  int bit = (int)(lin % kRecBits);
  int w = bit >> 5, o = bit & 31;
  uint32_t word = rec.bits[w];
  if (!((word >> o) & 1u)) return -1;
  int below = popc32(word & ((1u << o) - 1u));
  if (w > 0) below += popc32(rec.bits[0]);
  if (w > 1) below += popc32(rec.bits[1]);
  return (int64_t)rec.base + below;
}

// --------------------------------------------------------------------------
// Orbit search
// --------------------------------------------------------------------------
struct Orbit {
  uint64_t rep;  // smallest translate
  int g;         // translation index a + L1*b + L1*L2*c with rep = T1^a T2^b T3^c t
  int stab;      // number of translations mapping t to itself
};

// Apply a site permutation with 8-bit chunk tables: perm[c*256 + byte].
EDG_HD uint64_t apply_perm(uint64_t t, const uint64_t* perm, int n_chunks) {
  uint64_t out = 0;
  for (int c = 0; c < n_chunks; ++c) out |= perm[c * 256 + ((t >> (8 * c)) & 0xFFu)];
  return out;
}

// The reference's literal walk (Momentum_Basis.cpp:493-535, 3-D :566-634):
// for x < L1 { if x>0 apply T1; for y < L2 { if y>0 apply T2; for z < L3
// { if z>0 apply T3 } } }, first strict minimum wins.  Works for any
// T1/T2/T3; with L3 = 1 (2-D) the z loop applies nothing.  tx, ty, tz are
// the walk's step counts at the minimum, reduced mod L1/L2/L3 into g.
// chi_sum (optional) accumulates the p_id phase sum over walk positions
// equal to t.
EDG_HD Orbit orbit_walk(uint64_t t, const SectorParams& P, const uint64_t* perm1, const uint64_t* perm2,
                        const uint64_t* perm3, int n_chunks, double* chi_re_sum = nullptr,
                        double* chi_im_sum = nullptr) {
  Orbit o{t, 0, 1};
  uint64_t tmp = t;
  int tx = 0, ty = 0, tz = 0;
  const int G = P.L1 * P.L2 * P.L3;
  double cr = 1.0, ci = 0.0;
  for (int x = 0; x < P.L1; ++x) {
    for (int y = 0; y < P.L2; ++y) {
      for (int z = 0; z < P.L3; ++z) {
        if (x == 0 && y == 0 && z == 0) continue;
        if (z > 0) {
          tmp = apply_perm(tmp, perm3, n_chunks);
          ++tz;
        } else if (y > 0) {
          tmp = apply_perm(tmp, perm2, n_chunks);
          ++ty;
        } else {
          tmp = apply_perm(tmp, perm1, n_chunks);
          ++tx;
        }
        if (tmp == t) {
          ++o.stab;
          int m = (int)(((int64_t)P.kx * tx * P.L2 * P.L3 + (int64_t)P.ky * ty * P.L1 * P.L3 +
                         (int64_t)P.kz * tz * P.L1 * P.L2) % G);
          cr += P.chi_re[m];
          ci += P.chi_im[m];
        }
        if (tmp < o.rep) {
          o.rep = tmp;
          o.g = (tx % P.L1) + P.L1 * (ty % P.L2) + P.L1 * P.L2 * (tz % P.L3);
        }
      }
    }
  }
  if (chi_re_sum) { *chi_re_sum = cr; *chi_im_sum = ci; }
  return o;
}

// Early-exit test used by the basis build: is t smaller than every other
// translate (ties allowed)?  Any order of translates works.
EDG_HD bool walk_is_min(uint64_t t, const SectorParams& P, const uint64_t* perm1, const uint64_t* perm2,
                        const uint64_t* perm3, int n_chunks) {
  uint64_t row = t;
  for (int x = 0; x < P.L1; ++x) {
    uint64_t col = row;
    for (int y = 0; y < P.L2; ++y) {
      if (y > 0) {
        col = apply_perm(col, perm2, n_chunks);
        if (col < t) return false;
      }
      uint64_t tmp = col;
      for (int z = 1; z < P.L3; ++z) {
        tmp = apply_perm(tmp, perm3, n_chunks);
        if (tmp < t) return false;
      }
    }
    row = apply_perm(row, perm1, n_chunks);
    if (x + 1 < P.L1 && row < t) return false;
  }
  return true;
}

// Row-major torus, T1 = +x, T2 = +y, s = x + Lx*y, row y occupies bits
// [Lx*y, Lx*y+Lx).  The translate by (a, b) puts original row (r-b) mod Ly,
// rotated left by a, in row r.  The most significant row of the result is
// original row Ly-1-b rotated by a, so the minimum must put a row whose
// rotation minimum (necklace value, nk[]) is smallest on top, rotated to
// that minimum (rotations in rots[]).  Only those candidates are evaluated.
EDG_HD uint64_t torus_rotate_rows(uint64_t t, int shift, int N, uint64_t full_mask) {
  // rotate the N-bit word left by `shift` bits (0 <= shift < N)
  if (shift == 0) return t;
  return ((t << shift) | (t >> (N - shift))) & full_mask;
}
EDG_HD uint64_t torus_rotate_within(uint64_t u, int a, int Lx, const SectorParams& P) {
  if (a == 0) return u;
  return ((u << a) & P.rot_hi[a]) | ((u >> (Lx - a)) & P.rot_lo[a]);
}

EDG_HD Orbit orbit_torus(uint64_t t, const SectorParams& P, const uint8_t* nk, const uint16_t* rots) {
  const int Lx = P.L1, Ly = P.L2, N = P.n_sites;
  const uint64_t rmask = (1ull << Lx) - 1ull;
  int mstar = 1 << 30;
  uint32_t cand = 0;  // rows whose rotation minimum equals mstar
  for (int y = 0; y < Ly; ++y) {
    int v = nk[(int)((t >> (Lx * y)) & rmask)];
    if (v < mstar) { mstar = v; cand = 1u << y; }
    else if (v == mstar) cand |= 1u << y;
  }
  Orbit o{~0ull, 0, 0};
  while (cand) {
    int y = ffs64(cand);
    cand &= cand - 1;
    int r = (int)((t >> (Lx * y)) & rmask);
    int b = Ly - 1 - y;
    uint64_t u = torus_rotate_rows(t, Lx * b, N, P.full_mask);
    uint32_t rs = rots[r];
    while (rs) {
      int a = ffs64(rs);
      rs &= rs - 1;
      uint64_t V = torus_rotate_within(u, a, Lx, P);
      if (V < o.rep) {
        o.rep = V;
        o.g = a + Lx * b;
        o.stab = 1;
      } else if (V == o.rep) {
        ++o.stab;
      }
    }
  }
  return o;
}

// Is t an allowed representative (rep == t and p_id, Momentum_Basis.cpp:538-540
// and :761-770)?  Returns its stabiliser count, or 0.
EDG_HD int torus_allowed(uint64_t t, const SectorParams& P, const uint8_t* nk, const uint16_t* rots) {
  const int Lx = P.L1, Ly = P.L2, N = P.n_sites;
  const uint64_t rmask = (1ull << Lx) - 1ull;
  // quick reject: the top row must already be at its rotation minimum and no
  // row may have a smaller rotation minimum.
  int top = (int)((t >> (Lx * (Ly - 1))) & rmask);
  if (nk[top] != top) return 0;
  for (int y = 0; y < Ly - 1; ++y)
    if (nk[(int)((t >> (Lx * y)) & rmask)] < top) return 0;
  // full check over the candidates; translates equal to t form the stabiliser
  const int G = P.L1 * P.L2;
  int stab = 0;
  bool trivial = true;  // character trivial on the stabiliser <=> phase sum != 0
  for (int y = Ly - 1; y >= 0; --y) {
    int r = (int)((t >> (Lx * y)) & rmask);
    if (nk[r] != top) continue;
    int b = Ly - 1 - y;
    uint64_t u = torus_rotate_rows(t, Lx * b, N, P.full_mask);
    uint32_t rs = rots[r];
    while (rs) {
      int a = ffs64(rs);
      rs &= rs - 1;
      uint64_t V = torus_rotate_within(u, a, Lx, P);
      if (V < t) return 0;
      if (V == t) {
        ++stab;
        if ((((int64_t)P.kx * a * P.L2 + (int64_t)P.ky * b * P.L1) % G) != 0) trivial = false;
      }
    }
  }
  return trivial ? stab : 0;
}

EDG_HD int walk_allowed(uint64_t t, const SectorParams& P, const uint64_t* perm1, const uint64_t* perm2,
                        const uint64_t* perm3, int n_chunks) {
  if (!walk_is_min(t, P, perm1, perm2, perm3, n_chunks)) return 0;
  double cr, ci;
  Orbit o = orbit_walk(t, P, perm1, perm2, perm3, n_chunks, &cr, &ci);
  if (o.rep != t) return 0;
  bool pid = (cr > 1e-8 || cr < -1e-8 || ci > 1e-8 || ci < -1e-8);
  return pid ? o.stab : 0;
}

// --------------------------------------------------------------------------
// Combinatorics: unrank a Lin index into the configuration, and step to the
// next configuration of the same popcount (Basis_States.cpp:42-73).
// --------------------------------------------------------------------------
EDG_HD uint64_t next_same_popcount(uint64_t t) {
  uint64_t c = t & (0ull - t);
  uint64_t r = t + c;
  return (((r ^ t) >> 2) >> ffs64(c)) | r;
}

// binom[n*(kMaxSites+1)+k] = C(n, k)
EDG_HD uint64_t unrank_config(uint64_t lin, int n_sites, int n_ones, const uint64_t* binom) {
  uint64_t t = 0;
  int c = n_ones;
  for (int p = n_sites - 1; p >= 0 && c > 0; --p) {
    uint64_t below = binom[p * (kMaxSites + 1) + c];  // configurations with bit p clear
    if (lin >= below) {
      t |= 1ull << p;
      lin -= below;
      --c;
    }
  }
  return t;
}

}  // namespace edg
