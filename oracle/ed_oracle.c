/* CPU restatement of the reference's momentum-basis H*v path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker): called by tests/, by the smoke
 * check and by the benchmark's CPU-baseline leg, never by the GPU library.
 * Parity of this file is pinned against the reference compiled from its own
 * sources (oracle/Makefile "ref") through the fixtures in tests/golden/.
 *
 * Each routine follows one routine of the reference (src/ paths of
 * hiteshjc/ED_Code); the citation sits at each definition.  Bit tests use
 * plain shifts where the reference goes through std::bitset
 * (Basis_States.cpp:8-13); the results are the same bits.
 */
#define _GNU_SOURCE
#include "ed_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_PI 3.14159265358979323846 /* M_PI as global.h:17 defines it */

static inline int bit(int64_t a, int pos) { return (int)((((uint64_t)a) >> pos) & 1u); }

/* n_choose_k (Simple_Math_Func.cpp:49-55), exact in 64-bit for n <= 62. */
int64_t or_n_choose_k(int n, int k) {
  if (k < 0 || k > n) return 0;
  if (k > n - k) k = n - k;
  int64_t r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return r;
}

/* Next larger integer with the same popcount (Basis_States.cpp:42-73,
 * "constrained_dets", Gosper's hack). */
static inline int64_t next_same_popcount(int64_t t) {
  int64_t c = t & -t;
  int64_t r = t + c;
  return (((r ^ t) >> 2) / c) | r;
}

/* Lin_Tables (Lin_Tables.cpp:57-78): Ia[w] = 1-based rank of w among the
 * half-words of equal popcount in increasing order; Ib = -1 (filled by the
 * basis build). */
void or_lin_tables(int half_sites, int64_t *Ia, int64_t *Ib) {
  int64_t n = (int64_t)1 << half_sites;
  int64_t next_rank[65];
  for (int i = 0; i <= 64; ++i) next_rank[i] = 1;
  for (int64_t w = 0; w < n; ++w) {
    int pc = __builtin_popcountll((unsigned long long)w);
    Ia[w] = next_rank[pc]++;
    Ib[w] = -1;
  }
}

/* translateT (Momentum_Basis.cpp:4-16): bit i moves to T[i]. */
uint64_t or_translate(uint64_t state, const int *T, int n_sites) {
  uint64_t out = 0;
  for (int i = 0; i < n_sites; ++i)
    if ((state >> i) & 1u) out |= (uint64_t)1 << T[i];
  return out;
}

/* LxLy (Momentum_Basis.cpp:19-36): cycle lengths of state 1 under T1, T2. */
void or_LxLy(const int *T1, const int *T2, int n_sites, int *L1, int *L2) {
  uint64_t t = 1;
  *L1 = 0;
  do { t = or_translate(t, T1, n_sites); ++*L1; } while (t != 1 && *L1 <= 64);
  t = 1;
  *L2 = 0;
  do { t = or_translate(t, T2, n_sites); ++*L2; } while (t != 1 && *L2 <= 64);
}

/* representative_p (Momentum_Basis.cpp:472-543).  Walk order: for x < L1
 * { if x>0 apply T1; for y < L2 { if y>0 apply T2 } }; T2 is not reset
 * between x steps.  The first strict minimum wins and records lx = L1-tx,
 * ly = L2-ty.  lid counts translates equal to v (identity included); p_id
 * tests the accumulated phase sum against 1e-8. */
/* representative_p, 3-D (Momentum_Basis.cpp:545-643): for x < L1 { if x>0
 * T1; for y < L2 { if y>0 T2; for z < L3 { if z>0 T3 } } }.  With T3 == NULL
 * (L3 = 1) the z loop applies nothing and this is the 2-D walk
 * (Momentum_Basis.cpp:472-543) step for step. */
int64_t or_representative3(int64_t v, const int *T1, const int *T2, const int *T3, int n_sites, int L1, int L2,
                           int L3, double px, double py, double pz, int *lx, int *ly, int *lz, int *lid, int *p_id) {
  *lx = 0; *ly = 0; *lz = 0;
  int64_t rep = v, tmp = v;
  int tx = 0, ty = 0, tz = 0;
  double complex ph = 1.0, id_coeff = 1.0;
  const double complex ex = cexp(CMPLX(0.0, -px)), ey = cexp(CMPLX(0.0, -py)), ez = cexp(CMPLX(0.0, -pz));
  *lid = 1;
  for (int x = 0; x < L1; ++x) {
    if (x > 0) {
      tmp = (int64_t)or_translate((uint64_t)tmp, T1, n_sites);
      ++tx;
      ph = ph * ex;
      if (v == tmp) { id_coeff = id_coeff + ph; ++*lid; }
      if (rep > tmp) { rep = tmp; *lx = L1 - tx; *ly = L2 - ty; *lz = L3 - tz; }
    }
    for (int y = 0; y < L2; ++y) {
      if (y > 0) {
        tmp = (int64_t)or_translate((uint64_t)tmp, T2, n_sites);
        ++ty;
        ph = ph * ey;
        if (v == tmp) { id_coeff = id_coeff + ph; ++*lid; }
        if (rep > tmp) { rep = tmp; *lx = L1 - tx; *ly = L2 - ty; *lz = L3 - tz; }
      }
      for (int z = 1; z < L3; ++z) {
        tmp = (int64_t)or_translate((uint64_t)tmp, T3, n_sites);
        ++tz;
        ph = ph * ez;
        if (v == tmp) { id_coeff = id_coeff + ph; ++*lid; }
        if (rep > tmp) { rep = tmp; *lx = L1 - tx; *ly = L2 - ty; *lz = L3 - tz; }
      }
    }
  }
  *p_id = (fabs(creal(id_coeff)) > 1e-8 || fabs(cimag(id_coeff)) > 1e-8) ? 1 : 0;
  return rep;
}

int64_t or_representative(int64_t v, const int *T1, const int *T2, int n_sites, int L1, int L2, double px,
                          double py, int *lx, int *ly, int *lid, int *p_id) {
  int lz;
  return or_representative3(v, T1, T2, NULL, n_sites, L1, L2, 1, px, py, 0.0, lx, ly, &lz, lid, p_id);
}

/* L3 of LxLyLz (Momentum_Basis.cpp:38-63); 1 without T3. */
int or_L3(const int *T3, int n_sites) {
  if (!T3) return 1;
  int L3 = 0;
  uint64_t t = 1;
  do { t = or_translate(t, T3, n_sites); ++L3; } while (t != 1);
  return L3;
}

/* findstate (binary search over the ascending representatives, as
 * Heisenberg_Hamiltonian.cpp:51-69 does): position or -1. */
static int64_t find_state(int64_t key, const int64_t *reps, int64_t n) {
  int64_t lo = 0, hi = n - 1;
  while (lo <= hi) {
    int64_t mid = lo + (hi - lo) / 2;
    if (key < reps[mid]) hi = mid - 1;
    else if (key > reps[mid]) lo = mid + 1;
    else return mid;
  }
  return -1;
}

/* pConstruct_States, 2-D (Momentum_Basis.cpp:645-778) and 3-D (:781-895):
 * T3 == NULL is the 2-D case. */
or_basis *or_build_basis3(int n_sites, int n_ones, const int *T1, const int *T2, const int *T3, int kx, int ky,
                          int kz) {
  if (n_sites < 1 || n_sites > 62 || n_ones < 0 || n_ones > n_sites) return NULL;
  or_basis *b = (or_basis *)calloc(1, sizeof(or_basis));
  b->n_sites = n_sites; b->n_ones = n_ones; b->kx = kx; b->ky = ky; b->kz = kz;
  int half = n_sites / 2;
  if (n_sites % 2 == 1) ++half; /* Momentum_Basis.cpp:681-682 */
  b->half_sites = half;
  or_LxLy(T1, T2, n_sites, &b->L1, &b->L2);
  b->L3 = or_L3(T3, n_sites);
  const int L1 = b->L1, L2 = b->L2, L3 = b->L3;
  const double px = 2 * kx * OR_PI / L1, py = 2 * ky * OR_PI / L2; /* Lanczos_sector.cpp:57 */
  const double pz = 2 * kz * OR_PI / L3;                              /* Lanczos_sector.cpp:240 */
  const int64_t nc = or_n_choose_k(n_sites, n_ones);
  b->n_configs = nc;
  const int64_t nh = (int64_t)1 << half;
  b->Ia = (int64_t *)malloc(sizeof(int64_t) * nh);
  b->Ib = (int64_t *)malloc(sizeof(int64_t) * nh);
  or_lin_tables(half, b->Ia, b->Ib);
  b->bits_right = nh - 1; /* Momentum_Basis.cpp:720 */

  int64_t *all = (int64_t *)malloc(sizeof(int64_t) * (nc ? nc : 1));
  int64_t *rep_ids = (int64_t *)malloc(sizeof(int64_t) * (nc ? nc : 1));
  unsigned char *pids = (unsigned char *)malloc(nc ? nc : 1);
  int32_t *lids = (int32_t *)malloc(sizeof(int32_t) * (nc ? nc : 1));
  b->rep_loc = (int64_t *)malloc(sizeof(int64_t) * (nc ? nc : 1));
  b->state_ph = (double *)malloc(sizeof(double) * 2 * (nc ? nc : 1));
  b->lx = (int32_t *)malloc(sizeof(int32_t) * (nc ? nc : 1));
  b->ly = (int32_t *)malloc(sizeof(int32_t) * (nc ? nc : 1));
  b->lz = (int32_t *)malloc(sizeof(int32_t) * (nc ? nc : 1));

  /* constrained_dets: all states in increasing order. */
  int64_t t = n_ones ? (((int64_t)1 << n_ones) - 1) : 0;
  for (int64_t i = 0; i < nc; ++i) {
    all[i] = t;
    if (i + 1 < nc) t = next_same_popcount(t);
  }
  /* Ib fill and split_id (Lin_Tables.cpp:42-54; Momentum_Basis.cpp:731-737):
   * right = id & bits_right, left = id >> (n_sites/2). */
  const int split = n_sites / 2;
  for (int64_t i = 0; i < nc; ++i) {
    int64_t left = all[i] >> split, right = all[i] & b->bits_right;
    if (b->Ib[left] == -1) b->Ib[left] = i - b->Ia[right] + 1;
  }
#pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t i = 0; i < nc; ++i) {
    int lx, ly, lz, lid, pid;
    rep_ids[i] = or_representative3(all[i], T1, T2, T3, n_sites, L1, L2, L3, px, py, pz, &lx, &ly, &lz, &lid, &pid);
    pids[i] = (unsigned char)pid;
    lids[i] = lid;
    lx = lx % L1;
    ly = ly % L2;
    lz = lz % L3;
    if (lx < 0) lx += L1;
    if (ly < 0) ly += L2;
    if (lz < 0) lz += L3;
    b->lx[i] = lx;
    b->ly[i] = ly;
    b->lz[i] = lz;
    /* Momentum_Basis.cpp:753 (2-D), :872 (3-D); pz*lz is 0 without T3 */
    double complex ph = T3 ? cexp(CMPLX(0.0, -px * lx - py * ly - pz * lz)) : cexp(CMPLX(0.0, -px * lx - py * ly));
    b->state_ph[2 * i] = creal(ph);
    b->state_ph[2 * i + 1] = cimag(ph);
  }
  int64_t np = 0;
  for (int64_t i = 0; i < nc; ++i)
    if (rep_ids[i] == all[i] && pids[i]) ++np;
  b->n_p = np;
  b->states = (int64_t *)malloc(sizeof(int64_t) * (np ? np : 1));
  b->norm = (double *)malloc(sizeof(double) * (np ? np : 1));
  b->norm_inv = (double *)malloc(sizeof(double) * (np ? np : 1));
  b->lid = (int32_t *)malloc(sizeof(int32_t) * (np ? np : 1));
  np = 0;
  for (int64_t i = 0; i < nc; ++i) {
    if (rep_ids[i] == all[i] && pids[i]) {
      int64_t N = (int64_t)(L1 * L2 * L3) / lids[i]; /* integer division, Momentum_Basis.cpp:764, :883 */
      b->states[np] = all[i];
      b->norm[np] = sqrt((double)N);
      b->norm_inv[np] = 1 / sqrt((double)N);
      b->lid[np] = lids[i];
      ++np;
    }
  }
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < nc; ++i) b->rep_loc[i] = find_state(rep_ids[i], b->states, np);
  free(all); free(rep_ids); free(pids); free(lids);
  return b;
}

or_basis *or_build_basis(int n_sites, int n_ones, const int *T1, const int *T2, int kx, int ky) {
  return or_build_basis3(n_sites, n_ones, T1, T2, NULL, kx, ky, 0);
}

void or_free_basis(or_basis *b) {
  if (!b) return;
  free(b->states); free(b->norm); free(b->norm_inv); free(b->lid); free(b->rep_loc);
  free(b->state_ph); free(b->lx); free(b->ly); free(b->lz); free(b->Ia); free(b->Ib);
  free(b);
}

static inline int64_t flip2(int64_t s, int i, int j) { return s ^ (((int64_t)1 << i) | ((int64_t)1 << j)); }

/* One row of sHv (H_v.cpp:218-355), term for term and in the same order.
 * `lookup` maps a flipped state to (j, state_ph) the way the row needs it. */
typedef struct {
  const or_basis *tab;               /* table mode */
  /* walk mode */
  int n_sites, L1, L2;
  const int *T1, *T2;
  double px, py;
  const int64_t *reps;
  const int32_t *lid;
  int64_t n_p;
  /* list-free mode (reps == NULL): v_j is value_vector(rep, vseed) */
  uint64_t vseed;
  /* list-free mode's stand-in for the rank lookup: a binary search of the
   * representative in a sorted array of the list's size (the index found is
   * stored to a volatile sink, so the search is not optimised away) */
  const int64_t *probe;
  int64_t n_probe;
} or_lookup;
static volatile int64_t or_probe_sink;

/* Deterministic vector entry as a function of a representative's value (used
 * where the representative list is not built): splitmix64, uniform in [-1,1)^2. */
static uint64_t splitmix64_next(uint64_t *s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static double complex value_vector(int64_t rep, uint64_t seed) {
  uint64_t s = seed ^ ((uint64_t)rep * 0xD6E8FEB86659FD93ull);
  double a = (double)(splitmix64_next(&s) >> 11) * 0x1.0p-53, b = (double)(splitmix64_next(&s) >> 11) * 0x1.0p-53;
  return CMPLX(2 * a - 1, 2 * b - 1);
}

void or_value_vector(const int64_t *reps, int64_t n, uint64_t seed, double *v) {
  for (int64_t j = 0; j < n; ++j) {
    double complex x = value_vector(reps[j], seed);
    v[2 * j] = creal(x);
    v[2 * j + 1] = cimag(x);
  }
}

/* j of a flipped state (or -1) with its phase and 1/norm; *vj = v_j. */
static inline int64_t lookup_target(const or_lookup *L, int64_t tmp, const double *v, double complex *ph,
                                    double *ninv, double complex *vj) {
  if (L->tab) {
    const or_basis *b = L->tab;
    int64_t left = tmp >> (b->n_sites / 2), right = tmp & b->bits_right;
    int64_t loc = b->Ia[right] + b->Ib[left] - 1;
    int64_t j = b->rep_loc[loc];
    *ph = CMPLX(b->state_ph[2 * loc], b->state_ph[2 * loc + 1]);
    if (j >= 0) {
      *ninv = b->norm_inv[j];
      *vj = CMPLX(v[2 * j], v[2 * j + 1]);
    }
    return j;
  }
  int lx, ly, lid, pid;
  int64_t rep = or_representative(tmp, L->T1, L->T2, L->n_sites, L->L1, L->L2, L->px, L->py, &lx, &ly, &lid, &pid);
  lx %= L->L1; ly %= L->L2;
  if (lx < 0) lx += L->L1;
  if (ly < 0) ly += L->L2;
  *ph = cexp(CMPLX(0.0, -L->px * lx - L->py * ly));
  if (!L->reps) {
    if (!pid) return -1;
    *ninv = 1 / sqrt((double)((int64_t)(L->L1 * L->L2) / lid));
    *vj = value_vector(rep, L->vseed);
    if (L->probe) or_probe_sink = find_state(rep, L->probe, L->n_probe);
    return 0;
  }
  int64_t j = find_state(rep, L->reps, L->n_p);
  if (j >= 0) {
    *ninv = 1 / sqrt((double)((int64_t)(L->L1 * L->L2) / L->lid[j]));
    *vj = CMPLX(v[2 * j], v[2 * j + 1]);
  }
  return j;
}

static double complex hv_row(const or_lookup *L, int64_t idi, double norm_i, double complex v_i, const double *v,
                             double lambda, const or_bond *bonds, int nb, double Ch, const or_tri *tris, int nt,
                             double ChCh, const or_bowtie *bows, int nbw) {
  const double Ezzfac = 0.25 * lambda;
  double complex w = 0.0;
  double Ezz = 0.0;
  for (int k = 0; k < nb; ++k) {
    int x = bonds[k].x, y = bonds[k].y;
    double J = bonds[k].J;
    double complex e = CMPLX(bonds[k].re, bonds[k].im);
    if (fabs(J) < 1e-16) continue;
    int tx = bit(idi, x), ty = bit(idi, y);
    if (tx == ty) {
      Ezz += (Ezzfac * J);
    } else {
      if (tx == 1) e = conj(e);
      Ezz += -(Ezzfac * J);
      double complex ph, vj = 0; double ninv = 0;
      int64_t j = lookup_target(L, flip2(idi, x, y), v, &ph, &ninv, &vj);
      if (j >= 0) {
        w += e * J * 0.5 * vj * ph * norm_i * ninv;
      }
    }
  }
  w += v_i * Ezz;
  if (fabs(Ch) > 1e-16) {
    for (int k = 0; k < nt; ++k) {
      int x = tris[k].i, y = tris[k].j, z = tris[k].k;
      double complex ep = CMPLX(tris[k].re, tris[k].im);
      int tx = bit(idi, x), ty = bit(idi, y);
      if (tx != ty) {
        double complex ph, vj = 0; double ninv = 0;
        int64_t j = lookup_target(L, flip2(idi, x, y), v, &ph, &ninv, &vj);
        if (j >= 0) {
          double complex sgn = (ty == 1) ? CMPLX(0, 1) * ep : CMPLX(0, -1) * conj(ep);
          if (bit(idi, z) == 0) sgn = sgn * CMPLX(-1, 0);
          double complex ele = Ch * 0.25 * sgn * ph * norm_i * ninv;
          w += ele * vj;
        }
      }
    }
  }
  if (fabs(ChCh) > 1e-16) {
    for (int k = 0; k < nbw; ++k) {
      int x = bows[k].x, y = bows[k].y, z = bows[k].z, p = bows[k].p, q = bows[k].q, r = bows[k].r;
      int tx = bit(idi, x), ty = bit(idi, y);
      double complex s1 = (ty == 1) ? CMPLX(0, 1) : CMPLX(0, -1);
      if (tx != ty) {
        int64_t tmp = flip2(idi, x, y);
        int tz = bit(tmp, z), tp = bit(tmp, p), tq = bit(tmp, q);
        if (tz == 0) s1 = s1 * CMPLX(-1, 0);
        double complex s2 = (tq == 1) ? CMPLX(0, 1) : CMPLX(0, -1);
        if (tp != tq) {
          int64_t tmp2 = flip2(tmp, p, q);
          int tr = bit(tmp2, r);
          double complex ph, vj = 0; double ninv = 0;
          int64_t j = lookup_target(L, tmp2, v, &ph, &ninv, &vj);
          if (j >= 0) {
            if (tr == 0) s2 = s2 * CMPLX(-1, 0);
            double complex ele = ChCh * 0.25 * 0.25 * s1 * s2 * ph * norm_i * ninv;
            w += ele * vj;
          }
        }
      }
    }
  }
  return w;
}

/* sHv, 2-D (H_v.cpp:192-357), with the reference's tables. */
/* Threads of the OpenMP loops that take no thread count (table-mode H*v,
 * basis build); 0 or less leaves the runtime's default. */
void or_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

void or_hv_tables(const or_basis *b, const double *v, double *w, double lambda, const or_bond *bonds, int nb,
                  double Ch, const or_tri *tris, int nt, double ChCh, const or_bowtie *bows, int nbw) {
  or_lookup L;
  memset(&L, 0, sizeof L);
  L.tab = b;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < b->n_p; ++i) {
    double complex vi = CMPLX(v[2 * i], v[2 * i + 1]);
    double complex r = hv_row(&L, b->states[i], b->norm[i], vi, v, lambda, bonds, nb, Ch, tris, nt, ChCh, bows, nbw);
    w[2 * i] = creal(r);
    w[2 * i + 1] = cimag(r);
  }
}

void or_hv_rows(int n_sites, const int *T1, const int *T2, int kx, int ky, const int64_t *reps, const int32_t *lid,
                int64_t n_p, const double *v, const int64_t *rows, int64_t n_rows, double *w_rows, double lambda,
                const or_bond *bonds, int nb, double Ch, const or_tri *tris, int nt, double ChCh,
                const or_bowtie *bows, int nbw, int n_threads) {
  or_lookup L;
  memset(&L, 0, sizeof L);
  L.n_sites = n_sites; L.T1 = T1; L.T2 = T2; L.reps = reps; L.lid = lid; L.n_p = n_p;
  or_LxLy(T1, T2, n_sites, &L.L1, &L.L2);
  L.px = 2 * kx * OR_PI / L.L1;
  L.py = 2 * ky * OR_PI / L.L2;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#else
  (void)n_threads;
#endif
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t r = 0; r < n_rows; ++r) {
    int64_t i = rows[r];
    double norm_i = sqrt((double)((int64_t)(L.L1 * L.L2) / lid[i]));
    double complex vi = CMPLX(v[2 * i], v[2 * i + 1]);
    double complex o = hv_row(&L, reps[i], norm_i, vi, v, lambda, bonds, nb, Ch, tris, nt, ChCh, bows, nbw);
    w_rows[2 * r] = creal(o);
    w_rows[2 * r + 1] = cimag(o);
  }
}

/* Rows of H v without the representative list, for sectors whose list is too
 * large to build on the host: `rows` are representatives (or_sample_reps) and
 * v is value_vector(representative, vseed), so a target costs its orbit walk
 * (representative_p, Momentum_Basis.cpp:472-543).  With `probe` (a sorted
 * array of n_probe values, the list's size) each target also costs the
 * binary search that finds its rank in the list (find_state); without it, no
 * rank lookup. */
void or_hv_rows_listless(int n_sites, const int *T1, const int *T2, int kx, int ky, const int64_t *rows,
                         const int32_t *row_lid, int64_t n_rows, uint64_t vseed, double *w_rows, double lambda,
                         const or_bond *bonds, int nb, double Ch, const or_tri *tris, int nt, double ChCh,
                         const or_bowtie *bows, int nbw, int n_threads, const int64_t *probe, int64_t n_probe) {
  or_lookup L;
  memset(&L, 0, sizeof L);
  L.n_sites = n_sites; L.T1 = T1; L.T2 = T2; L.vseed = vseed;
  L.probe = probe; L.n_probe = n_probe;
  or_LxLy(T1, T2, n_sites, &L.L1, &L.L2);
  L.px = 2 * kx * OR_PI / L.L1;
  L.py = 2 * ky * OR_PI / L.L2;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#else
  (void)n_threads;
#endif
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t r = 0; r < n_rows; ++r) {
    double norm_i = sqrt((double)((int64_t)(L.L1 * L.L2) / row_lid[r]));
    double complex o = hv_row(&L, rows[r], norm_i, value_vector(rows[r], vseed), NULL, lambda, bonds, nb, Ch, tris,
                              nt, ChCh, bows, nbw);
    w_rows[2 * r] = creal(o);
    w_rows[2 * r + 1] = cimag(o);
  }
}

/* n representatives drawn by taking random n_ones-subsets (splitmix64 stream
 * `seed`) and keeping those that are their orbit's allowed representative. */
int64_t or_sample_reps(int n_sites, int n_ones, const int *T1, const int *T2, int kx, int ky, uint64_t seed,
                       int64_t n, int64_t *states, int32_t *lid_out) {
  int L1, L2;
  or_LxLy(T1, T2, n_sites, &L1, &L2);
  const double px = 2 * kx * OR_PI / L1, py = 2 * ky * OR_PI / L2;
  uint64_t s = seed;
  int64_t got = 0;
  for (int64_t tries = 0; got < n && tries < 1000 * (n + 10); ++tries) {
    int idx[64];
    for (int k = 0; k < n_sites; ++k) idx[k] = k;
    int64_t t = 0;
    for (int k = 0; k < n_ones; ++k) {
      int r = k + (int)(splitmix64_next(&s) % (uint64_t)(n_sites - k));
      int tmp = idx[k]; idx[k] = idx[r]; idx[r] = tmp;
      t |= (int64_t)1 << idx[k];
    }
    int lx, ly, lid, pid;
    int64_t rep = or_representative(t, T1, T2, n_sites, L1, L2, px, py, &lx, &ly, &lid, &pid);
    if (!pid) continue;
    states[got] = rep;
    lid_out[got] = lid;
    ++got;
  }
  return got;
}

int or_allowed_rep(int64_t state, const int *T1, const int *T2, int n_sites, int kx, int ky) {
  int L1, L2, lx, ly, lid, pid;
  or_LxLy(T1, T2, n_sites, &L1, &L2);
  double px = 2 * kx * OR_PI / L1, py = 2 * ky * OR_PI / L2;
  int64_t rep = or_representative(state, T1, T2, n_sites, L1, L2, px, py, &lx, &ly, &lid, &pid);
  return (rep == state && pid) ? lid : 0;
}

/* Character count of the sector dimension: (1/|G|) sum_{a,b} chi(a,b) Fix(T1^a T2^b),
 * Fix(g) = number of n_ones-subsets that are unions of cycles of g. */
int64_t or_sector_dim3(int n_sites, int n_ones, const int *T1, const int *T2, const int *T3, int kx, int ky, int kz) {
  int L1, L2;
  or_LxLy(T1, T2, n_sites, &L1, &L2);
  const int L3 = or_L3(T3, n_sites);
  int perm[64], seen[64];
  long double total = 0;
  for (int a = 0; a < L1; ++a) {
    for (int b = 0; b < L2; ++b) {
     for (int c3 = 0; c3 < L3; ++c3) {
      for (int s = 0; s < n_sites; ++s) {
        int t = s;
        for (int k = 0; k < a; ++k) t = T1[t];
        for (int k = 0; k < b; ++k) t = T2[t];
        for (int k = 0; k < c3; ++k) t = T3[t];
        perm[s] = t;
      }
      /* coefficient of x^n_ones in prod (1 + x^len) */
      long double poly[65];
      for (int k = 0; k <= 64; ++k) poly[k] = 0;
      poly[0] = 1;
      memset(seen, 0, sizeof seen);
      for (int s = 0; s < n_sites; ++s) {
        if (seen[s]) continue;
        int len = 0, t = s;
        while (!seen[t]) { seen[t] = 1; t = perm[t]; ++len; }
        for (int k = 64; k >= len; --k) poly[k] += poly[k - len];
      }
      double ang = 2 * OR_PI * ((double)kx * a / L1 + (double)ky * b / L2 + (double)kz * c3 / L3);
      total += poly[n_ones] * (long double)cos(ang);
     }
    }
  }
  return (int64_t)llroundl(total / (L1 * L2 * L3));
}

int64_t or_sector_dim(int n_sites, int n_ones, const int *T1, const int *T2, int kx, int ky) {
  return or_sector_dim3(n_sites, n_ones, T1, T2, NULL, kx, ky, 0);
}

/* Unrank Lin index r (increasing-integer order of n_sites-bit words with
 * n_ones bits) into the word. */
static int64_t unrank_lin(int64_t r, int n_sites, int n_ones) {
  int64_t t = 0;
  int c = n_ones;
  for (int p = n_sites - 1; p >= 0 && c > 0; --p) {
    int64_t below = or_n_choose_k(p, c);
    if (r >= below) { t |= (int64_t)1 << p; r -= below; --c; }
  }
  return t;
}

/* Any translate smaller than t?  (Early exit; order irrelevant.) */
static int smaller_translate(int64_t t, const int *T1, const int *T2, int n, int L1, int L2) {
  uint64_t row = (uint64_t)t;
  for (int x = 0; x < L1; ++x) {
    uint64_t tmp = row;
    for (int y = 1; y < L2; ++y) {
      tmp = or_translate(tmp, T2, n);
      if ((int64_t)tmp < t) return 1;
    }
    row = or_translate(row, T1, n);
    if (x + 1 < L1 && (int64_t)row < t) return 1;
  }
  return 0;
}

int64_t or_build_reps(int n_sites, int n_ones, const int *T1, const int *T2, int kx, int ky, int64_t **reps_out,
                      int32_t **lid_out, int n_threads) {
  int L1, L2;
  or_LxLy(T1, T2, n_sites, &L1, &L2);
  const double px = 2 * kx * OR_PI / L1, py = 2 * ky * OR_PI / L2;
  const int64_t nc = or_n_choose_k(n_sites, n_ones);
  const int64_t chunk = 1 << 16;
  const int64_t nchunks = (nc + chunk - 1) / chunk;
  int64_t *cnt = (int64_t *)calloc((size_t)nchunks + 1, sizeof(int64_t));
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#else
  (void)n_threads;
#endif
  for (int pass = 0; pass < 2; ++pass) {
    if (pass == 1) {
      int64_t run = 0;
      for (int64_t c = 0; c < nchunks; ++c) { int64_t k = cnt[c]; cnt[c] = run; run += k; }
      cnt[nchunks] = run;
      *reps_out = (int64_t *)malloc(sizeof(int64_t) * (run ? run : 1));
      *lid_out = (int32_t *)malloc(sizeof(int32_t) * (run ? run : 1));
    }
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t c = 0; c < nchunks; ++c) {
      int64_t i0 = c * chunk, i1 = i0 + chunk < nc ? i0 + chunk : nc;
      int64_t t = unrank_lin(i0, n_sites, n_ones);
      int64_t k = pass ? cnt[c] : 0;
      for (int64_t i = i0; i < i1; ++i) {
        if (!smaller_translate(t, T1, T2, n_sites, L1, L2)) {
          int lx, ly, lid, pid;
          int64_t rep = or_representative(t, T1, T2, n_sites, L1, L2, px, py, &lx, &ly, &lid, &pid);
          if (rep == t && pid) {
            if (pass) { (*reps_out)[k] = t; (*lid_out)[k] = lid; }
            ++k;
          }
        }
        if (i + 1 < i1) t = next_same_popcount(t);
      }
      if (!pass) cnt[c] = k;
    }
  }
  int64_t n = cnt[nchunks];
  free(cnt);
  return n;
}

void or_free(void *p) { free(p); }
