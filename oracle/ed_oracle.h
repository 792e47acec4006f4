/* CPU restatement of the reference's momentum-basis H*v path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and the CPU
 * baseline of the benchmark call this library as the checker.  The shipped
 * GPU library never links, loads or calls it.
 *
 * Every function restates one routine of the reference (hiteshjc/ED_Code,
 * files under src/), cited at the definition.  Parity of this restatement is
 * pinned against the reference itself compiled from its own sources
 * (oracle/Makefile target "ref") through golden fixtures in tests/golden/.
 */
#ifndef ED_ORACLE_H
#define ED_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { int x, y; double J, re, im; } or_bond;        /* coordinates (global.h:25-30) */
typedef struct { int i, j, k; double re, im; } or_tri;         /* triangles   (global.h:32-35) */
typedef struct { int x, y, z, p, q, r; } or_bowtie;            /* bowties     (global.h:37-40) */

typedef struct {
  int n_sites, n_ones, L1, L2, kx, ky, half_sites;
  int64_t bits_right;
  int64_t n_configs, n_p;
  int64_t *states;      /* pblock_states, ascending                       (n_p)        */
  double *norm;         /* sqrt(L1*L2/lid)                                (n_p)        */
  double *norm_inv;     /* 1/sqrt(L1*L2/lid)                              (n_p)        */
  int32_t *lid;         /* stabiliser count of each representative         (n_p)        */
  int64_t *rep_loc;     /* representative position or -1                  (n_configs)  */
  double *state_ph;     /* exp(-i(px lx + py ly)), interleaved re/im      (2*n_configs)*/
  int32_t *lx, *ly;     /* translation indices behind state_ph            (n_configs)  */
  int64_t *Ia, *Ib;     /* Lin tables                                      (2^half)     */
  int L3, kz;           /* 3-D tori (1, 0 otherwise)                                    */
  int32_t *lz;          /*                                                 (n_configs)  */
} or_basis;

int64_t or_n_choose_k(int n, int k);
void or_lin_tables(int half_sites, int64_t *Ia, int64_t *Ib);
uint64_t or_translate(uint64_t state, const int *T, int n_sites);
void or_LxLy(const int *T1, const int *T2, int n_sites, int *L1, int *L2);
int64_t or_representative(int64_t v, const int *T1, const int *T2, int n_sites, int L1, int L2, double px,
                          double py, int *lx, int *ly, int *lid, int *p_id);

/* Full tables as pConstruct_States builds them.  Returns NULL on bad input. */
or_basis *or_build_basis(int n_sites, int n_ones, const int *T1, const int *T2, int kx, int ky);
or_basis *or_build_basis3(int n_sites, int n_ones, const int *T1, const int *T2, const int *T3, int kx, int ky,
                          int kz);
int64_t or_representative3(int64_t v, const int *T1, const int *T2, const int *T3, int n_sites, int L1, int L2,
                           int L3, double px, double py, double pz, int *lx, int *ly, int *lz, int *lid, int *p_id);
int or_L3(const int *T3, int n_sites);
int64_t or_sector_dim3(int n_sites, int n_ones, const int *T1, const int *T2, const int *T3, int kx, int ky, int kz);
void or_free_basis(or_basis *b);

/* w = H v with the reference's tables (sHv, H_v.cpp:192-357).  v, w interleaved re/im. */
void or_set_threads(int n);
void or_hv_tables(const or_basis *b, const double *v, double *w, double lambda, const or_bond *bonds, int nb,
                  double Ch, const or_tri *tris, int nt, double ChCh, const or_bowtie *bows, int nbw);

/* Selected rows of w = H v without per-configuration tables: each flipped
 * state's representative comes from the orbit walk (representative_p) and its
 * position from a binary search over the sorted representatives (findstate).
 * For sectors whose C(N, n_up) tables do not fit in memory.
 *   reps/lid: the sector's representatives and stabiliser counts (n_p)
 *   rows:     row indices to compute; w_rows receives one complex per row. */
void or_hv_rows(int n_sites, const int *T1, const int *T2, int kx, int ky, const int64_t *reps, const int32_t *lid,
                int64_t n_p, const double *v, const int64_t *rows, int64_t n_rows, double *w_rows, double lambda,
                const or_bond *bonds, int nb, double Ch, const or_tri *tris, int nt, double ChCh,
                const or_bowtie *bows, int nbw, int n_threads);

/* Allowed representatives in increasing order with their stabiliser counts,
 * without the per-configuration tables: the enumeration and acceptance rule of
 * pConstruct_States (Momentum_Basis.cpp:724-770), run in parallel over chunks of
 * the Lin order.  *reps and *lid are malloc'ed (free with or_free). */
void or_value_vector(const int64_t *reps, int64_t n, uint64_t seed, double *v);
void or_hv_rows_listless(int n_sites, const int *T1, const int *T2, int kx, int ky, const int64_t *rows,
                         const int32_t *row_lid, int64_t n_rows, uint64_t vseed, double *w_rows, double lambda,
                         const or_bond *bonds, int nb, double Ch, const or_tri *tris, int nt, double ChCh,
                         const or_bowtie *bows, int nbw, int n_threads, const int64_t *probe, int64_t n_probe);
int64_t or_sample_reps(int n_sites, int n_ones, const int *T1, const int *T2, int kx, int ky, uint64_t seed,
                       int64_t n, int64_t *states, int32_t *lid);
int64_t or_build_reps(int n_sites, int n_ones, const int *T1, const int *T2, int kx, int ky, int64_t **reps,
                      int32_t **lid, int n_threads);
void or_free(void *p);

/* Is `state` an allowed representative (rep == state and p_id)?  Returns lid or 0. */
int or_allowed_rep(int64_t state, const int *T1, const int *T2, int n_sites, int kx, int ky);

/* Sector dimension by the character formula (1/|G|) sum_g conj(chi_k(g)) Fix(g),
 * an independent count for sectors too large to enumerate.  Assumes T1/T2
 * generate Z_L1 x Z_L2. */
int64_t or_sector_dim(int n_sites, int n_ones, const int *T1, const int *T2, int kx, int ky);

#ifdef __cplusplus
}
#endif
#endif
