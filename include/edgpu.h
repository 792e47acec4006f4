/* edgpu -- GB300 (sm_103a) momentum-sector exact diagonalisation, C ABI.
 *
 * Drop-in GPU replacement for the H*v hot path of hiteshjc/ED_Code and the
 * solvers around it.  Every entry point below names the reference interface
 * it replaces (paths are src/ files of the reference).  All pointers are
 * plain host or device pointers; no C++ or framework types cross this
 * boundary.  Every function returns EDG_OK (0) or an EDG_ERR_* code;
 * edg_last_error() returns the message of the last failure on the calling
 * thread.  Complex vectors are interleaved (re, im) arrays: EDG_C128 is
 * double[2*n] (std::complex<double>), EDG_C64 is float[2*n].
 */
#ifndef EDGPU_H
#define EDGPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define EDGPU_ABI_VERSION 8

enum {
  EDG_OK = 0,
  EDG_ERR_INVALID = 1,      /* malformed argument (bad permutation, odd N, n_ones out of range, ...) */
  EDG_ERR_MOMENTUM = 2,     /* kx/ky outside [0,L1)x[0,L2): the reference's "Invalid kx or ky" */
  EDG_ERR_EMPTY = 3,        /* the sector has no states: the reference's "No states in psector" */
  EDG_ERR_CUDA = 4,         /* a CUDA call failed */
  EDG_ERR_NOMEM = 5,        /* not enough device memory for the sector */
  EDG_ERR_UNSUPPORTED = 6,  /* outside what this library implements (N > 40, too many terms) */
  EDG_ERR_NOT_CONVERGED = 7, /* eigensolver stopped without meeting its tolerance */
  EDG_ERR_CANCELLED = 8      /* a batch segment withdrawn by edg_batch_cancel */
};

enum { EDG_C128 = 0, EDG_C64 = 1 };

/* Term-list entries, field for field the reference's structs (global.h:25-40).
 * expphase is given as (re, im). */
typedef struct { int x, y; double J, re, im; } edg_bond;          /* coordinates */
typedef struct { int i, j, k; double re, im; } edg_triangle;      /* triangles   */
typedef struct { int x, y, z, p, q, r; } edg_bowtie;              /* bowties     */

/* The Hamiltonian: what ED_2D_Lattice_Geometry (read_input_file.cpp:110-430)
 * hands to sector_lanczos.  lambda is Jz. */
typedef struct {
  int n_sites;
  const int* T1;
  const int* T2;
  double lambda;
  const edg_bond* bonds;
  int n_bonds;
  double Ch;
  const edg_triangle* triangles;
  int n_triangles;
  double ChCh;
  const edg_bowtie* bowties;
  int n_bowties;
  const int* T3;         /* third translation of a 3-D torus (ED_3D_Lattice_Geometry,
                            read_input_file.cpp:443); NULL for 2-D */
} edg_model;

typedef struct edg_sector edg_sector;

typedef struct {
  int n_sites, n_ones, L1, L2, kx, ky;
  int torus;             /* 1: row-rotation orbit search, 0: the reference's walk */
  int n_groups;          /* distinct flipped pairs after merging bond + chirality terms */
  int64_t n_p;           /* sector dimension */
  int64_t n_configs;     /* C(N, n_ones) */
  int64_t device_bytes;  /* device memory held by the sector */
  int64_t n_targets;     /* stored nonzeros (0: H*v searches on the fly) */
  int lanes_per_row;     /* stored-row H*v: lanes of a warp per row (edg_sector_tune) */
  int cache_policy;      /* stored-row H*v: 1 streaming row loads, 2 L2 evict-first row loads */
  int L3, kz;            /* third translation's cycle length and momentum (1, 0 in 2-D) */
  int entry_bytes;       /* bytes of one stored nonzero: 4 (column and value id packed in one
                            u32), 6 (u32 column + u16 value id), 0 without stored rows */
  int n_values;          /* distinct values of the stored rows' value table */
  int ctas_per_sm;       /* stored-row H*v: CTAs per SM (0: as many as fit) */
  int pipelined;         /* stored-row H*v: 1 when the next rows' entries load during the gathers */
} edg_sector_info;

const char* edg_last_error(void);
int edg_abi_version(void);

/* Build the (n_ones, kx, ky) sector on the current CUDA device.
 * Replaces: LxLy + pConstruct_States (Momentum_Basis.cpp:19-36, 645-778) and
 * Lin_Tables (Lin_Tables.cpp:57-78) as called from sector_lanczos
 * (Lanczos_sector.cpp:48-97).  Errors: EDG_ERR_MOMENTUM, EDG_ERR_EMPTY as the
 * reference's exit(1) paths (Lanczos_sector.cpp:51-55, 93-97). */
int edg_sector_create(const edg_model* model, int n_ones, int kx, int ky, edg_sector** out);
/* Same for a 3-D torus (model->T3 set) with momentum (kx, ky, kz).
 * Replaces: LxLyLz + the 3-D pConstruct_States (Momentum_Basis.cpp:38-63,
 * 781-895) as called from the 3-D sector_lanczos (Lanczos_sector.cpp:201-257);
 * the orbit walk, phases exp(-i(px lx + py ly + pz lz)) and norms
 * sqrt(L1 L2 L3 / lid) follow representative_p (Momentum_Basis.cpp:545-643).
 * With model->T3 == NULL and kz == 0 it is edg_sector_create. */
int edg_sector_create3(const edg_model* model, int n_ones, int kx, int ky, int kz, edg_sector** out);
int edg_sector_destroy(edg_sector* s);
int edg_sector_get_info(const edg_sector* s, edg_sector_info* info);

/* Host copies of pblock_states, norm and norm_inv (Momentum_Basis.cpp:756-770).
 * Any pointer may be NULL. */
int edg_sector_copy_basis(const edg_sector* s, int64_t* states, double* norm, double* norm_inv);

/* Host copies of the Lin tables Ia, Ib (2^(N/2) entries each; Lin_Tables.cpp:57-78,
 * Momentum_Basis.cpp:731-737) and bits_right. */
int edg_sector_copy_lin_tables(const edg_sector* s, int64_t* Ia, int64_t* Ib, int64_t* bits_right);

/* The reference's per-configuration tables rep_loc and state_ph
 * (Momentum_Basis.cpp:750-777), computed with the reference's own orbit walk,
 * for parity checks on sectors with at most max_configs configurations.
 * state_ph is interleaved (re, im); lxly receives lx, ly pairs; any output may be NULL. */
int edg_sector_copy_config_tables(const edg_sector* s, int64_t max_configs, int64_t* rep_loc, double* state_ph,
                                  int32_t* lxly);

/* w = H v on device pointers (n_p complex entries each, dtype EDG_C128 or
 * EDG_C64), enqueued on `stream` (a cudaStream_t; NULL is the legacy default
 * stream).  v and w must not overlap.
 * Replaces: sHv (H_v.cpp:192-357, declared H_v.h:36-57). */
int edg_hv(edg_sector* s, const void* v, void* w, int dtype, void* stream);

/* Search every row's flipped states once and keep the result in HBM as
 * compressed sparse rows: per nonzero its column and an index into a
 * deduplicated table of (pair coefficient x phase) values, per row its
 * diagonal.  Column and index share one u32 when both fit (4 bytes per
 * nonzero, 56 GB for the 36-site Sz=0, k=0 sector), else a u32 column and a
 * u16 index (6 bytes; the environment variable EDG_ROW_FORMAT=split forces
 * this form).  Afterwards edg_hv streams
 * these rows instead of searching orbits.  Fails with EDG_ERR_NOMEM (sector
 * unchanged, still matrix-free) when they need more than max_bytes (<= 0: no
 * limit) or than is free; EDG_ERR_UNSUPPORTED for ChCh terms or more than
 * 65536 distinct values.  H*v calls on one sector must not overlap: they
 * share a scratch vector.  Counterpart in the reference: the optional
 * sparse-matrix sHv (H_v.cpp:3-19), which stores complex values per nonzero. */
int edg_sector_build_targets(edg_sector* s, int64_t max_bytes);
int edg_sector_free_targets(edg_sector* s);

/* Lanes of a warp per stored row (8, 16 or 32, i.e. 4, 2 or 1 rows per warp),
 * the cache policy of the row loads, the CTAs per SM (as many as fit, or at
 * most 4, 3, 2 or 1: fewer rows in flight keep the gathered part of v in L2)
 * and pipelining (1: the next rows' entries loaded while the current rows
 * gather), timed on this sector: a nonzero lanes_per_row fixes the lanes and times the rest, 0 times
 * every lane count.  The fastest is kept.  *chosen receives the lanes, ms
 * (NULL allowed) the best time of 8, 16 and 32 lanes in that order (-1: not
 * timed); edg_sector_info reports the four choices. */
int edg_sector_tune(edg_sector* s, int lanes_per_row, int* chosen, double* ms);

/* Set the four choices without timing: lanes_per_row 8, 16 or 32,
 * cache_policy 1 or 2, ctas_per_sm 0 (as many as fit) to 32, pipelined 0 or
 * 1.  Results do not depend on them, bit for bit; only the speed does. */
int edg_sector_set_rows(edg_sector* s, int lanes_per_row, int cache_policy, int ctas_per_sm, int pipelined);

/* Same with host buffers: copies v in, applies H, returns w, synchronises.
 * When w is page-locked memory the device can address (cudaHostAlloc,
 * cudaHostRegister) the kernel stores w there directly while it runs;
 * otherwise w comes back by copies, overlapped with the rows still being
 * computed on stored-row sectors.  Either way w holds the same bits.  This is
 * the call the reference's sHv(v, w, ...) adapter makes. */
int edg_hv_host(edg_sector* s, const void* v, void* w, int dtype);

/* w = H v like edg_hv, for callers that must not have the library allocate
 * device memory during the call: applications whose own allocator already
 * holds the device's free memory, and loops where a cudaMalloc or cudaFree
 * would synchronise the device.  No counterpart in the reference (its sHv runs
 * on the host).  Needs stored rows (edg_sector_build_targets) and the sector's
 * device current.  The u = v/norm scratch is a fixed 16 MiB array in the
 * library's device image, held on every GPU that loads it until exit, so
 * n_p may be at most 1,048,576 (EDG_C128) or 2,097,152 (EDG_C64); larger
 * sectors return EDG_ERR_INVALID.  The first call on a device looks the
 * array's address up (cudaGetSymbolAddress); make that first call before any
 * stream capture.  All calls on a device share the array: calls that overlap
 * on the GPU race and must be ordered by the caller. */
int edg_hv_noalloc(edg_sector* s, const void* v, void* w, int dtype, void* stream);

/* W = H V for n_vectors = 2 or 4 vectors at once, interleaved by row: entry i
 * of vector q at index i * n_vectors + q of v and w (device pointers, n_p *
 * n_vectors complex entries each, dtype EDG_C128 or EDG_C64), enqueued on
 * `stream`.  Each row's stored entries are read once and each gathered line
 * serves all the vectors, so the bytes per vector fall with n_vectors; every
 * vector gets the bits edg_hv gives it alone.  Needs stored rows; keeps a
 * scratch of n_p * n_vectors entries on the sector.  No counterpart in the
 * reference (its sHv takes one vector, H_v.cpp:192); it serves block solvers
 * and the FP64 Rayleigh quotients of several Ritz vectors. */
int edg_hv_block(edg_sector* s, const void* v, void* w, int n_vectors, int dtype, void* stream);

/* Number of nonzero off-diagonal bond/chirality targets summed over rows
 * (the nnz_off of the algorithmic byte count). */
int edg_count_offdiag(edg_sector* s, int64_t* nnz_off);

/* Options of the plain (FP64) sector eigensolver. */
typedef struct {
  int n_ev;                 /* eigenvalues wanted: Num_Eigenvalues */
  int iterations;           /* Lanczos steps per cycle: Lanczos_iterations (at most 2048) */
  int ncycles;              /* restarts: Lanczos_ncycles */
  double tol;               /* |E0 - E0_previous| < tol ends the middle cycles: tol */
  uint64_t seed;            /* start vector of eigenvalue k: splitmix64 stream seed + k */
  int64_t dense_threshold;  /* n_p <= this takes the dense path (the reference: 10000); -1: never */
  void (*log_fn)(void* ctx, const char* line); /* optional: the reference's per-iteration log lines */
  void* log_ctx;
} edg_solver_opts;

typedef struct {
  int path;                 /* 0: Lanczos, 1: dense */
  int64_t hv_calls;
  double hv_seconds, ortho_seconds, total_seconds;
} edg_solver_stats;

/* The sector eigensolver of sector_lanczos in FP64 on the GPU.
 * Replaces: lanczos_evecs (lanczos.cpp:133-349) and, for n_p <= dense_threshold,
 * exact_evecs (lanczos.cpp:81-131), dispatched as Lanczos_sector.cpp:105-120.
 * eigs receives *n_eigs values: min(n_ev, n_p) for Lanczos (one per deflation
 * step, so degenerate levels repeat), all n_p for the dense path, ascending
 * for the dense path and in deflation order for Lanczos, as the reference
 * returns them.  evecs (NULL allowed) receives up to evecs_capacity
 * eigenvectors of n_p complex128 entries each, in the same order. */
int edg_solve_plain(edg_sector* s, const edg_solver_opts* opts, double* eigs, int64_t eigs_capacity,
                    int64_t* n_eigs, double* evecs, int64_t evecs_capacity, edg_solver_stats* stats);

/* Options of the mixed-precision solver. */
typedef struct {
  int n_ev;                 /* lowest eigenvalues wanted (at most 32) */
  int iterations;           /* Lanczos steps (2 .. 2000) */
  int reorth_every;         /* > 0: keep every FP32 Krylov vector and reorthogonalise the
                               last two against all of them every reorth_every steps
                               (1 or a few: FP32 vectors lose orthogonality fast);
                               -1: keep every vector, reorthogonalise w against the two
                               latest every step and against all of them only on the
                               steps where Simon's estimates of the lost orthogonality
                               (from alpha/beta alone) pass eps_FP32^(3/4), and the step
                               after (partial reorthogonalisation);
                               0: w reorthogonalised against the two latest vectors only;
                               every vector kept when they fit with room to spare, else
                               as many as fit and the Ritz vectors finished by a second
                               pass from the last stored vector */
  uint64_t seed;            /* start vector: splitmix64 stream */
  int want_vectors;         /* copy the FP64 eigenvectors out */
  int fp64_vectors;         /* 0: FP32 Krylov vectors and H*v (the precision form); 1: the same
                               algorithm with FP64 vectors, FP64 H*v and FP64 arithmetic throughout */
} edg_mixed_opts;

typedef struct {
  int64_t hv_calls;         /* FP32 H*v (both passes) plus one FP64 H*v per Ritz vector */
  double hv_seconds, total_seconds;
  int passes;
  int stored_vectors;       /* Krylov vectors kept in HBM (the rest lived in a ring) */
  int reorth_steps;         /* steps reorthogonalised against all stored vectors */
} edg_mixed_stats;

/* Lowest eigenvalues with FP32 Krylov vectors and FP32 H*v; FP64 for alpha/beta
 * (compensated sums), reorthogonalisation coefficients, the tridiagonal
 * eigensolve (on the device, edg_tridiag_lowest's kernels) and one FP64 H*v
 * per Ritz vector.  Copies of
 * converged eigenvalues that lost orthogonality produces are removed, so each
 * level is returned once.  eigs: FP64 Rayleigh quotients; ritz: the Ritz
 * values of T; residuals: |Hx - eig x|/|x| in FP64; evecs (NULL allowed):
 * n_ev x n_p complex128.  No reference counterpart: the reference keeps every
 * Krylov vector in FP64 (lanczos.cpp:241), which does not fit at N = 36. */
int edg_solve_mixed(edg_sector* s, const edg_mixed_opts* opts, double* eigs, double* ritz, double* residuals,
                    int64_t* n_eigs, double* evecs, edg_mixed_stats* stats);

/* ---- Batched solves: many sectors advanced together ----------------------
 * No counterpart in the reference, which diagonalises one sector at a time
 * (sector_lanczos in a loop over momenta, ED.cpp:120-131).  Each segment is a
 * sector with stored rows and a request; every Lanczos step of all live
 * segments is one replay of a captured CUDA graph.  FP32 Krylov vectors
 * (reorthogonalised every step, or partially: opts.reorth), FP64 alpha/beta, FP64 Rayleigh quotients and
 * residuals as in edg_solve_mixed.  A segment stops when the residual bounds
 * of its wanted Ritz pairs are below tol * max(1, |theta|) (tested every
 * check_every steps) or after max_iterations steps, and is then finished and
 * its memory released.  The caller keeps each sector alive until its result
 * has been polled.  One thread drives a batch. */
typedef struct {
  int tile_rows;      /* rows per CTA tile (0: 1024) */
  int lanes_per_row;  /* lanes per stored row: 8, 16 or 32 (0: 8) */
  int check_every;    /* steps between convergence tests (0: 10) */
  int reorth;         /* 0: reorthogonalise every step; 1: partial reorthogonalisation
                         (only the steps where estimates of the lost orthogonality,
                         from alpha/beta alone, pass eps_FP32^(3/4), and the step after) */
} edg_batch_opts;

typedef struct {
  int n_ev;            /* eigenvalues wanted, 1..32 */
  int max_iterations;  /* Lanczos steps at most, 2..511 */
  double tol;          /* residual-bound tolerance; 0 runs max_iterations steps */
  uint64_t seed;       /* start vector: edg_fill_random's stream, normalised */
  int64_t tag;         /* returned with the result */
} edg_batch_request;

typedef struct {
  int64_t tag;
  int status;          /* EDG_OK or the error that stopped the finish */
  int n_found;         /* distinct levels returned (<= n_ev) */
  int iterations;      /* Lanczos steps taken */
  int converged;       /* 1: stopped by the tolerance, 0: by max_iterations */
  int reorth_steps;    /* steps that reorthogonalised against the stored vectors */
  int reserved;
  double eigs[32];     /* FP64 Rayleigh quotients, ascending */
  double ritz[32];     /* the Ritz values of T they came from */
  double residuals[32];/* |Hx - eig x| / |x| in FP64 */
} edg_batch_result;

typedef struct edg_batch edg_batch;

int edg_batch_create(const edg_batch_opts* opts, edg_batch** out);
int edg_batch_destroy(edg_batch* b);
/* Device bytes a segment of this sector and request takes in a batch (the
 * sector's own basis and stored rows not included). */
int edg_batch_footprint(const edg_sector* s, const edg_batch_request* req, int64_t* bytes);
/* Queue a segment; it starts with the next step.  EDG_ERR_NOMEM if its
 * vectors do not fit (nothing is queued then). */
int edg_batch_add(edg_batch* b, edg_sector* s, const edg_batch_request* req);
/* Run up to n_steps steps of every live segment (fewer when none is left);
 * segments that stop are finished before this returns or at the next call. */
int edg_batch_step(edg_batch* b, int n_steps);
/* Autotuner of the batch kernels: times `steps` steps of the segments added so
 * far (before the batch's first step) for tiles of 256, 1024, 4096 and 16384
 * rows with 8 and 16 lanes per stored row, keeps the fastest for the rest of
 * the batch and returns it (NULL allowed); ms (NULL allowed) receives the 8
 * trial times per step, tiles major.  The segments are then put back at their
 * seeded start, so the results are those of an untuned batch created with the
 * chosen options.  A segment's arithmetic depends on the tile size and the
 * lanes per row (the order of its sums), not on the other segments. */
int edg_batch_tune(edg_batch* b, int steps, int* tile_rows, int* lanes_per_row, double* ms);
/* Withdraw the live segment with this tag: its memory is released now and its
 * result (status EDG_ERR_CANCELLED, no levels) comes back through
 * edg_batch_poll.  The other segments' arithmetic is unchanged.
 * EDG_ERR_INVALID when no live segment has the tag. */
int edg_batch_cancel(edg_batch* b, int64_t tag);
/* Move up to cap finished results into out; *n_out receives how many. */
int edg_batch_poll(edg_batch* b, edg_batch_result* out, int cap, int* n_out);
int edg_batch_info(const edg_batch* b, int* n_active, int64_t* device_bytes, int64_t* steps);
/* Host seconds spent so far, seconds[0..4]: adding segments, stepping (graph
 * replays up to the waits of the convergence tests), finishing segments,
 * releasing their memory, rebuilding the step graph. */
int edg_batch_timers(const edg_batch* b, double* seconds);

/* The k (1..32) lowest eigenpairs of the real symmetric tridiagonal matrix
 * with diagonal d[0..m-1] and off-diagonal e[1..m-1] (e[0] unused), m <= 4096,
 * computed on the current device by the kernels the solvers use for their
 * Lanczos T (bisection on Sturm counts, inverse iteration, FP64).  With
 * copy_filter = 0: eigs[0..k-1] ascending, vecs (NULL allowed) k x m,
 * *n_out = k.  With copy_filter = 1: the Ritz values the mixed-precision
 * solvers keep -- among the lowest 72, a simple eigenvalue that the matrix
 * without its first row and column shares is dropped as a copy made by lost
 * orthogonality, and one value is kept per cluster -- at most k of them,
 * *n_out of them returned.
 * Replaces: zMatrix_Diagonalize_Hermitian -> zheev on T (lanczos.cpp:271-286,
 * Matrix_Functions.cpp:28-48). */
int edg_tridiag_lowest(const double* d, const double* e, int m, int k, int copy_filter, double* eigs, double* vecs,
                       int* n_out);

/* Deterministic complex test vector (splitmix64, entries uniform in [-1,1)^2)
 * written to device memory; the same generator as the test suite's. */
int edg_fill_random(void* dst, int64_t n, int dtype, uint64_t seed, void* stream);

#ifdef __cplusplus
}
#endif
#endif
