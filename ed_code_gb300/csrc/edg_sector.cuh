// One (Sz, kx, ky) sector resident on the GPU, plus the kernel launchers that
// build and apply it.  Host-side only types live here next to the device view.
#pragma once
#include <cuda_runtime.h>

#include <complex>
#include <string>
#include <vector>

#include "../../include/edgpu.h"
#include "edg_core.cuh"

namespace edg {

// Device pointers of one sector, passed by value to every kernel.
struct SectorView {
  const SectorParams* params;
  const uint64_t* reps;
  const uint8_t* lid;
  RankRec* recs;         // Lin-indexed records, only while the basis is built
  const RankRec* vrecs;  // value-indexed rank records
  const uint32_t* Ia;
  const int64_t* Ib;
  const TermGroup* groups;
  const ChTerm* ch;
  const Bowtie* bows;
  const uint8_t* nk;       // torus: rotation minimum of each row value
  const uint16_t* rots;    // torus: rotations reaching it
  const uint64_t* perms;   // walk: n_perm x n_chunks x 256 permutation chunk tables (T1, T2[, T3])
  const uint64_t* binom;   // (kMaxSites+1)^2 binomials
  int n_chunks;
  int n_perm;              // 2, or 3 on a 3-D torus
  int row_bits;            // torus: Lx (table size 2^Lx)
};

// Shared-memory image a kernel stages per CTA (see stage_sector()).
template <typename Real>
struct SmemGroup {
  uint64_t mask;
  Real fac;
  Real Bre[2], Bim[2];
  int16_t a;
  int16_t ch_begin, ch_end;
  int8_t ya, yb;  // torus rows of the two flipped sites
};
template <typename Real>
struct SmemCh {
  Real Are[2], Aim[2];
  int z;
};

struct DeviceBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
};

struct Sector {
  int device = 0;
  SectorParams P{};
  SectorView V{};
  // device allocations
  SectorParams* dP = nullptr;
  uint64_t* reps = nullptr;
  uint8_t* lid = nullptr;
  RankRec* recs = nullptr;
  RankRec* vrecs = nullptr;
  uint32_t* Ia = nullptr;
  int64_t* Ib = nullptr;
  TermGroup* groups = nullptr;
  ChTerm* ch = nullptr;
  Bowtie* bows = nullptr;
  uint8_t* nk = nullptr;
  uint16_t* rots = nullptr;
  uint64_t* perms = nullptr;
  uint64_t* binom = nullptr;
  size_t device_bytes = 0;
  // host copies used by the adapters
  std::vector<int> T1, T2, T3;  // T3 empty in 2-D
  double lambda = 1, Ch = 0, ChCh = 0;
  // scratch kept for host-buffer H*v calls
  DeviceBuffer host_in, host_out;
  cudaStream_t stream = nullptr;
  // edg_hv_host: a second stream and per-chunk events to copy finished rows
  // of w back while the next rows are computed
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t chunk_done[8] = {};
  // Lanczos work area (allocated on first use)
  DeviceBuffer lz_work;
  // stored targets (targets.cu): CSR rows of (column, value id)
  uint64_t* row_ptr = nullptr;  // n_p + 1
  uint32_t* col = nullptr;      // column, or column | value id << pack_cb
  uint16_t* vid = nullptr;      // value ids; null when the entries are packed
  int pack_cb = 0;              // column bits of a packed entry (0: split arrays)
  double* ezz = nullptr;        // diagonal of each row
  double2* vtab64 = nullptr;    // value table: pair coefficient x phase class
  float2* vtab32 = nullptr;
  int n_vals = 0;
  DeviceBuffer ubuf;            // u = v / norm scratch
  DeviceBuffer ublk;            // the same for edg_hv_block's interleaved vectors
  size_t targets_bytes = 0;
  int csr_lpr = 16;             // lanes per CSR row (8, 16 or 32): edg_sector_tune
  int csr_pol = 1;              // cache policy of the CSR loads (1 or 2): edg_sector_tune
  int csr_cps = 0;              // CTAs per SM of the CSR kernel (0: as many as fit): edg_sector_tune
  int csr_pipe = 0;             // 1: the CSR kernel loads the next rows' entries ahead: edg_sector_tune
};

// basis.cu
cudaError_t build_basis(Sector& S, std::string& err);
cudaError_t export_walk_tables(const Sector& S, int64_t* rep_loc_dev, int32_t* g_dev, cudaStream_t st);
// hv.cu
cudaError_t launch_hv(const Sector& S, const void* v, void* w, bool fp64, cudaStream_t st);
cudaError_t launch_hv_generic(const Sector& S, const void* v, void* w, bool fp64, cudaStream_t st);
// dense.cu: exact_evecs on the device (all eigenvalues, the first evecs_cap eigenvectors)
int solve_dense_device(Sector& S, double* eigs, int64_t cap, int64_t* n_out, double* evecs, int64_t evecs_cap,
                       edg_solver_stats* stats);
// lanczos.cu
int solve_plain(Sector& S, const edg_solver_opts& o, double* eigs, int64_t cap, int64_t* n_out, double* evecs,
                int64_t evecs_cap, edg_solver_stats* stats);
int solve_mixed(Sector& S, const edg_mixed_opts& o, double* eigs, double* ritz, double* resid, int64_t* n_out,
                double* evecs, edg_mixed_stats* stats);
// lanczos_mixed.cu: the end of a mixed-precision Lanczos run, shared by the
// single-sector solver and the batch: FP64 Ritz vectors from the host-chosen
// Ritz coefficients (lanczos_common.cuh), and one FP64 H*v per Ritz vector
// for its Rayleigh quotient and residual.  Device scratch grows on demand.
struct MixedFinish {
  double* y = nullptr;    // Ritz coefficients, na x m
  double2 *X = nullptr, *HX = nullptr;
  double* part = nullptr;
  double* res = nullptr;  // 4 doubles per Ritz vector
  size_t y_bytes = 0, hx_bytes = 0, x_bytes = 0, res_bytes = 0;
  ~MixedFinish();
  cudaError_t reserve(int64_t n, int m, int n_res);
  cudaError_t reserve_x(int64_t n, int na);
  // X_q = sum_{j < cnt} y_q[j] V_j from the first cnt stored FP32 vectors
  // (y_q holds m coefficients, from ycoef or else this object's y; the
  // vectors' leading dimension is n)
  int ritz_stored(cudaStream_t st, const float2* V, int64_t n, int m, int na, int cnt,
                  const double* ycoef = nullptr);
  int ritz_stored(cudaStream_t st, const double2* V, int64_t n, int m, int na, int cnt,
                  const double* ycoef = nullptr);
  // the same, written to dst (na x n) instead of X
  int ritz_stored_to(cudaStream_t st, const float2* V, int64_t n, int m, int na, int cnt, const double* ycoef,
                     double2* dst);
  // res[4q..4q+3] = |x_q|^2, <x_q|H x_q>, Rayleigh quotient, residual, queued
  // on st (no wait)
  cudaError_t rayleigh_async(Sector& S, cudaStream_t st, int64_t n, int na, double* res_dev);
};
void pick_levels(const std::vector<double>& rr, const std::vector<double>& th, const std::vector<int>& acc_h, int na,
                 int want, double* eigs, double* ritz, double* resid, std::vector<int>& keep);
cudaError_t count_offdiag(const Sector& S, unsigned long long* nnz_dev, cudaStream_t st);
int build_targets(Sector& S, int64_t max_bytes, std::string& err);
void free_targets(Sector& S);
cudaError_t launch_hv_stored(const Sector& S, const void* v, void* w, bool fp64, cudaStream_t st);
// hv_block.cu: W = H V for nv = 2 or 4 vectors interleaved by row, u the n_p x nv scratch
cudaError_t launch_hv_block(const Sector& S, const void* v, void* w, int nv, bool fp64, void* u, cudaStream_t st);
// stored rows in row order: rows [r0, r1) of H*v, with the u = v/norm pass first when with_u
cudaError_t launch_hv_rows(const Sector& S, const void* v, void* w, bool fp64, int64_t r0, int64_t r1, bool with_u,
                           cudaStream_t st);
// stored rows: u = v / norm and v_dst = v from a v_src the device reads in
// place (mapped page-locked host memory)
cudaError_t launch_u_in(const Sector& S, const void* v_src, void* v_dst, bool fp64, cudaStream_t st);
int tune_rows(Sector& S, int lpr, int* chosen, double* ms_out);
int hv_grid_blocks(bool fp64, bool torus, bool chch);

}  // namespace edg
