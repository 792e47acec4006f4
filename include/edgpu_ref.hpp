// C++ drop-in: the reference's own sector-solver signatures, implemented on
// top of the C ABI (edgpu.h) by libedgpu_ref.so.
//
// A program written against hiteshjc/ED_Code -- in particular its driver
// ED.cpp and parser read_input_file.cpp, unchanged -- links against
// libedgpu_ref.so instead of the reference's Lanczos_sector.o, ARPACK_sector.o
// and H_v.o.  The term-list structs must be the reference's (global.h:25-40):
// their names and layouts are part of the C++ signatures (and of the mangled
// symbol names), so they are declared here with the same members.
#ifndef EDGPU_REF_HPP
#define EDGPU_REF_HPP

#include <stdint.h>

#include <complex>
#include <fstream>
#include <string>
#include <vector>

struct coordinates {  // global.h:25-30
  int x, y;
  double J;
  std::complex<double> expphase;
};
struct triangles {  // global.h:32-35
  int i, j, k;
  std::complex<double> expphase;
};
struct bowties {  // global.h:37-40
  int x, y, z;
  int p, q, r;
};

// Lanczos_sector.h:11-31: build the (Sz, kx, ky) sector, diagonalise it
// (dense below n_p = 10000, deflated Lanczos above, Lanczos_sector.cpp:105-120),
// print the Energies table to `outfile`, optionally write eigenvector files.
void sector_lanczos(int& kx, int& ky, double& cSz, int& n_spins, double& lambda, double& J2,
                    std::vector<coordinates>& adj_list, double& Ch, std::vector<triangles>& ch_list, double& ChCh,
                    std::vector<bowties>& chch_list, std::vector<int>& T1, std::vector<int>& T2, int& n_sec_ev,
                    bool& find_ev, bool& unwrap_peigvec, std::string& filepath_EV, double& tol, int& iterations,
                    int& ncycles, std::ofstream& outfile);

// Lanczos_sector.h:33-55 (3-D tori).  Declared so the reference driver links;
// 3-D sectors are not implemented on the GPU and end with a message and exit(1).
void sector_lanczos(int& kx, int& ky, int& kz, double& cSz, int& n_spins, double& lambda, double& J2,
                    std::vector<coordinates>& adj_list, double& Ch, std::vector<triangles>& ch_list, double& ChCh,
                    std::vector<bowties>& chch_list, std::vector<int>& T1, std::vector<int>& T2, std::vector<int>& T3,
                    int& n_sec_ev, bool& find_ev, bool& unwrap_peigvec, std::string& filepath_EV, double& tol,
                    int& iterations, int& ncycles, std::ofstream& outfile);

// ARPACK_sector.h:67-86: the same sector solve, called with an iteration cap
// instead of (iterations, ncycles); ARPACK is replaced by the GPU Lanczos.
void sector_eigs_eigvecs(int& kx, int& ky, double& cSz, int& n_spins, double& lambda, double& J2,
                         std::vector<coordinates>& adj_list, double& Ch, std::vector<triangles>& ch_list,
                         double& ChCh, std::vector<bowties>& chch_list, std::vector<int>& T1, std::vector<int>& T2,
                         int& n_sec_ev, bool& find_ev, bool& unwrap_peigvec, std::string& filepath_EV, double& tol,
                         int& maxiter, std::ofstream& outfile);

// H_v.h:36-57: w = H v for host vectors in the reference's momentum basis.
// The basis tables the reference passes (norm, rep_loc, state_ph, Ia, Ib)
// are not read: the GPU keeps its own copy of the sector, built once and
// reused while the term lists, translations and momentum stay the same, and
// checked against pblock_states.  kx, ky are the momenta in radians as the
// reference's callers pass them (lanczos.cpp:232).
void sHv(std::complex<double>* v, std::complex<double>* w, const std::vector<int64_t>& pblock_states,
         const std::vector<double>& norm, const std::vector<double>& norm_inv, const std::vector<int64_t>& rep_loc,
         const std::vector<std::complex<double> >& state_ph, const double& lambda,
         const std::vector<coordinates>& adj_list, const double& Ch, const std::vector<triangles>& ch_list,
         const double& ChCh, const std::vector<bowties>& chch_list, const int& n_sites, const std::vector<int64_t>& Ia,
         const std::vector<int64_t>& Ib, const int& bits_right, const std::vector<int>& T1, const std::vector<int>& T2,
         const double& kx, const double& ky, std::ofstream& outfile);

#endif
