// libedgpu_ref.so: the reference's C++ sector-solver surface (include/edgpu_ref.hpp)
// over the C ABI (include/edgpu.h).  Output lines follow Lanczos_sector.cpp:
// 68-197 and ARPACK_sector.cpp:309-398 so logs and eigenvector files read the
// same; error paths end with the reference's messages and exit(1).
#include <sys/time.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "edgpu.h"
#include "edgpu_ref.hpp"

namespace {

using cplx = std::complex<double>;
constexpr double kPi = 3.14159265358979323846;  // M_PI as global.h:17 defines it

double now_seconds() {
  timeval tp;
  gettimeofday(&tp, nullptr);
  return tp.tv_sec + tp.tv_usec / 1e6;
}

struct ModelArrays {
  std::vector<edg_bond> bonds;
  std::vector<edg_triangle> tris;
  std::vector<edg_bowtie> bows;
  edg_model m{};
};

void fill_model(ModelArrays& a, int n_sites, const std::vector<int>& T1, const std::vector<int>& T2, double lambda,
                const std::vector<coordinates>& adj, double Ch, const std::vector<triangles>& chl, double ChCh,
                const std::vector<bowties>& chch) {
  a.bonds.clear();
  for (const coordinates& c : adj) a.bonds.push_back(edg_bond{c.x, c.y, c.J, c.expphase.real(), c.expphase.imag()});
  a.tris.clear();
  for (const triangles& t : chl) a.tris.push_back(edg_triangle{t.i, t.j, t.k, t.expphase.real(), t.expphase.imag()});
  a.bows.clear();
  for (const bowties& b : chch) a.bows.push_back(edg_bowtie{b.x, b.y, b.z, b.p, b.q, b.r});
  a.m.n_sites = n_sites;
  a.m.T1 = T1.data();
  a.m.T2 = T2.data();
  a.m.lambda = lambda;
  a.m.bonds = a.bonds.data();
  a.m.n_bonds = (int)a.bonds.size();
  a.m.Ch = Ch;
  a.m.triangles = a.tris.data();
  a.m.n_triangles = (int)a.tris.size();
  a.m.ChCh = ChCh;
  a.m.bowties = a.bows.data();
  a.m.n_bowties = (int)a.bows.size();
}

[[noreturn]] void die(std::ofstream& out, const std::string& msg) {
  out << msg;
  out.flush();
  std::exit(1);
}

void log_to_stream(void* ctx, const char* line) { *static_cast<std::ofstream*>(ctx) << line << "\n"; }

uint64_t translate(uint64_t s, const std::vector<int>& T) {
  uint64_t out = 0;
  for (size_t i = 0; i < T.size(); ++i)
    if ((s >> i) & 1u) out |= 1ull << T[i];
  return out;
}

// Unwrap_pState (Momentum_Basis.cpp:978-1037; 3-D :901-976): expand a
// momentum eigenvector into the fixed-Sz basis by walking each
// representative's orbit with the reference's walk order and phases, merging
// repeated states, dropping coefficients below 1e-8 and sorting by state.
// T3 == nullptr is the 2-D walk.
std::vector<std::pair<int64_t, cplx>> unwrap(const std::vector<cplx>& coeff, const std::vector<int64_t>& reps,
                                             const std::vector<double>& norm, double px, double py, double pz, int L1,
                                             int L2, int L3, const std::vector<int>& T1, const std::vector<int>& T2,
                                             const std::vector<int>* T3) {
  std::vector<std::pair<int64_t, cplx>> out;
  const cplx ex = std::exp(cplx(0.0, -px)), ey = std::exp(cplx(0.0, -py)), ez = std::exp(cplx(0.0, -pz));
  for (size_t i = 0; i < reps.size(); ++i) {
    std::vector<std::pair<int64_t, cplx>> loc;
    auto add = [&](int64_t id, cplx c) {
      for (auto& e : loc)
        if (e.first == id) {
          e.second += c;
          return;
        }
      loc.push_back({id, c});
    };
    uint64_t v = (uint64_t)reps[i];
    cplx ph(1.0, 0.0);
    add((int64_t)v, coeff[i] / norm[i]);
    for (int x = 0; x < L1; ++x) {
      if (x > 0) {
        v = translate(v, T1);
        ph = ph * ex;
        add((int64_t)v, coeff[i] * ph / norm[i]);
      }
      for (int y = 0; y < L2; ++y) {
        if (y > 0) {
          v = translate(v, T2);
          ph = ph * ey;
          add((int64_t)v, coeff[i] * ph / norm[i]);
        }
        for (int z = 1; z < L3 && T3; ++z) {
          v = translate(v, *T3);
          ph = ph * ez;
          add((int64_t)v, coeff[i] * ph / norm[i]);
        }
      }
    }
    for (auto& e : loc)
      if (std::abs(e.second.real()) > 1e-8 || std::abs(e.second.imag()) > 1e-8) out.push_back(e);
  }
  std::stable_sort(out.begin(), out.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
  return out;
}

std::string index_string(int i) {
  std::stringstream ss;
  ss << i;
  return ss.str();
}

// The common body of sector_lanczos and sector_eigs_eigvecs.
void solve_sector(int kx, int ky, double cSz, int n_spins, double lambda, double J2,
                  const std::vector<coordinates>& adj_list, double Ch, const std::vector<triangles>& ch_list,
                  double ChCh, const std::vector<bowties>& chch_list, const std::vector<int>& T1,
                  const std::vector<int>& T2, int n_sec_ev, bool find_ev, bool unwrap_peigvec,
                  const std::string& filepath_EV, double tol, int iterations, int ncycles, std::ofstream& outfile,
                  const std::vector<int>* T3 = nullptr, int kz = 0) {
  // T3 != nullptr: the 3-D overload (Lanczos_sector.cpp:201-369)
  int n_ones = int(cSz + n_spins / 2 + 1.0e-6);  // Lanczos_sector.cpp:45-46
  if ((int)T1.size() != n_spins || (int)T2.size() != n_spins || (T3 && (int)T3->size() != n_spins))
    die(outfile, "\nERROR: input T1 != T2\n");
  ModelArrays ma;
  fill_model(ma, n_spins, T1, T2, lambda, adj_list, Ch, ch_list, ChCh, chch_list);
  if (T3) ma.m.T3 = T3->data();
  const double Sz = 0.5 * n_ones - 0.5 * (n_spins - n_ones);
  outfile << "\n--------------------------------------------------------------------\n";
  double t_states = now_seconds();
  outfile.flush();
  edg_sector* sec = nullptr;
  int rc = T3 ? edg_sector_create3(&ma.m, n_ones, kx, ky, kz, &sec) : edg_sector_create(&ma.m, n_ones, kx, ky, &sec);
  if (rc == EDG_ERR_MOMENTUM) die(outfile, "\nInvalid kx or ky\n");
  edg_sector_info info{};
  if (rc == EDG_OK) edg_sector_get_info(sec, &info);
  t_states = now_seconds() - t_states;
  if (rc != EDG_OK && rc != EDG_ERR_EMPTY) die(outfile, std::string("\nERROR: ") + edg_last_error() + "\n");
  // L1, L2 as the reference's LxLy (Momentum_Basis.cpp:19-36)
  int L1 = 0, L2 = 0, L3 = 1;
  {
    int s = 0;
    do { s = T1[s]; ++L1; } while (s != 0);
    s = 0;
    do { s = T2[s]; ++L2; } while (s != 0);
    if (T3) {
      L3 = 0;
      s = 0;
      do { s = (*T3)[s]; ++L3; } while (s != 0);
    }
  }
  const double px = 2 * kx * kPi / L1, py = 2 * ky * kPi / L2, pz = 2 * kz * kPi / L3;
  const int64_t n_p = (rc == EDG_OK) ? info.n_p : 0;
  int64_t n_configs = 1;
  for (int i = 1; i <= n_ones; ++i) n_configs = n_configs * (n_spins - n_ones + i) / i;
  outfile << std::endl << "Total size of all states/rep loc vector " << n_configs << std::endl;
  if (T3)
    outfile << " SECTOR : " << Sz << "\t(" << px << "," << py << "," << pz << ")\t" << n_p << std::endl;
  else
    outfile << " SECTOR : " << Sz << "\t(" << px << "," << py << ")\t" << n_p << std::endl;
  outfile << "Time to construct pStates\t " << t_states / 60.0 << " minutes" << std::endl;
  if (n_p == 0) die(outfile, "\nNo states in psector\n");
  outfile << "------------------------------------------------------------------" << std::endl;

  double lanczos_time = now_seconds();
  edg_solver_opts o{};
  o.n_ev = n_sec_ev;
  o.iterations = iterations;
  o.ncycles = ncycles;
  o.tol = tol;
  o.seed = 0;
  // the 2-D driver diagonalises sectors up to 10000 states densely
  // (Lanczos_sector.cpp:105); the 3-D one always runs lanczos_evecs (:285)
  o.dense_threshold = T3 ? -1 : 10000;
  o.log_fn = log_to_stream;
  o.log_ctx = &outfile;
  const bool dense = o.dense_threshold >= 0 && n_p <= o.dense_threshold;
  const int64_t cap = dense ? n_p : std::min<int64_t>(n_sec_ev, n_p);
  std::vector<double> eigs(std::max<int64_t>(cap, 1));
  const int64_t nvec = find_ev ? std::min<int64_t>(n_sec_ev, dense ? n_p : cap) : 0;
  std::vector<cplx> vecs((size_t)(nvec * n_p));
  int64_t n_eigs = 0;
  edg_solver_stats st{};
  if (!dense) {
    // the Lanczos path's H*v on stored rows with the row kernel timed on this
    // sector; sectors whose rows do not fit (EDG_ERR_NOMEM) or that have ChCh
    // terms (EDG_ERR_UNSUPPORTED) keep the matrix-free kernel
    if (edg_sector_build_targets(sec, 0) == EDG_OK) edg_sector_tune(sec, 0, nullptr, nullptr);
  }
  rc = edg_solve_plain(sec, &o, eigs.data(), cap, &n_eigs, nvec ? reinterpret_cast<double*>(vecs.data()) : nullptr,
                       nvec, &st);
  if (rc != EDG_OK) die(outfile, std::string("\nERROR: ") + edg_last_error() + "\n");
  if (st.path == 0) {
    outfile << "\n\n--------------------------------------------------\n";
    outfile << "\n Lanczos SUMMARY \n" << std::endl;
    outfile << " Hv calls\t\t\t" << st.hv_calls << std::endl;
    outfile << " Hv total time \t\t\t" << st.hv_seconds / 60.0 << " minutes" << std::endl;
    outfile << " Orthogonalize total time \t" << st.ortho_seconds / 60.0 << " minutes" << std::endl;
  } else {
    outfile << "\n\n--------------------------------------------------\n";
    outfile << "\n EXACT SUMMARY \n" << std::endl;
  }
  outfile << "-----------------------------------------------------------" << std::endl;
  outfile << "-----------------------------------------------------------" << std::endl;
  outfile << " Wall clock for Lanczos " << (now_seconds() - lanczos_time) / 60.0 << std::endl;
  outfile << "pblock_eigs.size() = " << n_eigs << std::endl;
  if (T3) {
    outfile << "\n\nEnergies\t\tEnergies/site\t\tSz\tkx\tky\tkz\tJz\tJ2\n\n";
    outfile.flush();
    for (int64_t i = 0; i < n_eigs; ++i)
      outfile << std::fixed << std::setprecision(15) << eigs[i] << "\t" << eigs[i] / double(n_spins) << "\t"
              << std::setprecision(3) << Sz << "\t" << px << "\t" << py << "\t" << pz << "\t" << lambda << "\t"
              << J2 << "\n";
    outfile.flush();
    outfile << " find_ev = " << find_ev << std::endl;
  } else {
    outfile << "\n\nEnergies\t\tEnergies/site\t\tSz\tkx\tky\tJz\tJ2\n\n";
    outfile.flush();
    for (int64_t i = 0; i < n_eigs; ++i)
      outfile << std::fixed << std::setprecision(15) << eigs[i] << "\t" << eigs[i] / double(n_spins) << "\t"
              << std::setprecision(3) << Sz << "\t" << px << "\t" << py << "\t" << lambda << "\t" << J2 << "\n";
  }
  outfile.flush();

  if (find_ev) {
    std::vector<int64_t> states(n_p);
    std::vector<double> norm(n_p), norm_inv(n_p);
    edg_sector_copy_basis(sec, states.data(), norm.data(), norm_inv.data());
    for (int iib = 0; iib < std::min<int64_t>(n_sec_ev, n_eigs); ++iib) {
      const std::string path =
          filepath_EV + (unwrap_peigvec ? "_EV" : "_pEV") + index_string(iib) + ".txt";  // Lanczos_sector.cpp:152-157
      std::ofstream ov(path.c_str());
      ov << "\n Eigenvector for state \n";
      if (T3) {
        ov << "Sz\t(kx,ky,kz)\tJz/lambda\n";
        ov << Sz << "\t(" << kx << "," << ky << "," << kz << ")\t" << lambda << std::endl;
      } else {
        ov << "Sz\t(kx,ky)\tJz/lambda\n";
        ov << Sz << "\t(" << kx << "," << ky << ")\t" << lambda << std::endl;
      }
      ov << "\n\n-------------------------------------------";
      ov << "\nState Energy " << cplx(eigs[iib], 0.0) << std::endl;
      std::vector<cplx> c(vecs.begin() + (size_t)iib * n_p, vecs.begin() + (size_t)(iib + 1) * n_p);
      if (unwrap_peigvec) {
        auto psi = unwrap(c, states, norm, px, py, pz, L1, L2, L3, T1, T2, T3);
        ov << "\nEIGENVECTOR\n";
        for (const auto& e : psi) ov << e.first << "\t" << std::fixed << std::setprecision(15) << e.second << std::endl;
      } else {
        ov << "\nMomentum EIGENVECTOR\n";
        if (T3) {
          ov << "\nnp \t\t px \t\tpy \t\tpz\n";
          ov << n_p << "\t\t" << px << "\t\t" << py << "\t\t" << pz << std::endl;
        } else {
          ov << "\nnp \t\t px \t\tpy\n";
          ov << n_p << "\t\t" << px << "\t\t" << py << std::endl;
        }
        ov << "\n\npblock_states \t\t Norm \t\t\t v_coeff\n\n";
        for (int64_t jb = 0; jb < n_p; ++jb)
          ov << states[jb] << "\t\t\t" << norm[jb] << "\t\t\t" << std::fixed << std::setprecision(15) << c[jb]
             << std::endl;
      }
    }
  }
  edg_sector_destroy(sec);
}

// sHv keeps the last sector it built; a call with different inputs rebuilds.
struct HvCache {
  std::vector<int> T1, T2;
  std::vector<double> key;  // every number the sector depends on
  int n_ones = -1, kx = -1, ky = -1;
  edg_sector* sec = nullptr;
  int64_t n_p = 0;
  ~HvCache() {
    if (sec) edg_sector_destroy(sec);
  }
};
HvCache g_hv;

}  // namespace

void sector_lanczos(int& kx, int& ky, double& cSz, int& n_spins, double& lambda, double& J2,
                    std::vector<coordinates>& adj_list, double& Ch, std::vector<triangles>& ch_list, double& ChCh,
                    std::vector<bowties>& chch_list, std::vector<int>& T1, std::vector<int>& T2, int& n_sec_ev,
                    bool& find_ev, bool& unwrap_peigvec, std::string& filepath_EV, double& tol, int& iterations,
                    int& ncycles, std::ofstream& outfile) {
  solve_sector(kx, ky, cSz, n_spins, lambda, J2, adj_list, Ch, ch_list, ChCh, chch_list, T1, T2, n_sec_ev, find_ev,
               unwrap_peigvec, filepath_EV, tol, iterations, ncycles, outfile);
}

void sector_lanczos(int& kx, int& ky, int& kz, double& cSz, int& n_spins, double& lambda, double& J2,
                    std::vector<coordinates>& adj_list, double& Ch, std::vector<triangles>& ch_list, double& ChCh,
                    std::vector<bowties>& chch_list, std::vector<int>& T1, std::vector<int>& T2, std::vector<int>& T3,
                    int& n_sec_ev, bool& find_ev, bool& unwrap_peigvec, std::string& filepath_EV, double& tol,
                    int& iterations, int& ncycles, std::ofstream& outfile) {
  solve_sector(kx, ky, cSz, n_spins, lambda, J2, adj_list, Ch, ch_list, ChCh, chch_list, T1, T2, n_sec_ev, find_ev,
               unwrap_peigvec, filepath_EV, tol, iterations, ncycles, outfile, &T3, kz);
}

void sector_eigs_eigvecs(int& kx, int& ky, double& cSz, int& n_spins, double& lambda, double& J2,
                         std::vector<coordinates>& adj_list, double& Ch, std::vector<triangles>& ch_list,
                         double& ChCh, std::vector<bowties>& chch_list, std::vector<int>& T1, std::vector<int>& T2,
                         int& n_sec_ev, bool& find_ev, bool& unwrap_peigvec, std::string& filepath_EV, double& tol,
                         int& maxiter, std::ofstream& outfile) {
  // ARPACK's implicitly restarted Arnoldi is replaced by the deflated Lanczos:
  // maxiter bounds the Lanczos steps per cycle, with the reference driver's
  // default of 10 cycles (ED.cpp:28).
  solve_sector(kx, ky, cSz, n_spins, lambda, J2, adj_list, Ch, ch_list, ChCh, chch_list, T1, T2, n_sec_ev, find_ev,
               unwrap_peigvec, filepath_EV, tol, std::max(1, std::min(maxiter, 300)), 10, outfile);
}

void sHv(std::complex<double>* v, std::complex<double>* w, const std::vector<int64_t>& pblock_states,
         const std::vector<double>& /*norm*/, const std::vector<double>& /*norm_inv*/,
         const std::vector<int64_t>& /*rep_loc*/, const std::vector<std::complex<double> >& /*state_ph*/,
         const double& lambda, const std::vector<coordinates>& adj_list, const double& Ch,
         const std::vector<triangles>& ch_list, const double& ChCh, const std::vector<bowties>& chch_list,
         const int& n_sites, const std::vector<int64_t>& /*Ia*/, const std::vector<int64_t>& /*Ib*/,
         const int& /*bits_right*/, const std::vector<int>& T1, const std::vector<int>& T2, const double& kx,
         const double& ky, std::ofstream& outfile) {
  if (pblock_states.empty()) return;
  int L1 = 0, L2 = 0;
  {
    int s = 0;
    do { s = T1[s]; ++L1; } while (s != 0);
    s = 0;
    do { s = T2[s]; ++L2; } while (s != 0);
  }
  const int ikx = (int)std::lround(kx * L1 / (2 * kPi)), iky = (int)std::lround(ky * L2 / (2 * kPi));
  const int n_ones = __builtin_popcountll((unsigned long long)pblock_states[0]);
  std::vector<double> key = {lambda, Ch, ChCh, (double)n_sites};
  for (const coordinates& c : adj_list) key.insert(key.end(), {(double)c.x, (double)c.y, c.J, c.expphase.real(), c.expphase.imag()});
  for (const triangles& t : ch_list) key.insert(key.end(), {(double)t.i, (double)t.j, (double)t.k, t.expphase.real(), t.expphase.imag()});
  for (const bowties& b : chch_list) key.insert(key.end(), {(double)b.x, (double)b.y, (double)b.z, (double)b.p, (double)b.q, (double)b.r});
  if (!g_hv.sec || g_hv.T1 != T1 || g_hv.T2 != T2 || g_hv.key != key || g_hv.n_ones != n_ones || g_hv.kx != ikx ||
      g_hv.ky != iky) {
    if (g_hv.sec) edg_sector_destroy(g_hv.sec);
    g_hv.sec = nullptr;
    ModelArrays ma;
    fill_model(ma, n_sites, T1, T2, lambda, adj_list, Ch, ch_list, ChCh, chch_list);
    if (edg_sector_create(&ma.m, n_ones, ikx, iky, &g_hv.sec) != EDG_OK)
      die(outfile, std::string("\nERROR: ") + edg_last_error() + "\n");
    edg_sector_info info{};
    edg_sector_get_info(g_hv.sec, &info);
    g_hv.n_p = info.n_p;
    // the caller's basis must be this sector's (same representatives, same order)
    std::vector<int64_t> states(info.n_p);
    edg_sector_copy_basis(g_hv.sec, states.data(), nullptr, nullptr);
    if (states != pblock_states) die(outfile, "\nERROR: sHv: pblock_states differ from the GPU sector's basis\n");
    g_hv.T1 = T1;
    g_hv.T2 = T2;
    g_hv.key = key;
    g_hv.n_ones = n_ones;
    g_hv.kx = ikx;
    g_hv.ky = iky;
  }
  if ((int64_t)pblock_states.size() != g_hv.n_p) die(outfile, "\nERROR: sHv: basis size mismatch\n");
  if (edg_hv_host(g_hv.sec, v, w, EDG_C128) != EDG_OK) die(outfile, std::string("\nERROR: ") + edg_last_error() + "\n");
}
