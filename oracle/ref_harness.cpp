// Dump harness for the reference implementation (test infrastructure only).
//
// Links the reference's own objects (everything but ED.o), parses a reference
// input file with the reference parser (read_input_file.cpp:110
// ED_2D_Lattice_Geometry), builds the momentum basis with the reference
// pConstruct_States (Momentum_Basis.cpp:645) and applies the reference sHv
// (H_v.cpp:192) to caller-supplied vectors.  Everything is written as raw
// little-endian arrays into an output directory:
//
//   meta.txt          n_sites n_ones L1 L2 kx ky n_p n_configs bits_right t_basis [L3 kz]
//   states.i64        pblock_states            (n_p)
//   norm.f64          norm                     (n_p)
//   rep_loc.i64       rep_loc                  (n_configs)      [tables mode]
//   state_ph.c128     state_ph                 (n_configs)      [tables mode]
//   Ia.i64, Ib.i64    Lin tables               (2^half)         [tables mode]
//   w<k>.c128         sHv(v<k>)                                 [if v<k>.c128 given]
//   terms.txt         adj_list / ch_list / chch_list / T1 / T2 as parsed
//
// An input file with a T3= line is read with ED_3D_Lattice_Geometry
// (read_input_file.cpp:443) and goes through the 3-D pConstruct_States
// (Momentum_Basis.cpp:781) and sHv (H_v.cpp:360); meta.txt then ends with L3 kz.
//
//   T.f64             Lanczos T matrix of m steps from vT.c128         [if tsteps > 0]
//                     (alpha as m complex pairs, then beta_0..beta_m)
//
// usage: ref_harness <input-file> <out-dir> [tables|notables] [nvec] [reps] [tsteps]
// The v<k>.c128 inputs are read from <out-dir>.  With reps > 1 each sHv call
// is repeated and the mean wall time per call is written to hv_time.txt.
// With tsteps > 0 the reference's three-term recurrence of its first Lanczos
// cycle (lanczos.cpp:196-254: reference sHv, zdotc, zaxpyk, zscalk, normalize;
// no reorthogonalisation) runs tsteps steps from vT.c128 and T is dumped.
#include <sys/stat.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include "H_v.h"
#include "Lanczos_sector.h"
#include "Momentum_Basis.h"
#include "read_input_file.h"

// The reference's BLAS-1 helpers (lanczos.cpp:8-55), linked from lanczos.o.
std::complex<double> zdotc(const int64_t& size, const std::vector<std::complex<double>>& v1,
                           const std::vector<std::complex<double>>& v2);
void zaxpyk(const int64_t size, std::complex<double> a, std::vector<std::complex<double>>& x,
            std::vector<std::complex<double>>& y);
void zscalk(const int64_t size, std::complex<double> a, std::vector<std::complex<double>>& x);
void normalize(std::vector<std::complex<double>>& v);

template <class T>
static void dump(const std::string& path, const std::vector<T>& a) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) { std::perror(path.c_str()); std::exit(2); }
  if (!a.empty()) std::fwrite(a.data(), sizeof(T), a.size(), f);
  std::fclose(f);
}

static bool read_vec(const std::string& path, std::vector<std::complex<double>>& v, int64_t n) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  v.resize(n);
  size_t got = std::fread(v.data(), sizeof(std::complex<double>), n, f);
  std::fclose(f);
  if ((int64_t)got != n) { std::fprintf(stderr, "short vector %s\n", path.c_str()); std::exit(2); }
  return true;
}

int main(int argc, char** argv) {
  if (argc < 3) { std::fprintf(stderr, "usage: %s input outdir [tables|notables] [nvec] [reps]\n", argv[0]); return 1; }
  std::string in = argv[1], out = argv[2];
  bool tables = argc < 4 || std::string(argv[3]) == "tables";
  int nvec = argc > 4 ? std::atoi(argv[4]) : 0;
  int reps = argc > 5 ? std::atoi(argv[5]) : 1;
  int tsteps = argc > 6 ? std::atoi(argv[6]) : 0;
  mkdir(out.c_str(), 0755);
  std::ofstream log((out + "/ref_log.txt").c_str());

  double tol = 1e-11; bool use_arpack = false; int iters = 100, ncyc = 10;
  routine_parameters(in, tol, use_arpack, iters, ncyc);
  int n_spins = 0; double Jz = 1, J1 = 1, J2 = 0, Ch = 0, ChCh = 0;
  std::vector<coordinates> adj; std::vector<triangles> chl; std::vector<bowties> chch;
  std::vector<int> T1, T2, cut; double sSz = -1; int kx = -1, ky = -1;
  bool all_s = false, psec = false, find_v = false, unwrap = true; double szs = -1;
  int nev = 2; std::string vpath;
  bool three_d = false;
  {
    std::ifstream f(in.c_str());
    std::string line;
    while (std::getline(f, line))
      if (line.compare(0, 3, "T3=") == 0) three_d = true;
  }
  std::vector<int> T3;
  int kz = 0;
  if (three_d)
    ED_3D_Lattice_Geometry(in, n_spins, Jz, J1, J2, adj, Ch, chl, ChCh, chch, T1, T2, T3, cut, sSz, kx, ky, kz, all_s,
                           szs, psec, nev, find_v, unwrap, vpath, log);
  else
    ED_2D_Lattice_Geometry(in, n_spins, Jz, J1, J2, adj, Ch, chl, ChCh, chch, T1, T2, cut, sSz, kx, ky, all_s, szs,
                           psec, nev, find_v, unwrap, vpath, log);
  // Same n_ones rule as Lanczos_sector.cpp:45-46.
  int n_ones = int(sSz + n_spins / 2 + 1.0e-6);
  int L1 = 0, L2 = 0, L3 = 1;
  if (three_d) LxLyLz(L1, L2, L3, T1, T2, T3);
  else LxLy(L1, L2, T1, T2);
  double px = 2 * kx * M_PI / L1, py = 2 * ky * M_PI / L2, pz = 2 * kz * M_PI / L3;
  std::vector<int64_t> states, rep_loc, Ia, Ib; std::vector<double> norm, norm_inv;
  std::vector<std::complex<double>> state_ph; int64_t n_p = 0; int bits_right = 0;
  double t0 = wall_clock();
  if (three_d)
    pConstruct_States(states, norm, norm_inv, T1, T2, T3, n_ones, px, py, pz, n_p, rep_loc, state_ph, Ia, Ib,
                      bits_right, log);
  else
    pConstruct_States(states, norm, norm_inv, T1, T2, n_ones, px, py, n_p, rep_loc, state_ph, Ia, Ib, bits_right, log);
  double t_basis = wall_clock() - t0;

  FILE* m = std::fopen((out + "/meta.txt").c_str(), "w");
  std::fprintf(m, "%d %d %d %d %d %d %lld %lld %d %.6f %d %d\n", n_spins, n_ones, L1, L2, kx, ky, (long long)n_p,
               (long long)rep_loc.size(), bits_right, t_basis, L3, kz);
  std::fclose(m);
  {
    // Term lists exactly as the reference parser produced them.
    FILE* t = std::fopen((out + "/terms.txt").c_str(), "w");
    std::fprintf(t, "lambda %.17g Ch %.17g ChCh %.17g J1 %.17g J2 %.17g\n", Jz, Ch, ChCh, J1, J2);
    std::fprintf(t, "T1");
    for (int v : T1) std::fprintf(t, " %d", v);
    std::fprintf(t, "\nT2");
    for (int v : T2) std::fprintf(t, " %d", v);
    if (three_d) {
      std::fprintf(t, "\nT3");
      for (int v : T3) std::fprintf(t, " %d", v);
    }
    std::fprintf(t, "\n");
    for (auto& b : adj) std::fprintf(t, "bond %d %d %.17g %.17g %.17g\n", b.x, b.y, b.J, b.expphase.real(), b.expphase.imag());
    for (auto& c : chl) std::fprintf(t, "ch %d %d %d %.17g %.17g\n", c.i, c.j, c.k, c.expphase.real(), c.expphase.imag());
    for (auto& c : chch) std::fprintf(t, "chch %d %d %d %d %d %d\n", c.x, c.y, c.z, c.p, c.q, c.r);
    std::fclose(t);
  }
  dump(out + "/states.i64", states);
  dump(out + "/norm.f64", norm);
  if (tables) {
    dump(out + "/rep_loc.i64", rep_loc);
    dump(out + "/state_ph.c128", state_ph);
    dump(out + "/Ia.i64", Ia);
    dump(out + "/Ib.i64", Ib);
  }
  double t_hv = 0; int calls = 0;
  for (int k = 0; k < nvec; ++k) {
    std::vector<std::complex<double>> v, w(n_p);
    if (!read_vec(out + "/v" + std::to_string(k) + ".c128", v, n_p)) break;
    for (int r = 0; r < reps; ++r) {
      double t1 = wall_clock();
      if (three_d)
        sHv(v.data(), w.data(), states, norm, norm_inv, rep_loc, state_ph, Jz, adj, Ch, chl, ChCh, chch, n_spins, Ia,
            Ib, bits_right, T1, T2, T3, px, py, pz, log);
      else
        sHv(v.data(), w.data(), states, norm, norm_inv, rep_loc, state_ph, Jz, adj, Ch, chl, ChCh, chch, n_spins, Ia,
            Ib, bits_right, T1, T2, px, py, log);
      t_hv += wall_clock() - t1; ++calls;
    }
    dump(out + "/w" + std::to_string(k) + ".c128", w);
  }
  if (calls) {
    FILE* t = std::fopen((out + "/hv_time.txt").c_str(), "w");
    std::fprintf(t, "%.9f %d\n", t_hv / calls, calls);
    std::fclose(t);
  }
  std::vector<std::complex<double>> vp;
  if (tsteps > 0 && !three_d && read_vec(out + "/vT.c128", vp, n_p)) {
    const int64_t size = n_p;
    std::vector<std::complex<double>> w(size, 0.0);
    std::vector<std::vector<std::complex<double>>> vs;
    std::vector<double> T;  // alpha (re, im) x m, then beta_0 .. beta_m
    std::vector<double> betas(1, 0.0);
    double beta = 0.0;
    normalize(vp);
    for (int it = 0; it < tsteps && it < size; ++it) {
      sHv(&*vp.begin(), &*w.begin(), states, norm, norm_inv, rep_loc, state_ph, Jz, adj, Ch, chl, ChCh, chch, n_spins,
          Ia, Ib, bits_right, T1, T2, px, py, log);
      if (it != 0) zaxpyk(size, -beta, vs[it - 1], w);
      const std::complex<double> alpha = std::conj(zdotc(size, w, vp));
      T.push_back(alpha.real());
      T.push_back(alpha.imag());
      zaxpyk(size, -alpha, vp, w);
      vs.push_back(vp);
      beta = std::sqrt(std::real(zdotc(size, w, w)));
      vp = w;
      zscalk(size, 1.0 / beta, vp);
      betas.push_back(beta);
      zscalk(size, 0.0, w);
    }
    T.insert(T.end(), betas.begin(), betas.end());
    dump(out + "/T.f64", T);
  }
  return 0;
}
