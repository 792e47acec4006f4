// Test driver for libedgpu_ref.so: calls the reference's C++ signatures
// (include/edgpu_ref.hpp) the way the reference's ED.cpp and lanczos.cpp do.
//
//   drive_ref_api sector <terms-file> <out-file>
//       runs sector_lanczos with the sector line of the terms file
//   drive_ref_api shv <terms-file> <states.i64> <v.c128> <w.c128> <out-file>
//       calls sHv(v, w, pblock_states, ...) with the given basis
//
// Terms file (one item per line): "n_sites N", "lambda x", "J2 x", "Ch x",
// "ChCh x", "T1 a b ...", "T2 a b ...", "bond x y J re im", "ch i j k re im",
// "chch x y z p q r", "sector Sz kx ky nev iterations ncycles tol find_ev
// unwrap vector_path"; a 3-D torus adds "T3 a b ..." and "kz k", and the
// 3-D sector_lanczos overload is called.
#include <complex>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "edgpu_ref.hpp"

struct Terms {
  int n_sites = 0;
  double lambda = 1, J2 = 0, Ch = 0, ChCh = 0;
  std::vector<int> T1, T2, T3;
  std::vector<coordinates> adj;
  std::vector<triangles> chl;
  std::vector<bowties> chch;
  double Sz = 0, tol = 1e-11;
  int kx = 0, ky = 0, kz = 0, nev = 2, iterations = 100, ncycles = 10, find_ev = 0, unwrap = 0;
  std::string vpath;
};

static Terms read_terms(const char* path) {
  Terms t;
  std::ifstream in(path);
  std::string line;
  while (std::getline(in, line)) {
    std::istringstream ss(line);
    std::string k;
    ss >> k;
    if (k == "n_sites") ss >> t.n_sites;
    else if (k == "lambda") ss >> t.lambda;
    else if (k == "J2") ss >> t.J2;
    else if (k == "Ch") ss >> t.Ch;
    else if (k == "ChCh") ss >> t.ChCh;
    else if (k == "kz") ss >> t.kz;
    else if (k == "T1" || k == "T2" || k == "T3") {
      int x;
      while (ss >> x) (k == "T1" ? t.T1 : (k == "T2" ? t.T2 : t.T3)).push_back(x);
    } else if (k == "bond") {
      coordinates c;
      double re, im;
      ss >> c.x >> c.y >> c.J >> re >> im;
      c.expphase = std::complex<double>(re, im);
      t.adj.push_back(c);
    } else if (k == "ch") {
      triangles c;
      double re, im;
      ss >> c.i >> c.j >> c.k >> re >> im;
      c.expphase = std::complex<double>(re, im);
      t.chl.push_back(c);
    } else if (k == "chch") {
      bowties b;
      ss >> b.x >> b.y >> b.z >> b.p >> b.q >> b.r;
      t.chch.push_back(b);
    } else if (k == "sector") {
      ss >> t.Sz >> t.kx >> t.ky >> t.nev >> t.iterations >> t.ncycles >> t.tol >> t.find_ev >> t.unwrap >> t.vpath;
    }
  }
  return t;
}

template <class T>
static std::vector<T> read_bin(const char* path) {
  std::vector<T> v;
  FILE* f = std::fopen(path, "rb");
  if (!f) return v;
  std::fseek(f, 0, SEEK_END);
  long n = std::ftell(f) / (long)sizeof(T);
  std::fseek(f, 0, SEEK_SET);
  v.resize(n);
  if (n && std::fread(v.data(), sizeof(T), n, f) != (size_t)n) v.clear();
  std::fclose(f);
  return v;
}

int main(int argc, char** argv) {
  if (argc < 4) {
    std::cerr << "usage: drive_ref_api sector|shv ...\n";
    return 2;
  }
  std::string mode = argv[1];
  Terms t = read_terms(argv[2]);
  if (mode == "sector") {
    std::ofstream out(argv[3]);
    bool find_ev = t.find_ev, unwrap = t.unwrap;
    if (!t.T3.empty())
      sector_lanczos(t.kx, t.ky, t.kz, t.Sz, t.n_sites, t.lambda, t.J2, t.adj, t.Ch, t.chl, t.ChCh, t.chch, t.T1, t.T2,
                     t.T3, t.nev, find_ev, unwrap, t.vpath, t.tol, t.iterations, t.ncycles, out);
    else
      sector_lanczos(t.kx, t.ky, t.Sz, t.n_sites, t.lambda, t.J2, t.adj, t.Ch, t.chl, t.ChCh, t.chch, t.T1, t.T2,
                     t.nev, find_ev, unwrap, t.vpath, t.tol, t.iterations, t.ncycles, out);
    return 0;
  }
  if (mode == "shv" && argc >= 7) {
    std::vector<int64_t> states = read_bin<int64_t>(argv[3]);
    std::vector<std::complex<double> > v = read_bin<std::complex<double> >(argv[4]);
    std::vector<std::complex<double> > w(states.size());
    std::vector<double> norm, norm_inv;
    std::vector<int64_t> rep_loc, Ia, Ib;
    std::vector<std::complex<double> > state_ph;
    std::ofstream out(argv[6]);
    const double px = 2 * t.kx * 3.14159265358979323846, py = 2 * t.ky * 3.14159265358979323846;
    int L1 = 0, L2 = 0, s = 0;
    do { s = t.T1[s]; ++L1; } while (s != 0);
    s = 0;
    do { s = t.T2[s]; ++L2; } while (s != 0);
    const double kxr = px / L1, kyr = py / L2;
    int bits_right = 0;
    for (int rep = 0; rep < 2; ++rep)  // second call reuses the cached sector
      sHv(v.data(), w.data(), states, norm, norm_inv, rep_loc, state_ph, t.lambda, t.adj, t.Ch, t.chl, t.ChCh,
          t.chch, t.n_sites, Ia, Ib, bits_right, t.T1, t.T2, kxr, kyr, out);
    FILE* f = std::fopen(argv[5], "wb");
    std::fwrite(w.data(), sizeof(std::complex<double>), w.size(), f);
    std::fclose(f);
    return 0;
  }
  std::cerr << "bad arguments\n";
  return 2;
}
