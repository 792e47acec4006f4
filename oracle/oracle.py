"""ctypes front end of the CPU restatement in ed_oracle.c.

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
benchmark's CPU-baseline leg as the checker.  The GPU library never imports
it.  ``build()`` compiles liboracle.so from ed_oracle.c with gcc.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")


class Bond(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int), ("J", C.c_double), ("re", C.c_double), ("im", C.c_double)]


class Tri(C.Structure):
    _fields_ = [("i", C.c_int), ("j", C.c_int), ("k", C.c_int), ("re", C.c_double), ("im", C.c_double)]


class Bowtie(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("x", "y", "z", "p", "q", "r")]


class Basis(C.Structure):
    _fields_ = [
        ("n_sites", C.c_int), ("n_ones", C.c_int), ("L1", C.c_int), ("L2", C.c_int), ("kx", C.c_int),
        ("ky", C.c_int), ("half_sites", C.c_int), ("bits_right", C.c_int64), ("n_configs", C.c_int64),
        ("n_p", C.c_int64), ("states", C.POINTER(C.c_int64)), ("norm", C.POINTER(C.c_double)),
        ("norm_inv", C.POINTER(C.c_double)), ("lid", C.POINTER(C.c_int32)), ("rep_loc", C.POINTER(C.c_int64)),
        ("state_ph", C.POINTER(C.c_double)), ("lx", C.POINTER(C.c_int32)), ("ly", C.POINTER(C.c_int32)),
        ("Ia", C.POINTER(C.c_int64)), ("Ib", C.POINTER(C.c_int64)), ("L3", C.c_int), ("kz", C.c_int),
        ("lz", C.POINTER(C.c_int32)),
    ]


_lib: Optional[C.CDLL] = None


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "ed_oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c11", "-o", LIB_PATH, src, "-lm"],
                       check=True)
    return LIB_PATH


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.or_build_basis.restype = C.POINTER(Basis)
        L.or_build_basis.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int, C.c_int]
        L.or_build_basis3.restype = C.POINTER(Basis)
        L.or_build_basis3.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                      C.c_int, C.c_int, C.c_int]
        L.or_free_basis.argtypes = [C.POINTER(Basis)]
        L.or_hv_tables.argtypes = [C.POINTER(Basis), C.c_void_p, C.c_void_p, C.c_double, C.POINTER(Bond), C.c_int,
                                   C.c_double, C.POINTER(Tri), C.c_int, C.c_double, C.POINTER(Bowtie), C.c_int]
        L.or_hv_rows.argtypes = [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int, C.c_int, C.c_void_p,
                                 C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_double,
                                 C.POINTER(Bond), C.c_int, C.c_double, C.POINTER(Tri), C.c_int, C.c_double,
                                 C.POINTER(Bowtie), C.c_int, C.c_int]
        L.or_allowed_rep.argtypes = [C.c_int64, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int, C.c_int, C.c_int]
        L.or_allowed_rep.restype = C.c_int
        L.or_sector_dim.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int, C.c_int]
        L.or_sector_dim.restype = C.c_int64
        L.or_sector_dim3.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                     C.c_int, C.c_int, C.c_int]
        L.or_sector_dim3.restype = C.c_int64
        L.or_build_reps.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int, C.c_int,
                                    C.POINTER(C.POINTER(C.c_int64)), C.POINTER(C.POINTER(C.c_int32)), C.c_int]
        L.or_build_reps.restype = C.c_int64
        L.or_hv_rows_listless.argtypes = [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int, C.c_int,
                                          C.c_void_p, C.c_void_p, C.c_int64, C.c_uint64, C.c_void_p, C.c_double,
                                          C.POINTER(Bond), C.c_int, C.c_double, C.POINTER(Tri), C.c_int,
                                          C.c_double, C.POINTER(Bowtie), C.c_int, C.c_int, C.c_void_p, C.c_int64]
        L.or_sample_reps.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int, C.c_int,
                                     C.c_uint64, C.c_int64, C.c_void_p, C.c_void_p]
        L.or_sample_reps.restype = C.c_int64
        L.or_value_vector.argtypes = [C.c_void_p, C.c_int64, C.c_uint64, C.c_void_p]
        L.or_free.argtypes = [C.c_void_p]
        L.or_set_threads.argtypes = [C.c_int]
        L.or_n_choose_k.argtypes = [C.c_int, C.c_int]
        L.or_n_choose_k.restype = C.c_int64
        _lib = L
    return _lib


def _ints(a: Sequence[int]):
    return (C.c_int * len(a))(*[int(x) for x in a])


class TermLists:
    """C arrays of the three term lists of a lattice.Model."""

    def __init__(self, model):
        self.model = model
        self.bonds = (Bond * max(1, len(model.adj_list)))(
            *[Bond(b.x, b.y, b.J, b.expphase.real, b.expphase.imag) for b in model.adj_list])
        self.nb = len(model.adj_list)
        self.tris = (Tri * max(1, len(model.ch_list)))(
            *[Tri(t.i, t.j, t.k, t.expphase.real, t.expphase.imag) for t in model.ch_list])
        self.nt = len(model.ch_list)
        self.bows = (Bowtie * max(1, len(model.chch_list)))(
            *[Bowtie(b.x, b.y, b.z, b.p, b.q, b.r) for b in model.chch_list])
        self.nbw = len(model.chch_list)
        self.T1 = _ints(model.T1)
        self.T2 = _ints(model.T2)
        self.T3 = _ints(model.T3) if getattr(model, "T3", None) else None


class OracleSector:
    """Full reference tables for one (Sz, kx, ky) sector (pConstruct_States)."""

    def __init__(self, model):
        self.model = model
        self.terms = TermLists(model)
        if self.terms.T3 is not None:
            p = lib().or_build_basis3(model.n_sites, model.n_ones, self.terms.T1, self.terms.T2, self.terms.T3,
                                      model.kx, model.ky, model.kz)
        else:
            p = lib().or_build_basis(model.n_sites, model.n_ones, self.terms.T1, self.terms.T2, model.kx, model.ky)
        if not p:
            raise ValueError("oracle: bad sector")
        self._p = p
        b = p.contents
        self.n_p = int(b.n_p)
        self.n_configs = int(b.n_configs)
        self.L1, self.L2, self.L3 = int(b.L1), int(b.L2), int(b.L3)
        self.bits_right = int(b.bits_right)
        arr = np.ctypeslib.as_array
        n, nc, nh = self.n_p, self.n_configs, 1 << b.half_sites
        self.states = arr(b.states, (max(n, 1),))[:n].copy()
        self.norm = arr(b.norm, (max(n, 1),))[:n].copy()
        self.norm_inv = arr(b.norm_inv, (max(n, 1),))[:n].copy()
        self.lid = arr(b.lid, (max(n, 1),))[:n].copy()
        self.rep_loc = arr(b.rep_loc, (nc,)).copy()
        self.state_ph = arr(b.state_ph, (2 * nc,)).copy().view(np.complex128)
        self.lx = arr(b.lx, (nc,)).copy()
        self.ly = arr(b.ly, (nc,)).copy()
        self.Ia = arr(b.Ia, (nh,)).copy()
        self.Ib = arr(b.Ib, (nh,)).copy()

    def hv(self, v: np.ndarray) -> np.ndarray:
        v = np.ascontiguousarray(v, dtype=np.complex128)
        assert v.shape == (self.n_p,)
        w = np.zeros_like(v)
        m, t = self.model, self.terms
        lib().or_hv_tables(self._p, v.ctypes.data, w.ctypes.data, m.Jz, t.bonds, t.nb, m.Ch, t.tris, t.nt, m.ChCh,
                           t.bows, t.nbw)
        return w

    def time_hv(self, v: np.ndarray, threads: int, min_seconds: float = 0.3):
        """Seconds per table-mode H*v (the reference's sHv row formula with its
        rep_loc/state_ph tables) on `threads` OpenMP threads, averaged over
        repeated calls until min_seconds have passed."""
        import time

        lib().or_set_threads(int(threads))
        try:
            self.hv(v)  # warm
            n, t0 = 0, time.perf_counter()
            while True:
                self.hv(v)
                n += 1
                dt = time.perf_counter() - t0
                if dt >= min_seconds:
                    return dt / n
        finally:
            lib().or_set_threads(os.cpu_count() or 1)

    def dense(self) -> np.ndarray:
        """Dense H (makeH, H_v.cpp:21-190, is the same row formula applied to unit vectors)."""
        H = np.zeros((self.n_p, self.n_p), dtype=np.complex128)
        e = np.zeros(self.n_p, dtype=np.complex128)
        for j in range(self.n_p):
            e[:] = 0
            e[j] = 1
            H[:, j] = self.hv(e)
        return H

    def __del__(self):
        try:
            lib().or_free_basis(self._p)
        except Exception:
            pass


def hv_rows(model, reps: np.ndarray, lid: np.ndarray, v: np.ndarray, rows: np.ndarray, n_threads: int = 0):
    """Rows of H v from the orbit walk + binary search (no per-configuration tables)."""
    t = TermLists(model)
    reps = np.ascontiguousarray(reps, dtype=np.int64)
    lid = np.ascontiguousarray(lid, dtype=np.int32)
    v = np.ascontiguousarray(v, dtype=np.complex128)
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    out = np.zeros(len(rows), dtype=np.complex128)
    lib().or_hv_rows(model.n_sites, t.T1, t.T2, model.kx, model.ky, reps.ctypes.data, lid.ctypes.data, len(reps),
                     v.ctypes.data, rows.ctypes.data, len(rows), out.ctypes.data, model.Jz, t.bonds, t.nb, model.Ch,
                     t.tris, t.nt, model.ChCh, t.bows, t.nbw, int(n_threads))
    return out


def build_reps(model, n_threads: int = 0):
    """(reps, lid) of the sector by parallel enumeration, without tables."""
    t = TermLists(model)
    rp = C.POINTER(C.c_int64)()
    lp = C.POINTER(C.c_int32)()
    n = lib().or_build_reps(model.n_sites, model.n_ones, t.T1, t.T2, model.kx, model.ky, C.byref(rp), C.byref(lp),
                            int(n_threads))
    reps = np.ctypeslib.as_array(rp, (max(n, 1),))[:n].copy()
    lid = np.ctypeslib.as_array(lp, (max(n, 1),))[:n].copy()
    lib().or_free(rp)
    lib().or_free(lp)
    return reps, lid


def sample_reps(model, n: int, seed: int = 1):
    """n allowed representatives (with their stabiliser counts) drawn at random,
    without building the sector's list."""
    t = TermLists(model)
    states = np.empty(n, np.int64)
    lid = np.empty(n, np.int32)
    got = lib().or_sample_reps(model.n_sites, model.n_ones, t.T1, t.T2, model.kx, model.ky, int(seed), int(n),
                               states.ctypes.data, lid.ctypes.data)
    return states[:got], lid[:got]


def value_vector(reps: np.ndarray, seed: int) -> np.ndarray:
    """The vector hv_rows_listless uses: entry j is a hash of reps[j]."""
    reps = np.ascontiguousarray(reps, dtype=np.int64)
    v = np.empty(len(reps), np.complex128)
    lib().or_value_vector(reps.ctypes.data, len(reps), int(seed), v.ctypes.data)
    return v


def hv_rows_listless(model, rows: np.ndarray, row_lid: np.ndarray, vseed: int, n_threads: int = 0,
                     probe: np.ndarray = None):
    """Rows of H v for representatives `rows`, with v = value_vector(., vseed),
    without the sector's representative list.  `probe`: a sorted int64 array
    of the list's size; each target then also pays the binary search of the
    rank lookup (its result unused)."""
    t = TermLists(model)
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    row_lid = np.ascontiguousarray(row_lid, dtype=np.int32)
    out = np.zeros(len(rows), dtype=np.complex128)
    pp, pn = (None, 0) if probe is None else (probe.ctypes.data, len(probe))
    lib().or_hv_rows_listless(model.n_sites, t.T1, t.T2, model.kx, model.ky, rows.ctypes.data, row_lid.ctypes.data,
                              len(rows), int(vseed), out.ctypes.data, model.Jz, t.bonds, t.nb, model.Ch, t.tris, t.nt,
                              model.ChCh, t.bows, t.nbw, int(n_threads), pp, pn)
    return out


def sorted_probe(n: int, lo: int, hi: int, seed: int = 9) -> np.ndarray:
    """n sorted int64 values spread over [lo, hi) (cumulative random gaps): the
    size and value range of a representative list, for hv_rows_listless's
    rank-lookup stand-in."""
    rng = np.random.default_rng(seed)
    gap = max(1, (hi - lo) // max(n, 1))
    out = np.cumsum(rng.integers(1, 2 * gap, size=n, dtype=np.int64))
    out += lo
    return out


def allowed_rep(model, state: int) -> int:
    t = TermLists(model)
    return int(lib().or_allowed_rep(int(state), t.T1, t.T2, model.n_sites, model.kx, model.ky))


def sector_dim(model) -> int:
    t = TermLists(model)
    if t.T3 is not None:
        return int(lib().or_sector_dim3(model.n_sites, model.n_ones, t.T1, t.T2, t.T3, model.kx, model.ky, model.kz))
    return int(lib().or_sector_dim(model.n_sites, model.n_ones, t.T1, t.T2, model.kx, model.ky))


def n_choose_k(n: int, k: int) -> int:
    return int(lib().or_n_choose_k(n, k))


def splitmix_vector(n: int, seed: int) -> np.ndarray:
    """Deterministic complex test vector, entries uniform in [-1, 1)^2.

    splitmix64 over the counter 2*i (real) and 2*i+1 (imaginary); the CUDA
    library has the same generator, so host and device draw identical vectors.
    """
    with np.errstate(over="ignore"):
        i = np.arange(2 * n, dtype=np.uint64)
        x = np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15) + (i + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15)
        z = x
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
        u = (z >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)
    u = 2.0 * u - 1.0
    return (u[0::2] + 1j * u[1::2]).astype(np.complex128)
