"""The C++ drop-in (libedgpu_ref.so): the reference's own sector_lanczos / sHv
signatures over the GPU library.

* On a machine with the reference sources, its unmodified ED.o and
  read_input_file.o (built into oracle/_ref) must link against the drop-in.
* On the GPU, a C++ driver calls those signatures; the printed Energies table
  must match what the reference's ED2 printed, unwrapped eigenvectors must be
  eigenvectors of the full fixed-Sz Hamiltonian, and sHv must match the
  reference's sHv output.
"""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden_arrays, golden_cases, golden_model

LIBDIR = os.path.join(ROOT, "ed_code_gb300")
BUILD = os.path.join(ROOT, "tests", "_build")
DRIVER_SRC = os.path.join(ROOT, "tests", "adapter", "drive_ref_api.cpp")


def libs():
    from ed_code_gb300 import build

    build.build()
    return os.path.join(LIBDIR, "libedgpu_ref.so")


def test_reference_driver_links_against_the_drop_in(tmp_path):
    ed_o = os.path.join(ROOT, "oracle", "_ref", "ED.o")
    rif_o = os.path.join(ROOT, "oracle", "_ref", "read_input_file.o")
    if not (os.path.exists(ed_o) and os.path.exists(rif_o)):
        pytest.skip("reference objects not built here (needs the reference sources)")
    libs()
    exe = str(tmp_path / "ED2_gpu")
    r = subprocess.run(["g++", "-o", exe, ed_o, rif_o, "-L", LIBDIR, "-ledgpu_ref", "-ledgpu", "-fopenmp",
                        f"-Wl,-rpath,{LIBDIR}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert os.path.exists(exe)


def driver():
    libs()
    os.makedirs(BUILD, exist_ok=True)
    exe = os.path.join(BUILD, "drive_ref_api")
    if not os.path.exists(exe) or os.path.getmtime(exe) < os.path.getmtime(DRIVER_SRC):
        subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), "-o", exe, DRIVER_SRC,
                        "-L", LIBDIR, "-ledgpu_ref", "-ledgpu", f"-Wl,-rpath,{LIBDIR}"], check=True)
    return exe


def write_terms(path, model, nev=4, iterations=100, ncycles=10, tol=1e-11, find_ev=0, unwrap=0, vpath="none"):
    with open(path, "w") as f:
        f.write(f"n_sites {model.n_sites}\nlambda {model.Jz!r}\nJ2 {model.J2!r}\nCh {model.Ch!r}\nChCh {model.ChCh!r}\n")
        f.write("T1 " + " ".join(map(str, model.T1)) + "\n")
        f.write("T2 " + " ".join(map(str, model.T2)) + "\n")
        if getattr(model, "T3", None):
            f.write("T3 " + " ".join(map(str, model.T3)) + "\n")
            f.write(f"kz {model.kz}\n")
        for b in model.adj_list:
            f.write(f"bond {b.x} {b.y} {b.J!r} {b.expphase.real!r} {b.expphase.imag!r}\n")
        for t in model.ch_list:
            f.write(f"ch {t.i} {t.j} {t.k} {t.expphase.real!r} {t.expphase.imag!r}\n")
        for b in model.chch_list:
            f.write(f"chch {b.x} {b.y} {b.z} {b.p} {b.q} {b.r}\n")
        f.write(f"sector {model.Sz!r} {model.kx} {model.ky} {nev} {iterations} {ncycles} {tol!r} {find_ev} {unwrap} "
                f"{vpath}\n")


def energies(text):
    lines = text.splitlines()
    i = next(k for k, l in enumerate(lines) if l.startswith("Energies"))
    out = []
    for l in lines[i + 1:]:
        p = l.split()
        if len(p) >= 7:
            out.append(float(p[0]))
    return np.array(out)


@pytest.mark.gpu
@pytest.mark.parametrize("name,idx", [("sq4x4", 0), ("tri4x3_chch", 0), ("tri6x4_k10", 0)])
def test_sector_lanczos_prints_reference_energies(cuda_device, tmp_path, name, idx):
    meta = golden_cases()[name]["sectors"][idx]
    kw = meta.get("ed2_kw", {})
    model = golden_model(name, idx)
    terms = tmp_path / "terms.txt"
    write_terms(terms, model, nev=kw.get("num_eigenvalues", 4), iterations=kw.get("iterations", 200),
                ncycles=kw.get("ncycles", 2), tol=kw.get("tol", 1e-12))
    out = tmp_path / "out.txt"
    subprocess.run([driver(), "sector", str(terms), str(out)], check=True)
    text = out.read_text()
    assert f" SECTOR : " in text and str(meta["n_p"]) in text
    e = energies(text)
    ref = np.array(meta["ed2_eigs"])
    np.testing.assert_allclose(e[: len(ref)], ref, rtol=1e-10)


def full_space_hamiltonian(model):
    """H in the fixed-Sz basis (no translation symmetry) from the reference's row formula."""
    from itertools import combinations

    n = model.n_sites
    states = sorted(sum(1 << b for b in c) for c in combinations(range(n), model.n_ones))
    index = {s: i for i, s in enumerate(states)}
    H = np.zeros((len(states), len(states)), dtype=np.complex128)
    bit = lambda s, k: (s >> k) & 1
    for i, s in enumerate(states):
        ezz = 0.0
        for b in model.adj_list:
            if abs(b.J) < 1e-16:
                continue
            if bit(s, b.x) == bit(s, b.y):
                ezz += 0.25 * model.Jz * b.J
            else:
                ezz -= 0.25 * model.Jz * b.J
                e = b.expphase.conjugate() if bit(s, b.x) else b.expphase
                H[i, index[s ^ (1 << b.x) ^ (1 << b.y)]] += e * b.J * 0.5
        H[i, i] += ezz
        if abs(model.Ch) > 1e-16:
            for t in model.ch_list:
                if bit(s, t.i) != bit(s, t.j):
                    sg = 1j * t.expphase if bit(s, t.j) else -1j * t.expphase.conjugate()
                    if not bit(s, t.k):
                        sg = -sg
                    H[i, index[s ^ (1 << t.i) ^ (1 << t.j)]] += model.Ch * 0.25 * sg
    return states, H


@pytest.mark.gpu
def test_unwrapped_eigenvectors_are_full_space_eigenvectors(cuda_device, tmp_path):
    model = golden_model("tri4x3", 5)
    terms = tmp_path / "terms.txt"
    vpath = str(tmp_path / "vec")
    write_terms(terms, model, nev=2, find_ev=1, unwrap=1, vpath=vpath)
    subprocess.run([driver(), "sector", str(terms), str(tmp_path / "out.txt")], check=True)
    e = energies((tmp_path / "out.txt").read_text())
    states, H = full_space_hamiltonian(model)
    assert np.abs(H - H.conj().T).max() < 1e-12
    index = {s: i for i, s in enumerate(states)}
    for k in range(2):
        text = open(f"{vpath}_EV{k}.txt").read().split("EIGENVECTOR")[1]
        psi = np.zeros(len(states), dtype=np.complex128)
        for line in text.strip().splitlines():
            sid, c = line.split("\t")
            re_, im_ = map(float, c.strip("()").split(","))
            psi[index[int(sid)]] = re_ + 1j * im_
        assert np.linalg.norm(psi) > 0.1
        r = H @ psi - e[k] * psi
        assert np.linalg.norm(r) / np.linalg.norm(psi) < 1e-9


@pytest.mark.gpu
def test_momentum_eigenvector_file_format(cuda_device, tmp_path):
    model = golden_model("sq4x4", 0)
    terms = tmp_path / "terms.txt"
    vpath = str(tmp_path / "vec")
    write_terms(terms, model, nev=1, find_ev=1, unwrap=0, vpath=vpath)
    subprocess.run([driver(), "sector", str(terms), str(tmp_path / "out.txt")], check=True)
    text = open(f"{vpath}_pEV0.txt").read()
    assert "Momentum EIGENVECTOR" in text and "pblock_states" in text
    rows = [l.split() for l in text.split("v_coeff")[1].strip().splitlines()]
    g = golden_arrays("sq4x4")
    assert [int(r[0]) for r in rows] == list(g["s0_states"])
    c = np.array([complex(*map(float, r[2].strip("()").split(","))) for r in rows])
    assert abs(np.vdot(c, c).real - 1.0) < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["sq4x4", "tri4x3_chch", "sq4x4_phase_sz1"])
def test_shv_signature_matches_reference(cuda_device, tmp_path, name):
    import oracle as O

    meta = golden_cases()[name]["sectors"][0]
    g = golden_arrays(name)
    model = golden_model(name, 0)
    terms = tmp_path / "terms.txt"
    write_terms(terms, model)
    states = g["s0_states"]
    states.astype(np.int64).tofile(tmp_path / "states.i64")
    v = O.splitmix_vector(len(states), meta["vec_seeds"][0])
    v.tofile(tmp_path / "v.c128")
    subprocess.run([driver(), "shv", str(terms), str(tmp_path / "states.i64"), str(tmp_path / "v.c128"),
                    str(tmp_path / "w.c128"), str(tmp_path / "out.txt")], check=True)
    w = np.fromfile(tmp_path / "w.c128", np.complex128)
    ref = g["s0_w0"]
    assert np.abs(w - ref).max() / max(1.0, np.abs(ref).max()) <= 1e-13


@pytest.mark.gpu
@pytest.mark.parametrize("name,idx", [("cub3x2x2", 1), ("cub4x2x2", 1)])
def test_three_d_sector_lanczos(cuda_device, tmp_path, name, idx):
    """The 3-D overload: Lanczos always (no dense path, Lanczos_sector.cpp:285),
    (px,py,pz) in the SECTOR line, kz in the tables and files, and unwrapped
    eigenvectors as the reference's Unwrap_pState writes them: it sums every
    orbit over all L1 L2 L3 translations, so a state whose stabiliser has lid
    elements comes out lid times too large; divided by lid the vector is an
    eigenvector of the full-space H."""
    import oracle as O

    model = golden_model(name, idx)
    terms = tmp_path / "terms.txt"
    vpath = str(tmp_path / "vec")
    write_terms(terms, model, nev=2, iterations=150, ncycles=10, tol=1e-12, find_ev=1, unwrap=1, vpath=vpath)
    subprocess.run([driver(), "sector", str(terms), str(tmp_path / "out.txt")], check=True)
    text = (tmp_path / "out.txt").read_text()
    assert "Lanczos SUMMARY" in text and "EXACT SUMMARY" not in text
    assert "Energies\t\tEnergies/site\t\tSz\tkx\tky\tkz\tJz\tJ2" in text and " find_ev = 1" in text
    sector_line = next(l for l in text.splitlines() if l.startswith(" SECTOR :"))
    assert sector_line.split("(")[1].split(")")[0].count(",") == 2
    e = energies(text)
    ev = np.linalg.eigvalsh(O.OracleSector(model).dense())
    np.testing.assert_allclose(e[:2], ev[:2], rtol=1e-10)
    states, H = full_space_hamiltonian(model)
    index = {s: i for i, s in enumerate(states)}
    osec = O.OracleSector(model)
    half = model.n_sites // 2

    def lid_of(s):  # stabiliser size of the orbit of s, from the reference's tables
        lin = osec.Ia[s & ((1 << half) - 1)] + osec.Ib[s >> half] - 1
        return osec.lid[osec.rep_loc[lin]]

    for k in range(2):
        body = open(f"{vpath}_EV{k}.txt").read()
        assert f"({model.kx},{model.ky},{model.kz})" in body
        psi = np.zeros(len(states), dtype=np.complex128)
        for line in body.split("EIGENVECTOR")[1].strip().splitlines():
            sid, c = line.split("\t")
            re_, im_ = map(float, c.strip("()").split(","))
            psi[index[int(sid)]] = (re_ + 1j * im_) / lid_of(int(sid))
        assert abs(np.linalg.norm(psi) - 1) < 1e-9
        r = H @ psi - e[k] * psi
        assert np.linalg.norm(r) < 1e-9
