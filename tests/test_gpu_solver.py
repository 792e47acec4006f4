"""The FP64 sector eigensolver (dense and Lanczos paths) against the reference's ED2 output.

The reference printed these eigenvalues (tests/golden/cases.json, "ed2_eigs"):
its dense zheev path for n_p <= 10000 and its deflated Lanczos above.  The
plain form must reproduce them to 1e-10 relative.
"""
import numpy as np
import pytest

from conftest import all_golden_sectors, golden_cases, golden_model

pytestmark = pytest.mark.gpu

REL = 1e-10


@pytest.fixture(scope="module")
def gpu(cuda_device):
    from ed_code_gb300 import sector

    return sector


def ed2(name, idx):
    return golden_cases()[name]["sectors"][idx]


@pytest.mark.parametrize("name,idx", [(n, i) for n, i in all_golden_sectors()
                                      if ed2(n, i).get("ed2_path") == "dense"])
def test_dense_path_matches_reference(gpu, name, idx):
    meta = ed2(name, idx)
    sec = gpu.GpuSector(golden_model(name, idx))
    eigs, _, st = sec.solve_plain(n_ev=4)
    assert st["path"] == 1 and len(eigs) == sec.n_p        # all eigenvalues, like exact_evecs
    ref = np.array(meta["ed2_eigs"])
    np.testing.assert_allclose(eigs[: len(ref)], ref, rtol=REL, atol=REL)


@pytest.mark.parametrize("name,idx", [(n, i) for n, i in all_golden_sectors()
                                      if ed2(n, i).get("ed2_path") == "lanczos"])
def test_lanczos_path_matches_reference(gpu, name, idx):
    meta = ed2(name, idx)
    kw = meta["ed2_kw"]
    sec = gpu.GpuSector(golden_model(name, idx))
    eigs, _, st = sec.solve_plain(n_ev=kw["num_eigenvalues"], iterations=kw["iterations"], ncycles=kw["ncycles"],
                                  tol=kw["tol"], seed=1)
    assert st["path"] == 0
    ref = np.array(meta["ed2_eigs"])
    np.testing.assert_allclose(eigs, ref, rtol=REL, atol=0)


def test_forced_lanczos_on_small_sector_matches_dense(gpu):
    """Deflated Lanczos on the 4x4 square sector returns the lowest levels of the dense spectrum."""
    sec = gpu.GpuSector(golden_model("sq4x4", 0))
    dense, _, _ = sec.solve_plain(n_ev=4)
    lz, vecs, st = sec.solve_plain(n_ev=4, iterations=200, ncycles=3, tol=1e-13, seed=7, dense_threshold=-1,
                                   want_vectors=True)
    assert st["path"] == 0
    np.testing.assert_allclose(lz, dense[:4], rtol=REL, atol=0)
    # Ritz vectors: orthonormal and eigenvectors of H (residual through the GPU H*v)
    G = vecs.conj() @ vecs.T
    assert np.abs(G - np.eye(4)).max() < 1e-9
    for k in range(4):
        r = sec.sHv(vecs[k]) - lz[k] * vecs[k]
        assert np.linalg.norm(r) < 1e-6


def test_solver_log_lines(gpu):
    lines = []
    sec = gpu.GpuSector(golden_model("tri4x3", 0))
    sec.solve_plain(n_ev=1, iterations=30, ncycles=3, tol=1e-12, dense_threshold=-1, log=lines.append)
    assert any(l.startswith("Eigs[0]") for l in lines)
    assert any(l.startswith("Eigenvalue number 0") for l in lines)


@pytest.mark.parametrize("name,idx", [("cub3x2x2", 1), ("cub4x2x2", 0), ("cub4x2x2", 1)])
def test_three_d_torus_spectrum(name, idx, cuda_device):
    """3-D tori: the plain solver (dense path) and the mixed solver against the
    oracle's dense spectrum, whose H matches the reference's 3-D sHv."""
    import oracle as O
    from ed_code_gb300 import sector

    model = golden_model(name, idx)
    assert model.T3
    ev = np.linalg.eigvalsh(O.OracleSector(model).dense())
    sec = sector.GpuSector(model)
    assert sec.info["L3"] == 2 and sec.info["kz"] == model.kz
    eigs, _, _ = sec.solve_plain(n_ev=3)
    np.testing.assert_allclose(eigs[:3], ev[:3], rtol=1e-10)
    assert sec.build_targets()
    out = sec.solve_mixed(n_ev=2, iterations=min(150, sec.n_p), reorth_every=1)
    levels = [ev[0]] + [x for x in ev[1:] if abs(x - ev[0]) > 1e-9 * abs(x)]
    np.testing.assert_allclose(out["eigs"][0], levels[0], rtol=1e-9)


def test_three_d_momentum_out_of_range(cuda_device):
    from ed_code_gb300 import lattice as L
    from ed_code_gb300 import sector
    from ed_code_gb300._native import EdgError

    m = L.make_model(L.TorusSpec("cubic", 3, 2, Lz=2, Jz=0.9), 0, 0, 0, kz=0)
    m.kz = 2
    with pytest.raises(EdgError, match="Invalid kx or ky"):
        sector.GpuSector(m)


def test_plain_solver_rejects_more_iterations_than_it_can_combine(gpu):
    """A cycle's Ritz vector combines at most 2048 stored Krylov vectors: more
    iterations per cycle are refused before any work."""
    from ed_code_gb300._native import EdgError

    sec = gpu.GpuSector(golden_model("tri4x3", 0))
    with pytest.raises(EdgError):
        sec.solve_plain(n_ev=1, iterations=4096, ncycles=1, tol=1e-12, dense_threshold=-1)


@pytest.mark.parametrize("spec_kw,sector", [
    (dict(lattice="triangular", Lx=6, Ly=3, Jz=0.9, Ch=0.15), (0, 0, 0)),   # n_p 2710
    (dict(lattice="square", Lx=6, Ly=3), (0, 1, 0)),                         # 2700, degenerate levels
    (dict(lattice="square", Lx=4, Ly=4), (0, 1, 1)),                         # 800, many degenerate levels
])
def test_dense_path_full_spectrum_against_oracle(gpu, spec_kw, sector):
    """The device dense path (Householder, bisection + Newton on T, inverse
    iteration, back-transformation) on 16- and 18-site sectors: every
    eigenvalue against numpy's spectrum of the oracle's dense H; eigenvectors
    up to the first degenerate pair (orthonormal within it) by their residual
    through the GPU H*v and their orthonormality."""
    import sys, os
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
    import oracle as O
    from ed_code_gb300 import lattice as L

    model = L.make_model(L.TorusSpec(**spec_kw), *sector)
    ref = np.linalg.eigvalsh(O.OracleSector(model).dense())
    scale = max(1.0, np.abs(ref).max())
    gaps = np.flatnonzero(np.diff(ref) < 1e-10 * scale)
    n_vec = int(min(32, gaps[0] + 2)) if len(gaps) else 6
    sec = gpu.GpuSector(model)
    assert sec.build_targets()
    eigs, vecs, st = sec.solve_plain(n_ev=n_vec, want_vectors=True)
    assert st["path"] == 1 and len(eigs) == sec.n_p
    assert np.abs(eigs - ref).max() <= 1e-10 * scale
    V = np.asarray(vecs)
    G = V.conj() @ V.T
    assert np.abs(G - np.eye(len(V))).max() <= 1e-10
    for k in range(len(V)):
        r = sec.sHv(V[k]) - eigs[k] * V[k]
        assert np.linalg.norm(r) <= 1e-9 * scale
