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
