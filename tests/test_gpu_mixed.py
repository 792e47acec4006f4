"""Mixed-precision solver (FP32 Krylov vectors and H*v, FP64 scalars, FP64
Rayleigh quotient on each Ritz vector) against the reference's FP64 results.

Target: |dE|/|E| <= 1e-9 against the eigenvalues the reference printed.
"""
import numpy as np
import pytest

from conftest import golden_cases, golden_model

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu(cuda_device):
    from ed_code_gb300 import sector

    return sector


@pytest.mark.parametrize("reorth", [1, 4, 0])
@pytest.mark.parametrize("name,n_ev", [("tri6x4_k10", 2), ("sq6x4_k00", 4)])
def test_mixed_matches_reference(gpu, name, n_ev, reorth):
    ref = np.array(golden_cases()[name]["sectors"][0]["ed2_eigs"][:n_ev])
    sec = gpu.GpuSector(golden_model(name, 0))
    out = sec.solve_mixed(n_ev=n_ev, iterations=300, reorth_every=reorth, seed=1)
    eigs = out["eigs"]
    assert len(eigs) >= n_ev, out
    rel = np.abs(eigs[:n_ev] - ref) / np.abs(ref)
    assert rel.max() <= 1e-9, (eigs, ref, out["residuals"])
    assert np.all(out["residuals"][:n_ev] < 1e-3)
    assert out["stats"]["passes"] == (1 if reorth else 2)


@pytest.mark.parametrize("reorth", [1, 0])
def test_mixed_eigenvectors(gpu, reorth):
    """Stored vectors (reorth 1) or the second pass over resident vectors (0)."""
    sec = gpu.GpuSector(golden_model("tri6x4_k10", 0))
    out = sec.solve_mixed(n_ev=2, iterations=250, reorth_every=reorth, want_vectors=True)
    assert out["stats"]["passes"] == (1 if reorth else 2)
    X = out["evecs"]
    for k in range(len(out["eigs"])):
        assert abs(np.vdot(X[k], X[k]).real - 1.0) < 1e-12
        r = sec.sHv(X[k]) - out["eigs"][k] * X[k]
        assert np.linalg.norm(r) <= 2 * out["residuals"][k] + 1e-12


@pytest.mark.parametrize("reorth", [1, 0])
def test_mixed_with_column_panels(gpu, reorth):
    sec = gpu.GpuSector(golden_model("sq6x4_k00", 0))
    ref = np.array(golden_cases()["sq6x4_k00"]["sectors"][0]["ed2_eigs"][:2])
    assert sec.build_targets()
    sec.pack_panels(6)
    out = sec.solve_mixed(n_ev=2, iterations=300, reorth_every=reorth)
    assert np.max(np.abs(out["eigs"][:2] - ref) / np.abs(ref)) <= 1e-9


def test_mixed_with_stored_targets(gpu):
    sec = gpu.GpuSector(golden_model("tri6x4_k10", 0))
    ref = np.array(golden_cases()["tri6x4_k10"]["sectors"][0]["ed2_eigs"][:2])
    assert sec.build_targets()
    out = sec.solve_mixed(n_ev=2, iterations=300, reorth_every=1)
    assert np.max(np.abs(out["eigs"][:2] - ref) / np.abs(ref)) <= 1e-9
