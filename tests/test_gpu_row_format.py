"""The two entry formats of the stored rows give the same bits.

build_targets deduplicates the value table and packs each nonzero into one
u32 (column below, value id above) when both fit, else keeps a u32 column
array and a u16 value-id array.  EDG_ROW_FORMAT=split forces the second
format.  Both read the same table values in the same order, so H*v and the
batch must agree bit for bit, and each must still match the
reference (the golden fixtures) within the H*v tolerances.
"""
import numpy as np
import pytest

from conftest import golden_arrays, golden_cases, golden_model

import oracle as O

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-13


@pytest.fixture(scope="module")
def mods(cuda_device):
    from ed_code_gb300 import batch, lattice, sector

    return batch, lattice, sector


def _pair(sector, model, monkeypatch):
    packed = sector.GpuSector(model)
    assert packed.build_targets()
    monkeypatch.setenv("EDG_ROW_FORMAT", "split")
    split = sector.GpuSector(model)
    assert split.build_targets()
    monkeypatch.delenv("EDG_ROW_FORMAT")
    return packed, split


def _models(L):
    return [
        golden_model("sq6x4_k00", 0),
        golden_model("tri6x4_k10", 0),
        golden_model("tri4x3_relabel", 1),
        L.make_model(L.TorusSpec("triangular", 5, 4, Jz=1.1, J2=0.3, Ch=0.2), 0, 2, 1),
    ]


@pytest.mark.parametrize("which", range(4))
def test_packed_and_split_rows_agree_bitwise(mods, monkeypatch, which):
    _, L, sector = mods
    packed, split = _pair(sector, _models(L)[which], monkeypatch)
    assert packed.info["entry_bytes"] == 4 and split.info["entry_bytes"] == 6
    assert packed.info["n_values"] == split.info["n_values"] > 0
    assert packed.info["n_targets"] == split.info["n_targets"]
    assert split.info["device_bytes"] - packed.info["device_bytes"] == 2 * packed.info["n_targets"]
    v = O.splitmix_vector(packed.n_p, 31 + which)
    for lanes in (8, 16, 32):
        for pol in (1, 2):
            for pipe in (0, 1):
                packed.set_rows(lanes, pol, 0, pipe)
                split.set_rows(lanes, pol, 0, pipe)
                for dt in (np.complex128, np.complex64):
                    a = packed.sHv(v.astype(dt), dtype=dt)
                    b = split.sHv(v.astype(dt), dtype=dt)
                    assert np.array_equal(a, b), (lanes, pol, pipe, dt)


def test_value_table_is_deduplicated_at_gamma(mods):
    """Uniform couplings at k = 0: one phase class, so the table holds only the
    distinct pair coefficients -- a handful, far below pairs x variants."""
    _, L, sector = mods
    sec = sector.GpuSector(golden_model("sq6x4_k00", 0))
    assert sec.build_targets()
    assert sec.info["n_values"] <= 16
    assert sec.info["entry_bytes"] == 4


@pytest.mark.parametrize("name,idx", [("sq6x4_k00", 0), ("tri6x4_k10", 0)])
def test_split_rows_match_reference(mods, monkeypatch, name, idx):
    _, _, sector = mods
    monkeypatch.setenv("EDG_ROW_FORMAT", "split")
    sec = sector.GpuSector(golden_model(name, idx))
    assert sec.build_targets() and sec.info["entry_bytes"] == 6
    meta = golden_cases()[name]["sectors"][idx]
    g = golden_arrays(name)
    tag = f"s{idx}"
    for k, seed in enumerate(meta["vec_seeds"]):
        w = sec.sHv(O.splitmix_vector(sec.n_p, seed))
        if meta["full"]:
            ref = g[f"{tag}_w{k}"]
            assert np.abs(w - ref).max() / max(1.0, np.abs(ref).max()) <= FP64_TOL
        else:
            rows = g[f"{tag}_rows"]
            ref = g[f"{tag}_w{k}_at_rows"]
            assert np.abs(w[rows] - ref).max() / max(1.0, np.abs(ref).max()) <= FP64_TOL


def test_batch_mixes_formats(mods, monkeypatch):
    """One batch launch serves packed and split segments side by side: the same
    sector in either format gives the same eigenvalues bit for bit."""
    batch, _, sector = mods
    packed, split = _pair(sector, golden_model("tri6x4_k10", 0), monkeypatch)
    B = batch.BatchSolver(tile_rows=512)
    B.add(packed, n_ev=2, max_iterations=120, tol=0.0, seed=5, tag=0)
    B.add(split, n_ev=2, max_iterations=120, tol=0.0, seed=5, tag=1)
    res = {r["tag"]: r for r in B.run()}
    assert res[0]["status"] == 0 and res[1]["status"] == 0
    assert np.array_equal(res[0]["eigs"], res[1]["eigs"])
    assert np.array_equal(res[0]["residuals"], res[1]["residuals"])
    ref = golden_cases()["tri6x4_k10"]["sectors"][0]["ed2_eigs"][0]
    assert abs(res[0]["eigs"][0] - ref) <= 1e-9 * abs(ref)
