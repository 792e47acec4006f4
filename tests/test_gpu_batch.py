"""Batched solves (edg_batch_*) against the reference's eigenvalues, and the
same result for a sector alone and in a mix that changes around it.

Target: |dE|/|E| <= 1e-9 against the eigenvalues the reference printed
(ED2, FP64), with FP32 Krylov vectors and FP64 Rayleigh quotients.
"""
import numpy as np
import pytest

from conftest import golden_cases, golden_model

pytestmark = pytest.mark.gpu

REL_TOL = 1e-9


@pytest.fixture(scope="module")
def mods(cuda_device):
    from ed_code_gb300 import batch, sector

    return batch, sector


def distinct(levels, tol=1e-9):
    out = []
    for x in levels:
        if not out or abs(x - out[-1]) > tol * abs(x):
            out.append(x)
    return np.array(out)


def stored_sector(sector, name, idx):
    sec = sector.GpuSector(golden_model(name, idx))
    assert sec.build_targets()
    return sec


CASES = [("sq4x4", 0, 3), ("sq4x4_j2", 0, 3), ("sq4x4_j2", 1, 3), ("sq4x4_phase_sz1", 0, 3), ("tri4x3", 0, 3),
         ("tri4x3", 4, 3), ("tri4x3_relabel", 1, 2), ("sq6x4_k00", 0, 3), ("tri6x4_k10", 0, 2)]


@pytest.mark.parametrize("reorth", [0, 1])
def test_batch_matches_reference(mods, reorth):
    """Every step reorthogonalised (0) or partially (1): the same eigenvalues
    to 1e-9; the partial form reorthogonalises on fewer steps."""
    batch, sector = mods
    B = batch.BatchSolver(tile_rows=512, reorth=reorth)
    secs = {}
    for k, (name, idx, n_ev) in enumerate(CASES):
        secs[k] = stored_sector(sector, name, idx)
        B.add(secs[k], n_ev=n_ev, max_iterations=200, tol=0.0, seed=1, tag=k)
    res = {r["tag"]: r for r in B.run()}
    assert sorted(res) == list(range(len(CASES)))
    for k, (name, idx, n_ev) in enumerate(CASES):
        r = res[k]
        assert r["status"] == 0, r
        ref = distinct(golden_cases()[name]["sectors"][idx]["ed2_eigs"])
        n = min(n_ev, len(ref))
        assert r["n_found"] >= n, (name, r)
        rel = np.abs(r["eigs"][:n] - ref[:n]) / np.abs(ref[:n])
        assert rel.max() <= REL_TOL, (name, r["eigs"], ref[:n])
        assert r["iterations"] == min(200, secs[k].n_p)
        if reorth == 0:
            assert r["reorth_steps"] == r["iterations"], r
        elif r["iterations"] >= 150:
            assert 0 < r["reorth_steps"] < r["iterations"], (name, r["reorth_steps"])


@pytest.mark.parametrize("reorth", [0, 1])
def test_alone_equals_in_mix(mods, reorth):
    """A segment's arithmetic reads only its own tiles: joining a batch whose
    composition changes before, during and after it gives the same bits."""
    batch, sector = mods
    a = stored_sector(sector, "sq6x4_k00", 0)
    B1 = batch.BatchSolver(tile_rows=512, reorth=reorth)
    B1.add(a, n_ev=2, max_iterations=120, tol=0.0, seed=7, tag=0)
    alone = B1.run()[0]
    B2 = batch.BatchSolver(tile_rows=512, reorth=reorth)
    others = [stored_sector(sector, "sq4x4", 0), stored_sector(sector, "tri6x4_k10", 0),
              stored_sector(sector, "sq4x4_j2", 1)]
    B2.add(others[0], n_ev=3, max_iterations=60, tol=0.0, seed=3, tag=10)
    B2.add(others[1], n_ev=2, max_iterations=150, tol=0.0, seed=4, tag=11)
    B2.step(37)
    B2.add(a, n_ev=2, max_iterations=120, tol=0.0, seed=7, tag=0)
    B2.step(15)
    B2.add(others[2], n_ev=3, max_iterations=40, tol=0.0, seed=5, tag=12)
    mixed = {r["tag"]: r for r in B2.run()}
    assert set(mixed) == {0, 10, 11, 12}
    assert mixed[0]["iterations"] == alone["iterations"] == 120
    assert np.array_equal(mixed[0]["eigs"], alone["eigs"])
    assert np.array_equal(mixed[0]["residuals"], alone["residuals"])
    assert mixed[0]["reorth_steps"] == alone["reorth_steps"]


@pytest.mark.parametrize("reorth", [0, 1])
def test_tolerance_stops_early(mods, reorth):
    batch, sector = mods
    sec = stored_sector(sector, "sq6x4_k00", 0)
    B = batch.BatchSolver(tile_rows=1024, check_every=5, reorth=reorth)
    B.add(sec, n_ev=2, max_iterations=400, tol=1e-6, seed=1)
    r = B.run()[0]
    assert r["converged"] and r["iterations"] < 400, r
    ref = distinct(golden_cases()["sq6x4_k00"]["sectors"][0]["ed2_eigs"])[:2]
    assert np.max(np.abs(r["eigs"][:2] - ref) / np.abs(ref)) <= REL_TOL, (r, ref)


def test_batch_rejects_bad_requests(mods):
    batch, sector = mods
    from ed_code_gb300._native import EdgError

    B = batch.BatchSolver()
    plain = sector.GpuSector(golden_model("tri4x3", 0))
    with pytest.raises(EdgError, match="stored rows"):
        B.add(plain, n_ev=2)
    assert plain.build_targets()
    with pytest.raises(EdgError, match="n_ev"):
        B.add(plain, n_ev=0)
    with pytest.raises(EdgError, match="max_iterations"):
        B.add(plain, n_ev=1, max_iterations=1000)
    assert B.info()["active"] == 0
    assert B.footprint(plain, 2, 50) > 0
    with pytest.raises(EdgError, match="reorth"):
        batch.BatchSolver(reorth=2)


@pytest.mark.parametrize("reorth", [0, 1])
def test_large_segment_matches_single_sector_solver(mods, reorth):
    """A segment of 5.2e6 rows (tiles of 4096, the Gram-Schmidt dots summed
    per tile by one warp per Krylov vector): its levels agree with the
    single-sector FP32 solver with full reorthogonalisation (itself within
    1e-14 of plain FP64 on this lattice) to 1e-9."""
    from ed_code_gb300 import lattice as L

    batch, sector = mods
    sec = sector.GpuSector(L.make_model(L.TorusSpec("triangular", 6, 5, Jz=0.8, Ch=0.2), 0, 2, 3, bowties=False))
    assert sec.n_p >= 1 << 20 and sec.build_targets()
    ref = sec.solve_mixed(n_ev=3, iterations=150, reorth_every=1, seed=2)["eigs"]
    B = batch.BatchSolver(tile_rows=4096, reorth=reorth)
    B.add(sec, n_ev=3, max_iterations=150, tol=0.0, seed=2, tag=0)
    r = B.run()[0]
    assert r["status"] == 0 and r["n_found"] >= 3, r
    rel = np.abs(r["eigs"][:3] - ref[:3]) / np.abs(ref[:3])
    assert rel.max() <= REL_TOL, (r["eigs"], ref, r["reorth_steps"])


def test_cancel_releases_a_segment_and_leaves_the_others(mods):
    """edg_batch_cancel: the withdrawn segment comes back as EDG_ERR_CANCELLED
    with no levels and its memory released; the segments beside it finish
    with the bits they have without it."""
    batch, sector = mods
    a = stored_sector(sector, "sq6x4_k00", 0)
    b = stored_sector(sector, "tri6x4_k10", 0)
    B1 = batch.BatchSolver(tile_rows=512)
    B1.add(a, n_ev=2, max_iterations=120, tol=0.0, seed=7, tag=0)
    alone = B1.run()[0]
    B2 = batch.BatchSolver(tile_rows=512)
    B2.add(a, n_ev=2, max_iterations=120, tol=0.0, seed=7, tag=0)
    B2.add(b, n_ev=2, max_iterations=120, tol=0.0, seed=8, tag=1)
    B2.step(30)
    before = B2.info()["device_bytes"]
    B2.cancel(1)
    assert B2.info()["device_bytes"] < before and B2.info()["active"] == 1
    res = {r["tag"]: r for r in B2.run()}
    assert res[1]["status"] == 8 and res[1]["n_found"] == 0
    assert res[0]["status"] == 0 and np.array_equal(res[0]["eigs"], alone["eigs"])
    with pytest.raises(Exception):
        B2.cancel(5)


def test_tuner_keeps_results_of_an_untuned_batch(mods):
    """edg_batch_tune times the tile and lane choices on the segments, then
    puts them back at their start: the tuned batch returns the bits of a
    fresh batch created with the chosen options."""
    batch, sector = mods
    secs = [stored_sector(sector, n, i) for n, i, _ in CASES[:6]]
    B = batch.BatchSolver()
    for k, sec in enumerate(secs):
        B.add(sec, n_ev=2, max_iterations=100, tol=0.0, seed=3 + k, tag=k)
    choice = B.tune(steps=2)
    assert choice["tile_rows"] in (256, 1024, 4096, 16384) and choice["lanes_per_row"] in (8, 16)
    assert len(choice["ms_per_step"]) == 8 and all(v > 0 for v in choice["ms_per_step"].values())
    tuned = {r["tag"]: r for r in B.run()}
    B2 = batch.BatchSolver(tile_rows=choice["tile_rows"], lanes_per_row=choice["lanes_per_row"])
    for k, sec in enumerate(secs):
        B2.add(sec, n_ev=2, max_iterations=100, tol=0.0, seed=3 + k, tag=k)
    fresh = {r["tag"]: r for r in B2.run()}
    for k in range(len(secs)):
        assert np.array_equal(tuned[k]["eigs"], fresh[k]["eigs"]), k
    B3 = batch.BatchSolver()
    B3.add(secs[0], n_ev=2, max_iterations=100, tol=0.0, seed=3, tag=0)
    B3.step(1)
    with pytest.raises(Exception):
        B3.tune()
