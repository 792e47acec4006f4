"""The serving loop: each request's result is the same alone and in the mix,
the eigenvalues meet the 1e-9 relative tolerance against the FP64 plain
solver, and admission keeps to the memory budget."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods(cuda_device):
    from ed_code_gb300 import batch, lattice, sector, serving

    return batch, lattice, sector, serving


@pytest.fixture(scope="module")
def stream(mods):
    serving = mods[3]
    return serving.make_stream(10, rate=400.0, seed=11, sizes=(20, 24))


# A segment's sums depend on the batch's tile size and lanes per row, so the
# alone runs share the choice the loop's tuner made (TUNED).
TUNED = {}


@pytest.fixture(scope="module")
def served(mods, stream):
    """The stream through the loop with the library's tuner choosing the
    batch's tiles; the alone runs below reuse its choice."""
    serving = mods[3]
    srv = serving.Server(max_iterations=300, res_tol=1e-6)
    out = srv.run(stream)
    srv.close()
    assert srv.tuned and srv.tuned["tile_rows"] in (256, 1024, 4096, 16384)
    TUNED.update(srv.tuned)
    return {s.rid: s for s in out}


def test_every_request_served(served, stream, mods):
    serving = mods[3]
    assert sorted(served) == [r.rid for r in stream]
    for s in served.values():
        assert s.status == 0 and s.converged and s.finished >= s.admitted >= 0
        assert len(s.eigs) >= 1
    summ = serving.summarize(list(served.values()))
    assert summ["p99_s"] >= summ["p50_s"] > 0 and summ["solves_per_s"] > 0


def test_alone_equals_in_mix(served, stream, mods):
    batch, lattice, sector, serving = mods
    for req in stream[:4]:
        sec = sector.GpuSector(lattice.make_model(req.spec, req.Sz, req.kx, req.ky))
        assert sec.build_targets()
        # the loop's batch: the tuner's tiles, partial reorthogonalisation (its default)
        B = batch.BatchSolver(tile_rows=TUNED["tile_rows"], lanes_per_row=TUNED["lanes_per_row"], check_every=10,
                              reorth=1)
        B.add(sec, n_ev=req.n_ev, max_iterations=min(300, sec.n_p), tol=1e-6, seed=1 + req.rid, tag=req.rid)
        alone = B.run()[0]
        mixed = served[req.rid]
        assert alone["iterations"] == mixed.iterations
        assert np.array_equal(alone["eigs"], mixed.eigs), (alone["eigs"], mixed.eigs)


def test_eigenvalues_match_plain_fp64(served, stream, mods):
    _, lattice, sector, _ = mods
    for req in stream[:5]:
        sec = sector.GpuSector(lattice.make_model(req.spec, req.Sz, req.kx, req.ky))
        eigs, _, _ = sec.solve_plain(n_ev=max(req.n_ev, 4), iterations=200, ncycles=10, tol=1e-12)
        levels = []
        for x in eigs:
            if not levels or abs(x - levels[-1]) > 1e-9 * abs(x):
                levels.append(x)
        got = served[req.rid].eigs
        levels = np.array(levels)
        assert abs(got[0] - levels[0]) <= 1e-9 * abs(levels[0]), (req, got, levels)
        for x in got[1:]:
            if x <= levels[-1]:  # levels the plain run reached
                assert np.min(np.abs(levels - x)) <= 1e-9 * abs(x), (req, got, levels)


def test_admission_keeps_to_the_budget(mods, stream):
    serving = mods[3]
    one = max(serving.estimate_bytes(r, 300) for r in stream[:6])
    srv = serving.Server(hbm_budget=one, max_iterations=300, res_tol=1e-6)
    out = srv.run(stream[:6])
    srv.close()
    assert len(out) == 6
    assert srv.peak_live == 1 and srv.peak_bytes <= one


def test_bad_requests_are_reported_and_the_rest_unchanged(served, stream, mods):
    """A malformed request and a cancelled one inside the stream come back
    with their status; every other request has the bits it has without them."""
    serving = mods[3]
    bad = serving.Request(900, stream[2].arrival, serving.L.TorusSpec("square", 5, 4), 0.0, 9, 0, 1)  # kx >= Lx
    extra = serving.Request(901, stream[3].arrival, stream[3].spec, stream[3].Sz, stream[3].kx, stream[3].ky, 1)
    srv = serving.Server(max_iterations=300, res_tol=1e-6, tile_rows=TUNED["tile_rows"],
                         lanes_per_row=TUNED["lanes_per_row"], tune=False)
    srv.cancel(901)  # withdrawn before it arrives
    out = {s.rid: s for s in srv.run(list(stream) + [bad, extra])}
    srv.close()
    assert out[900].status == serving.REJECTED_INVALID and "momentum" in out[900].reason
    assert out[901].status == serving.CANCELLED
    for rid, s in served.items():
        assert out[rid].ok and np.array_equal(out[rid].eigs, s.eigs)
