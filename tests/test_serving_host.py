"""Host side of the serving loop: the seeded request stream and the footprint
estimate (no GPU)."""
import math

import numpy as np

from ed_code_gb300 import serving


def test_stream_is_seeded_and_in_range():
    a = serving.make_stream(200, rate=200.0, seed=3)
    b = serving.make_stream(200, rate=200.0, seed=3)
    assert [(r.arrival, r.spec, r.Sz, r.kx, r.ky, r.n_ev) for r in a] == \
           [(r.arrival, r.spec, r.Sz, r.kx, r.ky, r.n_ev) for r in b]
    t = np.array([r.arrival for r in a])
    assert np.all(np.diff(t) > 0)
    assert 0.5 < t[-1] < 2.0  # about 200 arrivals at 200/s
    for r in a:
        assert r.n_sites in (20, 24, 28, 32)
        assert (r.spec.Lx, r.spec.Ly) == serving.SHAPES[r.n_sites]
        assert r.spec.lattice in ("triangular", "square")
        assert 0.5 <= r.spec.Jz <= 1.5 and 0.0 <= r.spec.Ch <= 0.3
        assert r.Sz in (0.0, 1.0) and r.n_ev in (1, 4)
        assert 0 <= r.kx < r.spec.Lx and 0 <= r.ky < r.spec.Ly
    assert {r.n_sites for r in a} == {20, 24, 28, 32}
    assert serving.make_stream(50, 200.0, seed=4)[0].arrival != a[0].arrival


def test_footprint_estimate_grows_with_size_and_steps():
    r = serving.make_stream(1, 1.0, seed=1)[0]
    small = serving.Request(0, 0.0, serving.L.TorusSpec("square", 5, 4), 0.0, 0, 0, 1)
    big = serving.Request(1, 0.0, serving.L.TorusSpec("triangular", 8, 4), 0.0, 0, 0, 4)
    assert serving.estimate_bytes(small, 100) < serving.estimate_bytes(small, 300) < serving.estimate_bytes(big, 300)
    n_p = math.comb(32, 16) / 32
    # at least the FP32 Krylov vectors of 300 steps
    assert serving.estimate_bytes(big, 300) > n_p * 8 * 300
    assert serving.estimate_bytes(r, 300) > 0


def test_sweep_sort_matches_the_reference_rules():
    from ed_code_gb300 import sweep as W

    mk = lambda i, E, Sz: W.Level(i, E, 0.0, 0.0, Sz, 0, 0)
    lv = [mk(0, -1.0, 1.0), mk(1, -2.0, 0.0), mk(2, -1.0, 0.0), mk(3, -1.0 + 4e-16, 2.0), mk(4, -1.0 + 4e-16, 0.5),
          mk(5, -3.0, 3.0)]
    out = W.sort_levels(lv)
    assert [q.id for q in out][:2] == [5, 1]
    assert all(a.En <= b.En + 1e-15 for a, b in zip(out, out[1:]))
    # within 1e-15 of each other the lowest Sz comes first
    tied = out[2:]
    assert tied[0].Sz == 0.0
    assert W.sector_list(W.L.TorusSpec("square", 4, 2))[:3] == [(4, 0, 0), (4, 0, 1), (4, 1, 0)]
    assert {s[0] for s in W.sector_list(W.L.TorusSpec("square", 4, 2))} == set(range(4, 9))
    assert {s[0] for s in W.sector_list(W.L.TorusSpec("square", 4, 2), Sz=1.0)} == {5}
    txt = W.table(out, 8, 1.0, 0.0)
    assert "ID\tEnergies\tEnergies/site\tSz\tpx\tpy\tJz\tJ2\tEnergies-E0" in txt
