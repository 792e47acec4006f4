"""Host side of the serving loop (no GPU): the seeded request stream, the
footprint estimate, and the loop's admission and continuous batching run
against a simulated batch and clock."""
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


class _Clock:
    """Simulated time: every call moves it on a little, batch steps move it
    on by a step's length."""

    def __init__(self):
        self.t = 0.0

    def __call__(self):
        self.t += 1e-4
        return self.t


class _Sector:
    """Stand-in for GpuSector: models whose Jz is exactly 1.25 do not fit
    (their stored rows fail like a full device), everything else builds."""

    def __init__(self, model):
        self.n_p = 100
        self.closed = False
        self.fits = model.Jz != 1.25

    def build_targets(self):
        return self.fits

    def close(self):
        self.closed = True


def _fake_batch(clock, log):
    class _Batch:
        """Each segment finishes a fixed number of steps after it joins."""

        def __init__(self, **kw):
            self.left = {}
            self.cancelled = set()

        def add(self, sec, n_ev, max_iterations, tol, seed, tag):
            self.left[tag] = 40 if tag == 5 else 2 + tag % 3  # request 5 runs long
            log.append(("add", tag, len(self.left)))

        def step(self, n):
            clock.t += 0.05
            for k in self.left:
                self.left[k] -= 1

        def tune(self, steps=3):
            log.append(("tune", len(self.left)))
            return {"tile_rows": 1024, "lanes_per_row": 8, "ms_per_step": {}}

        def cancel(self, tag):
            self.left[tag] = 0  # reported by the next poll
            self.cancelled.add(tag)
            log.append(("cancel", tag))

        def poll(self):
            out = []
            for k in [k for k, v in self.left.items() if v <= 0]:
                self.left.pop(k)
                cancelled = k in self.cancelled
                log.append(("done", k))
                out.append({"tag": k, "eigs": np.zeros(0) if cancelled else np.array([-1.0 - k]),
                            "residuals": np.array([1e-7]), "iterations": 30, "converged": not cancelled,
                            "status": serving.CANCELLED if cancelled else 0})
            return out

        def close(self):
            pass

    return _Batch


def _run(monkeypatch, requests, budget, build_ahead=True, on_result=None, setup=None):
    clock, log = _Clock(), []
    monkeypatch.setattr(serving, "GpuSector", _Sector)
    monkeypatch.setattr(serving, "BatchSolver", _fake_batch(clock, log))
    srv = serving.Server(hbm_budget=budget, max_iterations=300, build_ahead=build_ahead)
    if setup:
        setup(srv, log)
    out = srv.run(requests, clock=clock, on_result=on_result)
    return srv, out, log


def test_loop_serves_every_request_once_in_arrival_order(monkeypatch):
    reqs = serving.make_stream(24, rate=50.0, seed=7, sizes=(20, 24))
    srv, out, log = _run(monkeypatch, reqs, budget=1 << 50)
    assert sorted(s.rid for s in out) == [r.rid for r in reqs]
    adds = [e[1] for e in log if e[0] == "add"]
    assert adds == [r.rid for r in sorted(reqs, key=lambda r: r.arrival)]
    for s in out:
        assert s.finished >= s.admitted >= s.arrival - 1e-9 and s.status == 0
        assert s.eigs[0] == -1.0 - s.rid


def test_loop_batches_continuously_within_the_budget(monkeypatch):
    reqs = serving.make_stream(30, rate=30.0, seed=8, sizes=(20, 24))
    # requests join while others are still running, and after some finished
    srv, out, log = _run(monkeypatch, reqs, budget=1 << 50)
    assert max(e[2] for e in log if e[0] == "add") > 1
    first_done = next(i for i, e in enumerate(log) if e[0] == "done")
    assert any(e[0] == "add" for e in log[first_done:])
    unlimited = srv.peak_live
    # a budget of two of the largest requests: the estimated bytes of the live
    # requests never exceed it, and it holds fewer live than no budget does
    big = max(serving.estimate_bytes(r, 300) for r in reqs)
    srv, out, _ = _run(monkeypatch, reqs, budget=2 * big)
    assert len(out) == len(reqs)
    assert srv.peak_bytes <= 2 * big and 1 <= srv.peak_live < unlimited


def test_a_request_larger_than_the_budget_still_runs_alone(monkeypatch):
    reqs = serving.make_stream(3, rate=100.0, seed=9, sizes=(24,))
    srv, out, _ = _run(monkeypatch, reqs, budget=1)
    assert len(out) == 3 and srv.peak_live == 1


def _bad(rid, arrival, **kw):
    base = dict(spec=serving.L.TorusSpec("square", 5, 4), Sz=0.0, kx=0, ky=0, n_ev=1)
    base.update(kw)
    return serving.Request(rid, arrival, **base)


def test_malformed_and_oversized_requests_are_rejected_alone(monkeypatch):
    """Odd N, |Sz| > N/2, a momentum out of range, nev out of range and a
    request whose stored rows do not fit come back rejected with a reason;
    every other request is served exactly as in a stream without them."""
    good = serving.make_stream(12, rate=40.0, seed=11, sizes=(20, 24))
    _, ref, _ = _run(monkeypatch, good, budget=1 << 50)
    t = good[3].arrival
    bad = [
        _bad(100, t, spec=serving.L.TorusSpec("square", 5, 3)),                 # 15 sites
        _bad(101, t + 1e-3, Sz=11.0),                                             # |Sz| > N/2
        _bad(102, t + 2e-3, Sz=0.5),                                              # not an allowed Sz for even N
        _bad(103, t + 3e-3, kx=5),                                                # kx >= Lx
        _bad(104, t + 4e-3, n_ev=0),
        _bad(105, t + 5e-3, spec=serving.L.TorusSpec("square", 5, 4, Jz=1.25)),  # rows do not fit
    ]
    for build_ahead in (True, False):
        _, out, log = _run(monkeypatch, good + bad, budget=1 << 50, build_ahead=build_ahead)
        by = {s.rid: s for s in out}
        assert sorted(by) == sorted(r.rid for r in good + bad)
        for r in bad[:5]:
            assert by[r.rid].status == serving.REJECTED_INVALID and by[r.rid].reason, by[r.rid]
            assert ("add", r.rid) not in [e[:2] for e in log]
        assert by[105].status == serving.REJECTED_NOMEM and "fit" in by[105].reason
        for s in ref:
            assert by[s.rid].ok and np.array_equal(by[s.rid].eigs, s.eigs)
        summ = serving.summarize(out)
        assert summ["solved"] == len(good) and summ["rejected"] == len(bad) and summ["cancelled"] == 0


def test_cancel_queued_and_running_requests(monkeypatch):
    """cancel() withdraws a request still queued (before it arrived) and one
    already in the batch; both come back as CANCELLED, the rest are unchanged."""
    reqs = serving.make_stream(16, rate=40.0, seed=12, sizes=(20,))
    _, ref, _ = _run(monkeypatch, reqs, budget=1 << 50)
    ref_by = {s.rid: s for s in ref}
    late = reqs[-1].rid
    holder = {}

    def on_result(s):
        # once two requests run together, cancel one of them at the next
        # result, and one that has not arrived yet
        log = holder["log"]
        added = [e[1] for e in log if e[0] == "add"]
        if "running" not in holder and 5 in added:  # request 5 runs for 40 steps
            holder["running"] = 5
            holder["srv"].cancel(5)
            holder["srv"].cancel(late)

    def setup(srv, log):
        holder["srv"] = srv
        holder["log"] = log

    _, out, log = _run(monkeypatch, reqs, budget=1 << 50, on_result=on_result, setup=setup)
    by = {s.rid: s for s in out}
    assert sorted(by) == [r.rid for r in reqs]
    assert by[late].status == serving.CANCELLED and ("add", late) not in [e[:2] for e in log]
    assert by[holder["running"]].status == serving.CANCELLED
    assert ("cancel", holder["running"]) in log
    for rid, s in by.items():
        if rid not in (late, holder["running"]):
            assert s.ok and np.array_equal(s.eigs, ref_by[rid].eigs)
    assert serving.summarize(out)["cancelled"] == 2


def test_batch_is_tuned_once_before_its_first_step(monkeypatch):
    reqs = serving.make_stream(10, rate=40.0, seed=13, sizes=(20,))
    srv, out, log = _run(monkeypatch, reqs, budget=1 << 50)
    tunes = [i for i, e in enumerate(log) if e[0] == "tune"]
    assert len(tunes) == 1 and tunes[0] > 0 and log[tunes[0]][1] >= 1
    assert srv.tuned["tile_rows"] == 1024 and len(out) == len(reqs)
