"""A persistent request loop for sector diagonalisations (continuous batching).

Requests (lattice, Delta, J2, Jchi, Sz, momentum, nev) arrive over time.  The
loop admits them in arrival order while their estimated device footprint fits
the HBM budget, builds each one's sector with stored rows (on a builder
thread, so the construction overlaps the batch steps of the requests already
running), and adds it as a segment to one ``BatchSolver``; every call to
``BatchSolver.step`` advances all admitted requests together, and a request
leaves the batch (freeing its memory for the next ones) as soon as its own
tolerance is met.  Requests that arrive while others are on the GPU join at
the next step.

Failures stay with the request that caused them: a malformed request (odd
number of sites, Sz or momentum out of range, nev out of range) is rejected
before anything is built, a request whose sector or stored rows do not fit
is rejected with EDG_ERR_NOMEM, and ``cancel(rid)`` withdraws a queued or
running request; each comes back as a ``Served`` record with its status and
reason, and the other requests' results do not change.  The reference has no
serving path: it diagonalises one input file's sectors one at a time and
exits on a bad sector (Lanczos_sector.cpp:51-55, 93-97).
"""
from __future__ import annotations

import dataclasses
import math
import queue as _queue
import threading
import time
from typing import Callable, Dict, List, Optional, Sequence

import numpy as np

from . import _native as N
from . import lattice as L
from .batch import BatchSolver
from .sector import GpuSector

CANCELLED = 8          # EDG_ERR_CANCELLED
REJECTED_INVALID = 1   # EDG_ERR_INVALID
REJECTED_NOMEM = 5     # EDG_ERR_NOMEM


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float            # seconds after the start of the stream
    spec: L.TorusSpec
    Sz: float
    kx: int
    ky: int
    n_ev: int
    tol: float = 1e-9         # eigenvalue tolerance the request asks for

    @property
    def n_sites(self) -> int:
        return self.spec.n_sites


SHAPES = {20: (5, 4), 24: (6, 4), 28: (7, 4), 32: (8, 4)}


def make_stream(n_requests: int, rate: float, seed: int = 3, sizes: Sequence[int] = (20, 24, 28, 32),
                nevs: Sequence[int] = (1, 4)) -> List[Request]:
    """Poisson arrivals at `rate` per second; each request draws its size, a
    triangular or square torus, Delta ~ U[0.5, 1.5], Jchi ~ U[0, 0.3],
    Sz in {0, 1}, a momentum and nev, all from one seeded generator."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for rid in range(n_requests):
        t += rng.exponential(1.0 / rate)
        N = int(rng.choice(list(sizes)))
        Lx, Ly = SHAPES[N]
        lat = "triangular" if rng.random() < 0.5 else "square"
        spec = L.TorusSpec(lat, Lx, Ly, Jz=float(rng.uniform(0.5, 1.5)), Ch=float(rng.uniform(0.0, 0.3)))
        out.append(Request(rid, t, spec, float(rng.integers(0, 2)), int(rng.integers(0, Lx)), int(rng.integers(0, Ly)),
                           int(rng.choice(list(nevs)))))
    return out


def validate(req: Request) -> Optional[str]:
    """Why the request cannot be served, or None.  The checks the reference
    makes before building a sector (Lanczos_sector.cpp:45-55) plus this
    library's limits."""
    N_ = req.n_sites
    if N_ % 2:
        return f"odd number of sites ({N_})"
    n_up = N_ / 2 + req.Sz
    if abs(req.Sz) > N_ / 2 or abs(n_up - round(n_up)) > 1e-9:
        return f"Sz = {req.Sz} is not an allowed magnetisation for {N_} spins"
    if not (0 <= req.kx < req.spec.Lx and 0 <= req.ky < req.spec.Ly):
        return f"momentum ({req.kx}, {req.ky}) outside [0,{req.spec.Lx})x[0,{req.spec.Ly})"
    if not (1 <= req.n_ev <= 32):
        return f"nev = {req.n_ev} outside 1..32"
    return None


def estimate_bytes(req: Request, max_iterations: int) -> int:
    """Device bytes a request will hold at most: basis, stored rows (about 6
    bytes per anti-aligned bond and row, 16 per row), FP32 Krylov vectors, and
    the FP64 Ritz vectors of its finish."""
    N = req.n_sites
    n_up = int(round(N / 2 + req.Sz))
    n_p = math.comb(N, n_up) / N * 1.05 + 64
    n_bonds = 3 * N if req.spec.lattice == "triangular" else 2 * N
    per_row = 8 + 1 + 16 + 6 * 0.55 * n_bonds + 8 * (max_iterations + 3) + 16 * (req.n_ev + 5)
    return int(n_p * per_row) + (64 << 20)


@dataclasses.dataclass
class Served:
    rid: int
    arrival: float
    admitted: float
    finished: float
    n_p: int
    eigs: np.ndarray
    residuals: np.ndarray
    iterations: int
    converged: bool
    status: int            # 0, or the EDG_ERR_* code that ended the request
    reason: str = ""

    @property
    def latency(self) -> float:
        return self.finished - self.arrival

    @property
    def ok(self) -> bool:
        return self.status == 0


class Server:
    """Continuous-batching loop over one GPU.

    hbm_budget: device bytes the loop may hold for admitted requests (None:
    85% of the free memory when the loop starts).  res_tol: the batch's
    residual-bound tolerance relative to |theta|; with FP32 Krylov vectors and
    FP64 Rayleigh quotients 1e-6 gives eigenvalues within about 1e-10
    relative of the FP64 ones for these models (checked by the tests).
    build_ahead: build admitted requests' sectors on a builder thread while
    the batch steps (False: build them in the loop).  tune: before the first
    step of each run(), time the batch's tile sizes and lanes per row on the
    requests admitted first (edg_batch_tune) and keep the fastest; ``tuned`` then
    holds the choice (otherwise tile_rows and lanes_per_row stay).  reorth:
    the batch's reorthogonalisation (1, the default: partial; 0: every
    step)."""

    def __init__(self, hbm_budget: Optional[int] = None, max_iterations: int = 300, res_tol: float = 1e-6,
                 tile_rows: int = 4096, lanes_per_row: int = 8, check_every: int = 10, max_active: int = 4096,
                 build_ahead: bool = True, tune: bool = True, reorth: int = 1):
        if hbm_budget is None:
            import torch

            free, _ = torch.cuda.mem_get_info()
            hbm_budget = int(0.85 * free)
        self.budget = int(hbm_budget)
        self.max_iterations = int(max_iterations)
        self.res_tol = float(res_tol)
        self.check_every = int(check_every)
        self.max_active = int(max_active)
        self.build_ahead = bool(build_ahead)
        self.tune = bool(tune)
        self.tuned: Optional[dict] = None
        self.batch = BatchSolver(tile_rows=tile_rows, lanes_per_row=lanes_per_row, check_every=check_every,
                                 reorth=reorth)
        self.peak_live = 0
        self.peak_bytes = 0
        self.create_seconds = 0.0   # sector construction (basis and stored rows)
        self._cancel: set = set()
        self._lock = threading.Lock()

    def cancel(self, rid: int) -> None:
        """Withdraw request rid (safe from any thread): it is dropped if still
        queued or being built, or taken out of the batch if running; its
        record comes back with status CANCELLED."""
        with self._lock:
            self._cancel.add(int(rid))

    def _build(self, req: Request):
        """The request's sector with stored rows; (sector, None) or (None, (status, reason))."""
        try:
            model = L.make_model(req.spec, req.Sz, req.kx, req.ky, bowties=req.spec.ChCh != 0)
            sec = GpuSector(model)
        except N.EdgError as e:
            return None, (e.code, str(e))
        except (ValueError, KeyError) as e:
            return None, (REJECTED_INVALID, str(e))
        try:
            if not sec.build_targets():
                sec.close()
                return None, (REJECTED_NOMEM, "the sector's stored rows do not fit in device memory")
        except N.EdgError as e:
            sec.close()
            return None, (e.code, str(e))
        return sec, None

    def run(self, requests: Sequence[Request], clock: Callable[[], float] = time.perf_counter,
            on_result: Optional[Callable[[Served], None]] = None) -> List[Served]:
        pending = sorted(requests, key=lambda r: r.arrival)
        if self.tune:
            self.tuned = None  # each stream is tuned on its own first requests
        queue: List[Request] = []
        live: Dict[int, tuple] = {}       # rid -> (request, sector, bytes, admitted)
        building: Dict[int, tuple] = {}   # rid -> (request, bytes, admitted)
        used = 0
        done: List[Served] = []
        t0 = clock()
        nxt = 0
        build_q: "_queue.Queue" = _queue.Queue()
        ready: "_queue.Queue" = _queue.Queue()
        stash: list = []   # built sectors taken from `ready` while waiting
        builder = None

        def emit(s: Served):
            done.append(s)
            if on_result:
                on_result(s)

        def fail(req: Request, status: int, reason: str, adm: float):
            now = clock() - t0
            emit(Served(req.rid, req.arrival, adm, now, 0, np.zeros(0), np.zeros(0), 0, False, status, reason))

        def build_loop():
            while True:
                req = build_q.get()
                if req is None:
                    return
                tc = time.perf_counter()
                sec, err = self._build(req)
                ready.put((req, sec, err, time.perf_counter() - tc))

        if self.build_ahead:
            builder = threading.Thread(target=build_loop, name="sector-builder", daemon=True)
            builder.start()
        try:
            while nxt < len(pending) or queue or live or building:
                now = clock() - t0
                while nxt < len(pending) and pending[nxt].arrival <= now:
                    queue.append(pending[nxt])
                    nxt += 1
                # cancellations: queued ones leave now, running ones through the batch
                with self._lock:
                    cancel, self._cancel = self._cancel, set()
                for rid in cancel:
                    q = next((r for r in queue if r.rid == rid), None)
                    if q is not None:
                        queue.remove(q)
                        fail(q, CANCELLED, "cancelled while queued", now)
                    elif rid in live:
                        self.batch.cancel(rid)
                    elif rid in building or any(r.rid == rid for r in pending[nxt:]):
                        with self._lock:
                            self._cancel.add(rid)  # act when it is built or has arrived
                # admission in arrival order, by estimated footprint
                while queue and len(live) + len(building) < self.max_active:
                    req = queue[0]
                    why = validate(req)
                    if why is not None:
                        queue.pop(0)
                        fail(req, REJECTED_INVALID, why, clock() - t0)
                        continue
                    need = estimate_bytes(req, self.max_iterations)
                    if (live or building) and used + need > self.budget:
                        break
                    queue.pop(0)
                    used += need
                    building[req.rid] = (req, need, clock() - t0)
                    if self.build_ahead:
                        build_q.put(req)
                    else:
                        tc = time.perf_counter()
                        sec, err = self._build(req)
                        ready.put((req, sec, err, time.perf_counter() - tc))
                # built sectors join the batch, in the order they were built
                while True:
                    if stash:
                        req, sec, err, dt = stash.pop(0)
                    else:
                        try:
                            req, sec, err, dt = ready.get_nowait()
                        except _queue.Empty:
                            break
                    self.create_seconds += dt
                    _, need, adm = building.pop(req.rid)
                    with self._lock:
                        was_cancelled = req.rid in self._cancel
                        self._cancel.discard(req.rid)
                    if err is not None or was_cancelled:
                        used -= need
                        if sec is not None:
                            sec.close()
                        if was_cancelled:
                            fail(req, CANCELLED, "cancelled while its sector was built", adm)
                        else:
                            fail(req, err[0], err[1], adm)
                        continue
                    try:
                        self.batch.add(sec, n_ev=req.n_ev, max_iterations=min(self.max_iterations, sec.n_p),
                                       tol=self.res_tol, seed=1 + req.rid, tag=req.rid)
                    except N.EdgError as e:
                        used -= need
                        sec.close()
                        fail(req, e.code, str(e), adm)
                        continue
                    live[req.rid] = (req, sec, need, adm)
                    self.peak_live = max(self.peak_live, len(live))
                    self.peak_bytes = max(self.peak_bytes, used)
                if live:
                    if self.tune and self.tuned is None:
                        self.tuned = self.batch.tune()
                    self.batch.step(self.check_every)
                    for r in self.batch.poll():
                        req, sec, need, adm = live.pop(r["tag"])
                        st = r["status"]
                        s = Served(req.rid, req.arrival, adm, clock() - t0, sec.n_p, r["eigs"], r["residuals"],
                                   r["iterations"], r["converged"], st,
                                   "cancelled while running" if st == CANCELLED else "")
                        sec.close()
                        used -= need
                        emit(s)
                elif building:
                    try:  # nothing to step: wait for a sector to be built
                        stash.append(ready.get(timeout=0.05))
                    except _queue.Empty:
                        pass
                elif nxt < len(pending):
                    time.sleep(max(0.0, min(0.01, pending[nxt].arrival - (clock() - t0))))
        finally:
            if builder is not None:
                build_q.put(None)
                builder.join()
        return done

    def close(self) -> None:
        self.batch.close()


def summarize(served: Sequence[Served]) -> dict:
    """Solves/s and time-to-eigenvalue over the requests that were solved;
    rejected and cancelled ones are counted apart."""
    ok = [s for s in served if s.ok]
    lat = np.array([s.latency for s in ok]) if ok else np.zeros(1)
    span = (max(s.finished for s in ok) - min(s.arrival for s in ok)) if ok else 0.0
    return {"requests": len(served), "solved": len(ok), "solves_per_s": len(ok) / span if span > 0 else None,
            "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "makespan_s": span, "converged": int(sum(s.converged for s in ok)),
            "rejected": int(sum(s.status not in (0, CANCELLED) for s in served)),
            "cancelled": int(sum(s.status == CANCELLED for s in served))}
