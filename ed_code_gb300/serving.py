"""A persistent request loop for sector diagonalisations (continuous batching).

Requests (lattice, Delta, J2, Jchi, Sz, momentum, nev) arrive over time.  The
loop admits them in arrival order while their estimated device footprint fits
the HBM budget, builds each one's sector with stored rows, and adds it as a
segment to one ``BatchSolver``; every call to ``BatchSolver.step`` advances
all admitted requests together, and a request leaves the batch (freeing its
memory for the next ones) as soon as its own tolerance is met.  Requests that
arrive while others are on the GPU join at the next step.  The reference has
no serving path: it diagonalises one input file's sectors one at a time.
"""
from __future__ import annotations

import dataclasses
import math
import time
from typing import Callable, Dict, List, Optional, Sequence

import numpy as np

from . import lattice as L
from .batch import BatchSolver
from .sector import GpuSector


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
    status: int

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


class Server:
    """Continuous-batching loop over one GPU.

    hbm_budget: device bytes the loop may hold for admitted requests (None:
    85% of the free memory when the loop starts).  res_tol: the batch's
    residual-bound tolerance relative to |theta|; with FP32 Krylov vectors and
    FP64 Rayleigh quotients 1e-6 gives eigenvalues within about 1e-10
    relative of the FP64 ones for these models (checked by the tests)."""

    def __init__(self, hbm_budget: Optional[int] = None, max_iterations: int = 300, res_tol: float = 1e-6,
                 tile_rows: int = 4096, lanes_per_row: int = 8, check_every: int = 10, max_active: int = 4096):
        if hbm_budget is None:
            import torch

            free, _ = torch.cuda.mem_get_info()
            hbm_budget = int(0.85 * free)
        self.budget = int(hbm_budget)
        self.max_iterations = int(max_iterations)
        self.res_tol = float(res_tol)
        self.check_every = int(check_every)
        self.max_active = int(max_active)
        self.batch = BatchSolver(tile_rows=tile_rows, lanes_per_row=lanes_per_row, check_every=check_every)
        self.peak_live = 0
        self.peak_bytes = 0
        self.create_seconds = 0.0   # sector construction (basis and stored rows)

    def run(self, requests: Sequence[Request], clock: Callable[[], float] = time.perf_counter,
            on_result: Optional[Callable[[Served], None]] = None) -> List[Served]:
        pending = sorted(requests, key=lambda r: r.arrival)
        queue: List[Request] = []
        live: Dict[int, tuple] = {}   # rid -> (request, sector, bytes, admitted)
        used = 0
        done: List[Served] = []
        t0 = clock()
        nxt = 0
        while nxt < len(pending) or queue or live:
            now = clock() - t0
            while nxt < len(pending) and pending[nxt].arrival <= now:
                queue.append(pending[nxt])
                nxt += 1
            # admission in arrival order, by estimated footprint
            while queue and len(live) < self.max_active:
                req = queue[0]
                need = estimate_bytes(req, self.max_iterations)
                if live and used + need > self.budget:
                    break
                queue.pop(0)
                tc = clock()
                model = L.make_model(req.spec, req.Sz, req.kx, req.ky, bowties=req.spec.ChCh != 0)
                sec = GpuSector(model)
                if not sec.build_targets():
                    raise MemoryError(f"request {req.rid}: stored rows do not fit")
                self.create_seconds += clock() - tc
                self.batch.add(sec, n_ev=req.n_ev, max_iterations=min(self.max_iterations, sec.n_p),
                               tol=self.res_tol, seed=1 + req.rid, tag=req.rid)
                live[req.rid] = (req, sec, need, clock() - t0)
                used += need
                self.peak_live = max(self.peak_live, len(live))
                self.peak_bytes = max(self.peak_bytes, used)
            if live:
                self.batch.step(self.check_every)
                for r in self.batch.poll():
                    req, sec, need, adm = live.pop(r["tag"])
                    s = Served(req.rid, req.arrival, adm, clock() - t0, sec.n_p, r["eigs"], r["residuals"],
                               r["iterations"], r["converged"], r["status"])
                    sec.close()
                    used -= need
                    done.append(s)
                    if on_result:
                        on_result(s)
            elif nxt < len(pending):
                time.sleep(max(0.0, min(0.01, pending[nxt].arrival - (clock() - t0))))
        return done

    def close(self) -> None:
        self.batch.close()


def summarize(served: Sequence[Served]) -> dict:
    lat = np.array([s.latency for s in served])
    span = max(s.finished for s in served) - min(s.arrival for s in served)
    return {"requests": len(served), "solves_per_s": len(served) / span if span > 0 else None,
            "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "makespan_s": span, "converged": int(sum(s.converged for s in served))}
