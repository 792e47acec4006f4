"""Batched mixed-precision solves over the C ABI (edg_batch_*).

``BatchSolver`` advances many sectors' Lanczos runs together on one GPU: every
step of all live segments is one replay of a captured CUDA graph, segments
join and leave independently, and each segment stops on its own tolerance or
step limit.  The reference has no counterpart: it diagonalises one sector at a
time (``sector_lanczos`` in a loop over momenta, ED.cpp:120-131).
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, List, Optional

import numpy as np

from . import _native as N


class BatchSolver:
    def __init__(self, tile_rows: int = 1024, lanes_per_row: int = 8, check_every: int = 10, reorth: int = 0):
        """reorth: 0 reorthogonalises every step; 1 only where Simon's
        estimates of the lost orthogonality call for it (partial)."""
        h = C.c_void_p()
        opts = N.edg_batch_opts(int(tile_rows), int(lanes_per_row), int(check_every), int(reorth))
        N.check(N.lib().edg_batch_create(C.byref(opts), C.byref(h)))
        self._h = h
        self._sectors: Dict[int, object] = {}  # tag -> sector, kept alive until polled
        self._next_tag = 0

    @staticmethod
    def _request(n_ev, max_iterations, tol, seed, tag):
        return N.edg_batch_request(int(n_ev), int(max_iterations), float(tol), int(seed), int(tag))

    def footprint(self, sec, n_ev: int, max_iterations: int) -> int:
        """Device bytes the segment would take (vectors and scalars; the
        sector's own basis and stored rows are reported by the sector)."""
        b = C.c_int64()
        N.check(N.lib().edg_batch_footprint(sec._h, C.byref(self._request(n_ev, max_iterations, 0, 0, 0)),
                                            C.byref(b)))
        return int(b.value)

    def add(self, sec, n_ev: int, max_iterations: int = 300, tol: float = 0.0, seed: int = 1,
            tag: Optional[int] = None) -> int:
        """Queue a sector (it needs stored rows); returns the result's tag."""
        if tag is None:
            tag = self._next_tag
        self._next_tag = max(self._next_tag, int(tag)) + 1
        N.check(N.lib().edg_batch_add(self._h, sec._h, C.byref(self._request(n_ev, max_iterations, tol, seed, tag))))
        self._sectors[int(tag)] = sec
        return int(tag)

    def step(self, n_steps: int = 1) -> None:
        N.check(N.lib().edg_batch_step(self._h, int(n_steps)))

    def tune(self, steps: int = 3) -> dict:
        """edg_batch_tune: time the tile sizes and lanes per row on the
        segments added so far (before the first step), keep the fastest.
        Returns {"tile_rows", "lanes_per_row", "ms_per_step": {"RxL": ms}}."""
        t, l = C.c_int(), C.c_int()
        ms = np.zeros(8, np.float64)
        N.check(N.lib().edg_batch_tune(self._h, int(steps), C.byref(t), C.byref(l), ms.ctypes.data))
        trials = {f"{r}x{k}": round(float(ms[2 * i + j]), 3)
                  for i, r in enumerate((256, 1024, 4096, 16384)) for j, k in enumerate((8, 16))}
        return {"tile_rows": t.value, "lanes_per_row": l.value, "ms_per_step": trials}

    def cancel(self, tag: int) -> None:
        """Withdraw a live segment (edg_batch_cancel); its result comes back
        from poll() with status EDG_ERR_CANCELLED."""
        N.check(N.lib().edg_batch_cancel(self._h, int(tag)))

    def poll(self) -> List[dict]:
        out = []
        buf = (N.edg_batch_result * 64)()
        while True:
            n = C.c_int()
            N.check(N.lib().edg_batch_poll(self._h, buf, 64, C.byref(n)))
            for r in buf[: n.value]:
                k = r.n_found
                out.append({"tag": int(r.tag), "status": int(r.status), "n_found": k,
                            "iterations": int(r.iterations), "converged": bool(r.converged),
                            "reorth_steps": int(r.reorth_steps),
                            "eigs": np.array(r.eigs[:k]), "ritz": np.array(r.ritz[:k]),
                            "residuals": np.array(r.residuals[:k])})
                self._sectors.pop(int(r.tag), None)
            if n.value < 64:
                return out

    def info(self) -> dict:
        a, b, s = C.c_int(), C.c_int64(), C.c_int64()
        N.check(N.lib().edg_batch_info(self._h, C.byref(a), C.byref(b), C.byref(s)))
        return {"active": a.value, "device_bytes": b.value, "steps": s.value}

    def timers(self) -> dict:
        t = np.zeros(5, np.float64)
        N.check(N.lib().edg_batch_timers(self._h, t.ctypes.data))
        return dict(zip(("add", "step", "finish", "release", "rebuild"), (float(x) for x in t)))

    def run(self, chunk: int = 10) -> List[dict]:
        """Step until no segment is left; return every result."""
        out = []
        while self.info()["active"]:
            self.step(chunk)
            out += self.poll()
        return out + self.poll()

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().edg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
