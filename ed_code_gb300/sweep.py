"""All-sectors sweep: every (Sz, kx, ky) sector of one Hamiltonian, solved as
segments of one batch, levels sorted by energy.

Counterpart of the reference's full sweep (ARPACK, ARPACK_full_eigs.cpp:169-279):
the same sector loop (n_ones from N/2 up to N, or the one Sz asked for; every
momentum), the dense path for sectors with n_p <= n_ev + 1, and the same
ordering of the collected levels (pVector::sort_by_En, pClasses.cpp:125-208):
ascending energy, the lower Sz first among equal energies.  One difference:
Lanczos with one start vector returns each level of a sector once, where
ARPACK returns degenerate copies.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, List, Optional, Sequence

from . import _native as N
from . import lattice as L
from . import replicas as R
from .batch import BatchSolver
from .sector import GpuSector

TIE = 10e-16  # the reference's `pres` (global.h:20)


@dataclasses.dataclass
class Level:
    id: int
    En: float
    px: float
    py: float
    Sz: float
    kx: int
    ky: int


def sort_levels(levels: Sequence[Level]) -> List[Level]:
    """Ascending energy; among exactly equal energies the lower Sz first; then,
    within |dE| < 1e-15, the lowest Sz moved to the front (sort_by_Sz)."""
    E = sorted(levels, key=lambda q: (q.En, q.Sz))
    for i in range(len(E)):
        tE, tSz, k = E[i].En, E[i].Sz, i
        j = i
        while j < len(E) and abs(E[j].En - tE) < TIE:
            if tSz > E[j].Sz:
                k, tSz = j, E[j].Sz
            j += 1
        E[k], E[i] = E[i], E[k]
    return E


def sector_list(spec: L.TorusSpec, Sz: Optional[float] = None):
    """(n_ones, kx, ky) in the reference's loop order."""
    n = spec.n_sites
    lo = n // 2 if n % 2 == 0 else (n + 1) // 2
    hi = n
    if Sz is not None and Sz > -1.0:
        lo += int(Sz)
        hi = lo
    return [(n_ones, kx, ky) for n_ones in range(lo, hi + 1) for kx in range(spec.Lx) for ky in range(spec.Ly)]


def sweep(spec: L.TorusSpec, Sz: Optional[float] = None, n_ev: int = 4, max_iterations: int = 300,
          res_tol: float = 1e-6, hbm_budget: Optional[int] = None, seed: int = 1,
          distributed: bool = False, tune: bool = True) -> List[Level]:
    """Lowest levels of every sector, sorted as the reference sorts them.

    distributed: with a process group up (one rank per GPU), each rank solves
    every world-th sector and the levels are collected on every rank.
    tune: pick the batch's tile size and lanes per row with the library's
    autotuner (edg_batch_tune) on each group of sectors before it runs."""
    if hbm_budget is None:
        import torch

        hbm_budget = int(0.8 * torch.cuda.mem_get_info()[0])
    n = spec.n_sites
    per_sector = {}  # loop position -> ascending levels of that sector
    batch = BatchSolver()
    live = {}
    used = 0

    def drain():
        nonlocal used
        if tune and live:
            batch.tune()
        for r in batch.run():
            sec, meta, need = live.pop(r["tag"])
            N.check(r["status"])
            per_sector[r["tag"]] = [Level(0, float(E), *meta) for E in sorted(r["eigs"])]
            sec.close()
            used -= need
        assert not live

    rank, world = 0, 1
    if distributed:
        import torch.distributed as dist

        if dist.is_initialized():
            rank, world = dist.get_rank(), dist.get_world_size()
    for tag, (n_ones, kx, ky) in R.share(list(enumerate(sector_list(spec, Sz))), rank, world):
        sz = 0.5 * n_ones - 0.5 * (n - n_ones)
        meta = (2 * kx * math.pi / spec.Lx, 2 * ky * math.pi / spec.Ly, sz, kx, ky)
        try:
            sec = GpuSector(L.make_model(spec, sz, kx, ky, bowties=spec.ChCh != 0))
        except N.EdgError as e:
            if e.code == 3:  # EDG_ERR_EMPTY: the reference skips empty sectors too
                continue
            raise
        if sec.n_p <= n_ev + 1 or sec.n_p < 3:
            eigs, _, _ = sec.solve_plain(n_ev=sec.n_p, dense_threshold=max(sec.n_p, 1))
            per_sector[tag] = [Level(0, float(E), *meta) for E in sorted(eigs)]
            sec.close()
            continue
        if not sec.build_targets():
            raise MemoryError(f"sector ({sz}, {kx}, {ky}): stored rows do not fit")
        need = batch.footprint(sec, n_ev, max_iterations) + sec.info["device_bytes"]
        if live and used + need > hbm_budget:
            drain()
        batch.add(sec, n_ev=n_ev, max_iterations=min(max_iterations, sec.n_p), tol=res_tol, seed=seed, tag=tag)
        live[tag] = (sec, meta, need)
        used += need
    if live:
        drain()
    batch.close()
    if world > 1:
        per_sector = R.merge(per_sector)
    return assemble(per_sector)


def assemble(per_sector: Dict[int, List[Level]]) -> List[Level]:
    """Levels of all sectors ({loop position: levels}) in the reference's
    order, ids counting the levels in sector-loop order as its push_back does."""
    levels: List[Level] = []
    for tag in sorted(per_sector):
        for q in per_sector[tag]:
            q.id = len(levels)
            levels.append(q)
    return sort_levels(levels)


def table(levels: Sequence[Level], n_sites: int, Jz: float, J2: float) -> str:
    """The reference's level table (pVector::outfile, pClasses.h:102-110)."""
    lines = ["", "", "ID\tEnergies\tEnergies/site\tSz\tpx\tpy\tJz\tJ2\tEnergies-E0", ""]
    E0 = levels[0].En if levels else 0.0
    for q in levels:
        lines.append(f"{q.id}\t{q.En:.10f}\t{q.En / n_sites:.10f}\t{q.Sz:.3f}\t{q.px:.3f}\t{q.py:.3f}\t{Jz:.3f}\t"
                     f"{J2:.3f}\t{q.En - E0:.10f}")
    return "\n".join(lines) + "\n"
