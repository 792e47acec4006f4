"""Runs with one process per GPU.

Sectors, momenta and requests are independent, so a multi-GPU run is a set of
replicas: each rank takes its own share of the units and no vector crosses a
rank.  The only exchanges are on the host side of the data path: the
max-over-ranks time of a timed region, and the collection of per-sector
levels after a sweep.  Both work on any torch.distributed backend (NCCL on
GPUs, gloo on CPU).
"""
from __future__ import annotations

import os
from typing import Dict, List, Sequence, Tuple, TypeVar

T = TypeVar("T")


def rank_world() -> Tuple[int, int]:
    """(rank, world size) from the launcher's environment; (0, 1) alone."""
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


def share(items: Sequence[T], rank: int, world: int) -> List[T]:
    """This rank's units: every world-th item starting at rank, so that ranks
    with neighbouring sectors (similar sizes) get similar amounts of work."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    return list(items[rank::world])


def _active():
    import torch.distributed as dist

    return dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1


def _device():
    import torch
    import torch.distributed as dist

    if dist.get_backend() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def barrier() -> None:
    if _active():
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float) -> float:
    """The largest x over all ranks (x itself without a process group)."""
    if not _active():
        return float(x)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(world: int, units_per_rank: int, seconds_max: float) -> float:
    """Whole-job throughput: the units all ranks processed over the slowest
    rank's time."""
    if seconds_max <= 0:
        raise ValueError("timed region must be positive")
    return world * units_per_rank / seconds_max


def merge(per_rank: Dict[int, T]) -> Dict[int, T]:
    """Union of the {unit index: result} maps of all ranks (the map itself
    without a process group).  Unit indices must not repeat across ranks."""
    if not _active():
        return dict(per_rank)
    import torch.distributed as dist

    parts: List[Dict[int, T]] = [None] * dist.get_world_size()  # type: ignore[list-item]
    dist.all_gather_object(parts, dict(per_rank))
    out: Dict[int, T] = {}
    for p in parts:
        for k, v in p.items():
            if k in out:
                raise ValueError(f"unit {k} reported by two ranks")
            out[k] = v
    return out
