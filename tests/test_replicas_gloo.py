"""The N > 1 path on CPU: two gloo ranks exercise the replica bookkeeping that
bench.py and the sharded sweep use (max over ranks, whole-job rate, disjoint
sector shares, merge of per-sector levels), and the reference arm's other
ranks exit without work."""
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from ed_code_gb300 import lattice as L  # noqa: E402
from ed_code_gb300 import replicas as R  # noqa: E402
from ed_code_gb300 import sweep as S  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _levels_for(tag, n_ones, kx, ky, spec):
    """Deterministic stand-in levels for one sector (no GPU)."""
    sz = 0.5 * n_ones - 0.5 * (spec.n_sites - n_ones)
    meta = (0.0, 0.0, sz, kx, ky)
    return [S.Level(0, -1.0 + 0.01 * ((7 * tag + j) % 13) + 0.001 * j, *meta) for j in range(2)]


def _worker(rank, world, port, out_q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        R.barrier()
        ms_max = R.max_over_ranks(10.0 + 5.0 * rank)
        rate = R.job_rate(world, 20, ms_max / 1e3)
        spec = L.TorusSpec("triangular", 3, 2)
        units = list(enumerate(S.sector_list(spec)))
        mine = R.share(units, rank, world)
        per_sector = {tag: _levels_for(tag, *sec, spec) for tag, sec in mine}
        merged = R.merge(per_sector)
        levels = S.assemble(merged)
        out_q.put((rank, ms_max, rate, [t for t, _ in mine],
                   [(q.id, q.En, q.Sz, q.kx, q.ky) for q in levels]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = {}
    for _ in procs:
        r = q.get(timeout=120)
        res[r[0]] = r
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # max over ranks and the whole-job rate (units of both ranks over the slowest time)
    assert res[0][1] == res[1][1] == 15.0
    assert res[0][2] == pytest.approx(2 * 20 / 0.015)
    # shares are disjoint and cover every sector
    spec = L.TorusSpec("triangular", 3, 2)
    n_units = len(S.sector_list(spec))
    assert sorted(res[0][3] + res[1][3]) == list(range(n_units))
    assert not set(res[0][3]) & set(res[1][3])
    # every rank ends with the levels one process would have produced
    alone = {tag: _levels_for(tag, *sec, spec) for tag, sec in enumerate(S.sector_list(spec))}
    want = [(q.id, q.En, q.Sz, q.kx, q.ky) for q in S.assemble(alone)]
    assert res[0][4] == want and res[1][4] == want


def test_single_process_helpers():
    assert R.max_over_ranks(3.5) == 3.5
    assert R.merge({1: "a"}) == {1: "a"}
    assert R.share(list(range(7)), 1, 3) == [1, 4]
    with pytest.raises(ValueError):
        R.share([1, 2], 2, 2)
    with pytest.raises(ValueError):
        R.job_rate(1, 1, 0.0)


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert p.returncode == 0
    assert p.stdout.strip() == ""
