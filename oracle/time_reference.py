"""Time the reference's own sHv against the oracle's table-mode restatement.

Test infrastructure: runs only where the reference was compiled from its
sources (make -C oracle ref REF_SRC=...).  For each sector the reference
harness (oracle/_ref/ref_harness, reference pConstruct_States + sHv, OpenMP)
applies sHv to a seeded vector `reps` times on all host threads and on one
thread (the reference's own wall_clock around each call), and the oracle's
table-mode port (oracle.OracleSector.time_hv) is timed on the same host.  The
ratio reference / port shows how well the port, which is what the GPU machine can
run, stands in for the reference's CPU path.  Prints a markdown table.

With --solves it times the reference's whole sector solve instead: ED2 (the
reference's driver, sector_lanczos) on config 1's 4x4 sector and on one
5x4 triangular sector of config 3's kind, both through the reference's dense
path (n_p <= 10000), on all host threads and on one.

usage: python oracle/time_reference.py [--solves]
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from ed_code_gb300 import lattice as L  # noqa: E402
import oracle as O  # noqa: E402

HARNESS = os.path.join(HERE, "_ref", "ref_harness")

# the CPU-baseline sectors of bench.py: config 1, a serving-size 28-site
# sector, and one of config 2's 30-site sectors
SECTORS = [
    ("sq4x4_k00", dict(lattice="square", Lx=4, Ly=4), (0, 0, 0)),
    ("tri7x4_k00", dict(lattice="triangular", Lx=7, Ly=4, Jz=1.0, Ch=0.15), (0, 0, 0)),
    ("tri6x5_k23", dict(lattice="triangular", Lx=6, Ly=5, Jz=0.8, Ch=0.2), (0, 2, 3)),
]


def run_ref(inp: str, d: str, threads: int, reps: int) -> float:
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    subprocess.run([HARNESS, inp, d, "tables", "1", str(reps)], check=True, stdout=subprocess.DEVNULL, env=env)
    return float(open(os.path.join(d, "hv_time.txt")).read().split()[0])


ED2 = os.path.join(HERE, "_ref", "ED2")
SOLVES = [
    ("cfg1_sq4x4_k00", dict(lattice="square", Lx=4, Ly=4), (0, 0, 0), 4),
    ("cfg3_tri5x4_k00", dict(lattice="triangular", Lx=5, Ly=4, Jz=0.9, J2=0.3, Ch=0.25), (0, 0, 0), 3),
]


def solves(threads_list):
    """Wall time of ED2 on each SOLVES sector (input file from lattice.py)."""
    import time

    if not os.path.exists(ED2):
        raise SystemExit("build the reference first: make -C oracle ref REF_SRC=<reference src/>")
    print("| sector | n_p | threads | ED2 wall time (s) | lowest level |")
    print("|---|---|---|---|---|")
    for name, kw, (Sz, kx, ky), nev in SOLVES:
        spec = L.TorusSpec(**kw)
        n_p = O.sector_dim(L.make_model(spec, Sz, kx, ky))
        for thr in threads_list:
            with tempfile.TemporaryDirectory() as d:
                inp = os.path.join(d, "in.txt")
                with open(inp, "w") as f:
                    f.write(L.input_file_text(spec, Sz, kx, ky, num_eigenvalues=nev))
                env = dict(os.environ, OMP_NUM_THREADS=str(thr), OPENBLAS_NUM_THREADS=str(thr))
                t = time.perf_counter()
                subprocess.run([ED2, inp, os.path.join(d, "out.txt")], check=True, stdout=subprocess.DEVNULL, env=env)
                dt = time.perf_counter() - t
                first, seen = None, False
                for line in open(os.path.join(d, "out.txt")):
                    if line.startswith("Energies"):
                        seen = True
                    elif seen and first is None and line.split():
                        first = float(line.split()[0])
            print(f"| {name} | {n_p} | {thr} | {dt:.2f} | {first} |", flush=True)


def main():
    if "--solves" in sys.argv:
        threads = [int(x) for x in os.environ.get("EDG_SOLVE_THREADS", f"{os.cpu_count() or 1},1").split(",")]
        solves(threads)
        return
    if not os.path.exists(HARNESS):
        raise SystemExit("build the reference first: make -C oracle ref REF_SRC=<reference src/>")
    cores = os.cpu_count() or 1
    rows = []
    with tempfile.TemporaryDirectory() as tmp:
        for name, kw, (Sz, kx, ky) in SECTORS:
            spec = L.TorusSpec(**kw)
            model = L.make_model(spec, Sz, kx, ky)
            d = os.path.join(tmp, name)
            os.makedirs(d)
            inp = os.path.join(d, "in.txt")
            with open(inp, "w") as f:
                f.write(L.input_file_text(spec, Sz, kx, ky))
            S = O.OracleSector(model)
            v = O.splitmix_vector(S.n_p, 5)
            v.tofile(os.path.join(d, "v0.c128"))
            reps = max(1, int(2e6 // S.n_p))
            ref_all = run_ref(inp, d, cores, reps)
            ref_one = run_ref(inp, d, 1, max(1, reps // 4))
            w_ref = np.fromfile(os.path.join(d, "w0.c128"), np.complex128)
            err = float(np.abs(S.hv(v) - w_ref).max() / max(1.0, np.abs(w_ref).max()))
            port_all = S.time_hv(v, cores)
            port_one = S.time_hv(v, 1, 0.1)
            rows.append((name, S.n_p, ref_all, ref_one, port_all, port_one, err))
            print(f"{name}: n_p={S.n_p} ref {ref_all * 1e3:.2f}/{ref_one * 1e3:.2f} ms, "
                  f"port {port_all * 1e3:.2f}/{port_one * 1e3:.2f} ms, |w-w_ref| {err:.1e}", file=sys.stderr)
    print(f"| sector | n_p | reference sHv, {cores} threads (ms) | reference, 1 thread (ms) | "
          f"port, {cores} threads (ms) | port, 1 thread (ms) | reference / port ({cores} thr, 1 thr) | "
          "max |w_port - w_ref| / max |w_ref| |")
    print("|---|---|---|---|---|---|---|---|")
    for name, n, ra, r1, pa, p1, err in rows:
        print(f"| {name} | {n} | {ra * 1e3:.3f} | {r1 * 1e3:.3f} | {pa * 1e3:.3f} | {p1 * 1e3:.3f} | "
              f"{ra / pa:.2f}, {r1 / p1:.2f} | {err:.1e} |")


if __name__ == "__main__":
    main()
