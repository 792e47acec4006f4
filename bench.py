#!/usr/bin/env python
"""Benchmark of the momentum-sector H*v (the hot path of ED_Code's sHv).

Workload (default): triangular 6x6 torus, N=36, J1=1, Delta=1, Jchi=0.15,
Sz=0, k=Gamma -- 252,091,362 basis states, FP32 complex vectors (2 GB each),
synthetic seeded start vector.  One step is one full H*v.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
  python bench.py --impl reference ...   # the reference algorithm on the host cores

Timed region (device arm): K back-to-back H*v launches on the stream they are
enqueued on, bracketed by a barrier and a synchronize, timed with CUDA events;
inputs (2 GB vectors, 3.8 GB sector) are far larger than L2, so no flush is
needed.  `e2e` repeats the measurement through the C ABI's host-buffer call
(edg_hv_host): pinned host v in, host w out, transfers inside the timed
region (v by a copy, w stored into the pinned buffer by the kernel itself).
The CPU baseline runs the oracle's restatement of the reference's sHv row
formula (orbit walk + binary search, as the reference's tables cannot exist at
N=36) on a bounded sample of rows, on every host core.

Multi-GPU: sectors are independent units, so N GPUs run N replicas with no
data-path collective ("weak" scaling); value = all ranks' H*v / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "36-site H*v/s, GB/s; mixed-stream solves/s, p99 at |ΔE|≤1e-9 vs FP64 plain"
UNIT = "H*v/s"

WORKLOADS = {
    # the large single sector: 6x6 triangular, Delta=1, Jchi=0.15, Sz=0, k=Gamma
    "tri6x6_k00": dict(lattice="triangular", Lx=6, Ly=6, Jz=1.0, Ch=0.15, Sz=0, kx=0, ky=0),
    # smaller cases of the same kernel (profiling, quick checks)
    "tri8x4_k00": dict(lattice="triangular", Lx=8, Ly=4, Jz=1.0, Ch=0.15, Sz=0, kx=0, ky=0),
    "tri6x5_k23": dict(lattice="triangular", Lx=6, Ly=5, Jz=0.8, Ch=0.2, Sz=0, kx=2, ky=3),
}


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


TRAFFIC_FILE = os.path.join(ROOT, "profiles", "traffic.json")


def profile_traffic(kernel_tag: str):
    """DRAM bytes per launch of the dominant kernel, as recorded by
    `bench.py --ingest-ncu` from an ncu capture (profiles/traffic.json)."""
    try:
        with open(TRAFFIC_FILE) as f:
            rec = json.load(f).get(kernel_tag)
    except (OSError, ValueError):
        return None
    return float(rec["dram_bytes_per_launch"]) if rec else None


def roofline_record(B: float, B_base: float, ms: float, peak: float, peak_kind: str, traffic) -> dict:
    """The line's roofline object: achieved GB/s and its fraction of the peak
    by the kernel's algorithmic bytes B and by the problem's own bytes B_base,
    with the DRAM traffic per launch (None when no capture is recorded)."""
    achieved = B / (ms / 1e3) / 1e9
    base = B_base / (ms / 1e3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_kind": peak_kind, "traffic": traffic,
            "traffic_over_algorithmic": None if traffic is None else traffic / B,
            "base_bytes": B_base, "base_achieved": base, "base_frac": base / peak}


def ingest_ncu(csv_path: str, tag: str, kernel: str, scale: float, note: str) -> dict:
    """Sum dram__bytes_read.sum + dram__bytes_write.sum per launch of `kernel`
    from an ncu --csv log (--metrics or --page raw layout), average over the
    launches, multiply by `scale` (units of a full launch / units captured) and
    store it under `tag` in profiles/traffic.json."""
    import csv

    per = {}
    with open(csv_path, newline="") as f:
        rows = [r for r in csv.reader(f) if r]
    head = None
    for k, r in enumerate(rows):
        if "Kernel Name" in r and ("Metric Name" in r or any(c.startswith("dram__bytes") for c in r)):
            head = k
            break
    if head is None:
        raise SystemExit(f"{csv_path}: no ncu CSV header found")
    h = rows[head]
    kname, lid = h.index("Kernel Name"), h.index("ID")
    if "Metric Name" in h:  # --metrics layout: one row per (launch, metric)
        mname, mval, munit = h.index("Metric Name"), h.index("Metric Value"), h.index("Metric Unit")
        mult = {"byte": 1, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9, "Tbyte": 1e12}
        for r in rows[head + 1:]:
            if len(r) <= mval or kernel not in r[kname] or not r[mname].startswith("dram__bytes_"):
                continue
            per.setdefault(r[lid], 0.0)
            per[r[lid]] += float(r[mval].replace(",", "")) * mult.get(r[munit], 1)
    else:  # --page raw layout: one row per launch, a units row under the header
        cols = [h.index(c) for c in ("dram__bytes_read.sum", "dram__bytes_write.sum")]
        units = rows[head + 1]
        mult = {"byte": 1, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9, "Tbyte": 1e12}
        for r in rows[head + 2:]:
            if len(r) <= max(cols) or kernel not in r[kname]:
                continue
            per[r[lid]] = sum(float(r[c].replace(",", "")) * mult.get(units[c], 1) for c in cols)
    if not per:
        raise SystemExit(f"{csv_path}: no dram__bytes rows for kernel {kernel!r}")
    mean = sum(per.values()) / len(per)
    try:
        with open(TRAFFIC_FILE) as f:
            data = json.load(f)
    except (OSError, ValueError):
        data = {}
    data[tag] = {"dram_bytes_per_launch": mean * scale, "captured_bytes_per_launch": mean, "scale": scale,
                 "launches": len(per), "kernel": kernel, "source": os.path.basename(csv_path), "note": note}
    with open(TRAFFIC_FILE, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
        f.write("\n")
    return data[tag]


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.idx = device_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def build_model(name):
    from ed_code_gb300 import lattice as L

    w = dict(WORKLOADS[name])
    spec = L.TorusSpec(w.pop("lattice"), w.pop("Lx"), w.pop("Ly"), Jz=w.pop("Jz"), Ch=w.pop("Ch"))
    return L.make_model(spec, w["Sz"], w["kx"], w["ky"])


def cpu_sample_rate(model, reps, lid, budget_s: float, threads: int, seed: int = 4):
    """H*v per second of the oracle's row formula, from a timed sample of rows."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    n_p = len(reps)
    rng = np.random.default_rng(seed)
    v = O.splitmix_vector(n_p, seed)
    n_rows = 256
    while True:
        rows = np.sort(rng.choice(n_p, size=min(n_rows, n_p), replace=False))
        t0 = time.perf_counter()
        O.hv_rows(model, reps, lid, v, rows, threads)
        dt = time.perf_counter() - t0
        if dt >= 0.25 * budget_s or n_rows >= n_p:
            break
        n_rows = int(min(n_p, n_rows * max(2.0, 0.5 * budget_s / max(dt, 1e-3))))
    return len(rows) / dt / n_p, len(rows), dt


def cpu_sector_baselines(args, threads):
    """The reference's sHv row formula with its per-configuration tables (the
    oracle's table-mode restatement, oracle/time_reference.py shows it against
    the reference's own sHv) beside this library's H*v on the same sectors:
    config 1, a 28-site serving-size sector and one of config 2's 30-site
    sectors.  CPU on all host threads and on one; GPU in FP64 and FP32."""
    import torch

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from time_reference import SECTORS

    from ed_code_gb300 import lattice as L
    from ed_code_gb300.sector import GpuSector, fill_random

    out = []
    for name, kw, (Sz, kx, ky) in SECTORS:
        if args.cpu_sectors != "all" and name not in args.cpu_sectors.split(","):
            continue
        model = L.make_model(L.TorusSpec(**kw), Sz, kx, ky)
        sec = GpuSector(model)
        sec.build_targets()
        sec.tune(0)
        st = torch.cuda.Stream()
        gpu = {}
        for dt, tag in ((torch.complex128, "fp64"), (torch.complex64, "fp32")):
            v = torch.empty(sec.n_p, dtype=dt, device="cuda")
            w = torch.empty_like(v)
            fill_random(v, 5, st)
            reps = max(10, min(1000, int(5e7 // sec.n_p)))
            with torch.cuda.stream(st):
                for _ in range(3):
                    sec.hv(v, w, st)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(st)
                for _ in range(reps):
                    sec.hv(v, w, st)
                e1.record(st)
            torch.cuda.synchronize()
            gpu[tag] = e0.elapsed_time(e1) / reps
        n_p = sec.n_p
        sec.close()
        t0 = time.perf_counter()
        S = O.OracleSector(model)
        t_tables = time.perf_counter() - t0
        vh = O.splitmix_vector(S.n_p, 5)
        all_s = S.time_hv(vh, threads)
        one_s = S.time_hv(vh, 1, 0.1)
        del S
        out.append({"sector": name, "n_p": n_p, "cpu_ms_all_threads": round(all_s * 1e3, 4),
                    "cpu_ms_1_thread": round(one_s * 1e3, 4), "cpu_tables_seconds": round(t_tables, 2),
                    "gpu_ms_fp64": round(gpu["fp64"], 4), "gpu_ms_fp32": round(gpu["fp32"], 4),
                    "gpu_fp64_over_cpu_all_threads": round(all_s * 1e3 / gpu["fp64"], 1)})
    return out


def run_reference(args, world, rank):
    """The reference's algorithm on the host cores: the sHv row formula with
    the orbit walk of representative_p per target (the oracle's restatement;
    the reference's own per-configuration tables need ~217 GB at N=36).  The
    representative list (2 GB, ~15 min of orbit tests on the host) is not
    built: rows are sampled representatives and v is a hash of each
    representative's value.  Each target still pays the rank lookup: a binary
    search in a sorted array of the list's size and value range (its result
    unused), as the tableless restatement searches the real list."""
    if rank != 0:
        return 0
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    model = build_model(args.workload)
    threads = os.cpu_count() or 1
    n_p = O.sector_dim(model)
    t0 = time.perf_counter()
    pool, pool_lid = O.sample_reps(model, 1 << 15, seed=4)
    probe = O.sorted_probe(n_p, int(pool.min()), int(pool.max()) + 1)
    t_sample = time.perf_counter() - t0
    rng = np.random.default_rng(4)
    pick = rng.integers(0, len(pool), 1024)
    t1 = time.perf_counter()
    O.hv_rows_listless(model, pool[pick], pool_lid[pick], 4, threads, probe)
    per_row = (time.perf_counter() - t1) / len(pick)
    n_rows = int(min(n_p, max(256, args.ref_step_seconds / per_row)))
    for _ in range(args.warmup):
        r = rng.integers(0, len(pool), 256)
        O.hv_rows_listless(model, pool[r], pool_lid[r], 4, threads, probe)
    times = []
    for _ in range(args.steps):
        r = rng.integers(0, len(pool), n_rows)
        t = time.perf_counter()
        O.hv_rows_listless(model, pool[r], pool_lid[r], 4, threads, probe)
        times.append(time.perf_counter() - t)
    sec_per_hv = sum(times) / len(times) * n_p / n_rows
    value = 1.0 / sec_per_hv
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sec_per_hv * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": {"workload": args.workload, "n_p": n_p, "row_pool_seconds": round(t_sample, 2)},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{n_rows} sampled representative rows per step of the {n_p}-row sector, scaled "
                                   "to one H*v; orbit walk and a binary search of a list-sized sorted array per "
                                   "target (v hashed from the representative's value)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)
    return 0


def run_device(args, world, rank, local_rank):
    import ctypes as C

    import numpy as np
    import torch

    from ed_code_gb300 import _native as N
    from ed_code_gb300 import replicas as R
    from ed_code_gb300.sector import GpuSector, fill_random

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    model = build_model(args.workload)
    t0 = time.perf_counter()
    sec = GpuSector(model)
    torch.cuda.synchronize()
    t_basis = time.perf_counter() - t0
    nnz = sec.count_offdiag()
    fp64 = args.dtype == "c128"
    ctype = torch.complex128 if fp64 else torch.complex64
    elem = 16 if fp64 else 8
    B = sec.algorithmic_bytes(elem, nnz)
    v = torch.empty(sec.n_p, dtype=ctype, device=dev)
    w = torch.empty_like(v)
    stream = torch.cuda.Stream(device=dev)
    # page-locked host buffers of the e2e leg, allocated before anything else
    # is staged through host memory
    hv_in = hv_out = None
    if not args.no_e2e:
        hv_in = torch.empty(sec.n_p, dtype=ctype, pin_memory=True)
        hv_out = torch.empty(sec.n_p, dtype=ctype, pin_memory=True)

    def timed(steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(steps):
                sec.hv(v, w, stream)
            e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    with torch.cuda.stream(stream):
        fill_random(v, 4, stream)
    # matrix-free H*v (orbit search on the fly), timed for the record
    mf_steps = max(1, min(args.steps, 3))
    with torch.cuda.stream(stream):
        sec.hv(v, w, stream)
    mf_ms = timed(mf_steps) / mf_steps
    B_mf = sec.algorithmic_bytes(elem, nnz)
    # stored targets: the search done once, its results streamed every H*v
    mode = "matrix-free"
    t_tgt = None
    lpr, tune_ms = None, None
    if not args.matrix_free:
        t0 = time.perf_counter()
        if sec.build_targets():
            torch.cuda.synchronize()
            t_tgt = time.perf_counter() - t0
            mode = "stored-rows"
            B = sec.algorithmic_bytes(elem, nnz)
            if args.rows:
                lanes, pol, *rest = (int(x) for x in args.rows.split(","))
                sec.set_rows(lanes, pol, *rest)
                lpr = lanes
            else:
                lpr, tune_ms = sec.tune(0)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            sec.hv(v, w, stream)
    stream.synchronize()

    sampler = ClockSampler(local_rank)
    sampler.start()
    time.sleep(0.3)
    R.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        e0.record(stream)
        for _ in range(args.steps):
            sec.hv(v, w, stream)
        e1.record(stream)
    torch.cuda.synchronize()
    R.barrier()
    clocks = sampler.stop()
    ms_max = R.max_over_ranks(e0.elapsed_time(e1))
    value = R.job_rate(world, args.steps, ms_max / 1e3)
    ms_step = ms_max / args.steps

    # the block H*v: 2 and 4 vectors per pass (each row's entries read once,
    # each gathered line serving every vector), timed the same way
    block = None
    if mode == "stored-rows" and not args.no_block:
        block = {}
        for nv in (2, 4):
            V = torch.empty((sec.n_p, nv), dtype=ctype, device=dev)
            W = torch.empty_like(V)
            with torch.cuda.stream(stream):
                fill_random(V, 7, stream)
                for _ in range(args.warmup):
                    sec.hv_block(V, W, stream)
                b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                b0.record(stream)
                for _ in range(args.steps):
                    sec.hv_block(V, W, stream)
                b1.record(stream)
            torch.cuda.synchronize()
            ms_b = b0.elapsed_time(b1) / args.steps
            # algorithmic bytes of one block launch: the entry stream and row
            # offsets once, every vector's own bytes nv times
            Bb = sec.algorithmic_bytes_block(elem, nnz, nv)
            tb = profile_traffic(f"hv_block_nv{nv}_{args.workload}_{args.dtype}")
            block[f"nv{nv}"] = {"ms_per_launch": ms_b, "hv_per_s": nv * 1e3 / ms_b,
                                "algorithmic_bytes_per_launch": Bb, "GBps": Bb / (ms_b / 1e3) / 1e9,
                                "frac_of_measured_hbm": Bb / (ms_b / 1e3) / 1e9 / measured_peak_hbm()[0],
                                "traffic": tb, "traffic_over_algorithmic": None if tb is None else tb / Bb}
            del V, W
        torch.cuda.empty_cache()

    # the other vector precision on the same rows (FP64 when the line is FP32:
    # the plain form's sHv), timed the same way
    other = None
    if mode == "stored-rows" and not args.no_other_dtype:
        o_ct, o_elem = (torch.complex64, 8) if fp64 else (torch.complex128, 16)
        vo = torch.empty(sec.n_p, dtype=o_ct, device=dev)
        wo = torch.empty_like(vo)
        with torch.cuda.stream(stream):
            fill_random(vo, 4, stream)
            for _ in range(args.warmup):
                sec.hv(vo, wo, stream)
            o0, o1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            o0.record(stream)
            for _ in range(args.steps):
                sec.hv(vo, wo, stream)
            o1.record(stream)
        torch.cuda.synchronize()
        ms_o = o0.elapsed_time(o1) / args.steps
        Bo = sec.algorithmic_bytes(o_elem, nnz)
        other = {"vector": "c64" if fp64 else "c128", "ms_per_step": ms_o, "hv_per_s": 1e3 / ms_o,
                 "algorithmic_bytes": Bo, "GBps": Bo / (ms_o / 1e3) / 1e9,
                 "frac_of_measured_hbm": Bo / (ms_o / 1e3) / 1e9 / measured_peak_hbm()[0]}
        del vo, wo
        torch.cuda.empty_cache()

    # e2e through the C ABI host-buffer call: pinned v in, w out, every step
    e2e = None
    if not args.no_e2e:
        hv_in.copy_(v)
        code = N.EDG_C128 if fp64 else N.EDG_C64
        lib = N.lib()
        N.check(lib.edg_hv_host(sec._h, C.c_void_p(hv_in.data_ptr()), C.c_void_p(hv_out.data_ptr()), code))
        R.barrier()
        calls = []
        te = time.perf_counter()
        for _ in range(args.steps):
            tc = time.perf_counter()
            N.check(lib.edg_hv_host(sec._h, C.c_void_p(hv_in.data_ptr()), C.c_void_p(hv_out.data_ptr()), code))
            calls.append(time.perf_counter() - tc)
        dt = R.max_over_ranks(time.perf_counter() - te)
        e2e = {"value": R.job_rate(world, args.steps, dt), "unit": UNIT,
               "h2d_bytes_per_step": sec.n_p * elem, "d2h_bytes_per_step": sec.n_p * elem,
               "ms_per_call_min_median_max": [round(1e3 * f(calls), 2) for f in (min, np.median, max)]}
        del hv_in, hv_out

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        states, norm, _ = sec.basis()
        lid = np.rint(model.n_sites / norm.astype(np.float64) ** 2).astype(np.int32)
        threads = os.cpu_count() or 1
        rate, n_rows, dt = cpu_sample_rate(model, states, lid, args.cpu_seconds, threads)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{n_rows} random rows of the {sec.n_p}-row sector in {dt:.1f} s, scaled to one H*v "
                         "(oracle row formula in FP64: orbit walk + binary search per target; the reference's "
                         "own tables need ~217 GB at 36 sites)"}
        if args.cpu_sectors != "none":
            cpu["per_sector"] = cpu_sector_baselines(args, threads)
            cpu["per_sector_kind"] = ("port: the reference's table-mode sHv row formula (oracle), full H*v per "
                                      "call; profiles/cpu_reference_shv.md times it against the reference's own "
                                      "sHv on the same sectors")

    peak, peak_kind = measured_peak_hbm()
    traffic = profile_traffic(f"hv_{mode}_{args.workload}_{args.dtype}")
    # the problem's own bytes (per row the representative, stabiliser byte,
    # v_i and w_i; per nonzero one v_j), whatever the kernel stores
    B_base = sec.n_p * (8 + 1 + 2 * elem) + nnz * elem
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if fp64 else "f32", "data": "synthetic",
        "config": {"workload": args.workload, "n_p": sec.n_p, "nnz_off": nnz, "vector": args.dtype,
                   "hv_mode": mode, "algorithmic_bytes_per_hv": B, "basis_seconds": round(t_basis, 3),
                   "target_build_seconds": None if t_tgt is None else round(t_tgt, 3),
                   "stored_row_bytes": (sec.info.get("entry_bytes") or 6) * sec.info.get("n_targets", 0) + 16 * sec.n_p,
                   "entry_bytes": sec.info.get("entry_bytes"), "n_values": sec.info.get("n_values"),
                   "matrix_free_ms_per_step": mf_ms,
                   "lanes_per_row": lpr, "cache_policy": sec.info.get("cache_policy"),
                   "ctas_per_sm": sec.info.get("ctas_per_sm"), "pipelined": sec.info.get("pipelined"),
                   "row_kernel_ms": None if tune_ms is None else round(float(min(x for x in tune_ms if x > 0)), 3),
                   "tune_ms_lpr_8_16_32": None if tune_ms is None else [round(float(x), 3) for x in tune_ms],
                   "matrix_free_GBps": B_mf / (mf_ms / 1e3) / 1e9,
                   "l2": "inputs larger than L2 (no flush needed)", "orbit_search": "torus" if sec.info["torus"] else "walk"},
        "roofline": roofline_record(B, B_base, ms_step, peak, peak_kind, traffic),
        "block_hv": block,
        "other_precision_hv": other,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": clocks,
        # per step: the u = v/norm pass plus one row kernel; the matrix-free
        # kernel is one launch
        "gpu_launches": args.steps * (2 if mode == "stored-rows" else 1),
    }
    if rank == 0:
        print(json.dumps(out), flush=True)
    return 0


def _distinct(levels, tol=1e-9):
    out = []
    for x in sorted(levels):
        if not out or abs(x - out[-1]) > tol * abs(x):
            out.append(x)
    return out


def _rel_err(got, plain):
    """Largest |dE|/|E| of the levels in `got` against the plain FP64 levels
    (each compared with the nearest plain level the plain run reached)."""
    import numpy as np

    lev = np.array(_distinct(plain))
    errs = [abs(got[0] - lev[0]) / abs(lev[0])]
    for x in got[1:]:
        if x <= lev[-1]:
            errs.append(float(np.min(np.abs(lev - x))) / abs(x))
    return float(max(errs))


def _plain(sec, n_ev):
    """The plain FP64 form (lanczos_evecs / exact_evecs replica) on the GPU."""
    t0 = time.perf_counter()
    eigs, _, _ = sec.solve_plain(n_ev=n_ev, iterations=200, ncycles=10, tol=1e-11)
    return list(eigs), time.perf_counter() - t0


def run_serve(args):
    """Serving stream: Poisson arrivals, mixed sizes, continuous batching."""
    import numpy as np
    import torch

    from ed_code_gb300 import lattice as L
    from ed_code_gb300 import serving
    from ed_code_gb300.sector import GpuSector

    torch.cuda.init()
    warm = serving.make_stream(4, rate=1e6, seed=99, sizes=(20,))
    srv = serving.Server(max_iterations=300, res_tol=args.res_tol, tile_rows=args.serve_tile,
                         reorth=args.batch_reorth, tune=bool(args.serve_tune))
    srv.run(warm)
    stream = serving.make_stream(args.requests, rate=args.rate, seed=3)
    t0 = time.perf_counter()
    t_create0 = srv.create_seconds
    served = srv.run(stream)
    wall = time.perf_counter() - t0
    timers = srv.batch.timers()
    t_create = srv.create_seconds - t_create0
    srv.close()
    summ = serving.summarize(served)
    by = {s.rid: s for s in served}
    unconverged = [[s.rid, stream[s.rid].n_sites, stream[s.rid].n_ev, s.iterations,
                    float(max(s.residuals)) if len(s.residuals) else None]
                   for s in served if not s.converged]
    # plain FP64, one request after another, on a seeded sample (two per size)
    rng = np.random.default_rng(5)
    sample = []
    for N in (20, 24, 28, 32):
        ids = [r.rid for r in stream if r.n_sites == N]
        sample += list(rng.choice(ids, size=min(args.plain_per_size, len(ids)), replace=False)) if ids else []
    plain_t, errs = {}, []
    for rid in sample:
        req = stream[int(rid)]
        t0 = time.perf_counter()
        sec = GpuSector(L.make_model(req.spec, req.Sz, req.kx, req.ky, bowties=False))
        sec.build_targets()
        eigs, _ = _plain(sec, max(req.n_ev, 4))
        plain_t.setdefault(req.n_sites, []).append(time.perf_counter() - t0)
        errs.append(_rel_err(by[req.rid].eigs, eigs))
        sec.close()
    seq_plain = sum(float(np.mean(plain_t[r.n_sites])) for r in stream if r.n_sites in plain_t)
    out = {"metric": "mixed-stream solves/s (serving)", "mode": "serve", "value": summ["solves_per_s"],
           "unit": "solves/s", "higher_is_better": True, "n_gpus": 1, "data": "synthetic",
           "p50_s": summ["p50_s"], "p99_s": summ["p99_s"], "makespan_s": summ["makespan_s"], "wall_s": wall,
           "requests": len(served), "converged": summ["converged"],
           "unconverged_rid_sites_nev_steps_resid": unconverged,
           "max_rel_err_vs_plain_fp64": max(errs) if errs else None, "checked": len(errs),
           "plain_fp64_seconds_per_request": {str(k): float(np.mean(v)) for k, v in sorted(plain_t.items())},
           "sequential_plain_solves_per_s": len(stream) / seq_plain if seq_plain else None,
           "speedup_vs_sequential_plain": (summ["solves_per_s"] * seq_plain / len(stream)) if seq_plain else None,
           "peak_active": srv.peak_live, "create_seconds": t_create, "batch_timers": timers, "tuned": srv.tuned,
           "config": {"workload": f"poisson {args.rate}/s, {args.requests} requests, N in 20/24/28/32, seed 3",
                      "tile_rows": args.serve_tile, "reorth": "partial" if args.batch_reorth else "every step",
                      "res_tol": args.res_tol, "max_iterations": 300, "vectors": "c64 Krylov, f64 alpha/beta/RQ"}}
    print(json.dumps(out), flush=True)
    return 0


def run_batch(args):
    """64 small Hamiltonians, every momentum at Sz=0, one batch."""
    import numpy as np
    import torch

    from ed_code_gb300 import lattice as L
    from ed_code_gb300.batch import BatchSolver
    from ed_code_gb300.sector import GpuSector

    torch.cuda.init()
    rng = np.random.default_rng(2)
    specs = []
    for h in range(args.hamiltonians):
        if args.batch_shape == "tri7x4":  # 28-site sectors (1.43e6 states), the first --momenta momenta
            spec = L.TorusSpec("triangular", 7, 4, Jz=float(rng.uniform(0.5, 1.5)), Ch=float(rng.uniform(0, 0.4)))
        elif rng.random() < 0.5:
            spec = L.TorusSpec("square", 4, 4, Jz=float(rng.uniform(0.5, 1.5)), J2=float(rng.uniform(0, 0.5)),
                               Ch=float(rng.uniform(0, 0.4)))
        else:
            spec = L.TorusSpec("triangular", 5, 4, Jz=float(rng.uniform(0.5, 1.5)), J2=float(rng.uniform(0, 0.5)),
                               Ch=float(rng.uniform(0, 0.4)))
        moms = [(kx, ky) for kx in range(spec.Lx) for ky in range(spec.Ly)]
        if args.batch_shape == "tri7x4":
            moms = moms[: args.momenta]
        specs += [(spec, kx, ky) for kx, ky in moms]
    t0 = time.perf_counter()
    secs = []
    t_model = t_create = 0.0
    for spec, kx, ky in specs:
        ta = time.perf_counter()
        model = L.make_model(spec, 0, kx, ky, bowties=False)
        tb = time.perf_counter()
        sec = GpuSector(model)
        assert sec.build_targets()
        secs.append(sec)
        t_model += tb - ta
        t_create += time.perf_counter() - tb
    torch.cuda.synchronize()
    t_build = time.perf_counter() - t0
    # the library's autotuner picks the tiles on a few steps of the whole batch
    B = BatchSolver(reorth=args.batch_reorth)
    t1 = time.perf_counter()
    for k, sec in enumerate(secs):
        B.add(sec, n_ev=3, max_iterations=150, tol=0.0, seed=2, tag=k)
    choice = B.tune(steps=5)
    t_tune = time.perf_counter() - t1
    res = {r["tag"]: r for r in B.run(chunk=10)}
    t_solve = time.perf_counter() - t1
    timers = B.timers()
    # accuracy and the plain FP64 time on a seeded sample
    pick = rng.choice(len(secs), size=min(args.plain_sample, len(secs)), replace=False)
    errs, pt = [], []
    for k in pick:
        eigs, dt = _plain(secs[int(k)], 3)
        pt.append(dt)
        errs.append(_rel_err(res[int(k)]["eigs"], eigs))
    n = len(secs)
    out = {"metric": "batched small-sector solves/s", "mode": "batch", "value": n / t_solve, "unit": "solves/s",
           "higher_is_better": True, "n_gpus": 1, "data": "synthetic", "sectors": n,
           "dims": [int(min(s.n_p for s in secs)), int(max(s.n_p for s in secs))],
           "solve_seconds": t_solve, "build_seconds": t_build, "batch_timers": timers,
           "build_split": {"term_lists": t_model, "sector_and_rows": t_create}, "e2e_solves_per_s": n / (t_solve + t_build),
           "tiles": choice, "tune_seconds": t_tune,
           "max_rel_err_vs_plain_fp64": max(errs) if errs else None, "checked": len(errs),
           "plain_fp64_seconds_per_sector": float(np.mean(pt)) if pt else None,
           "speedup_vs_sequential_plain": float(np.mean(pt)) * n / t_solve if pt else None,
           "config": {"workload": (f"{args.hamiltonians} Hamiltonians (4x4 square / 5x4 triangular), all momenta, "
                                   "Sz=0, seed 2") if args.batch_shape == "small" else
                      f"{args.hamiltonians} 7x4 triangular Hamiltonians, {args.momenta} momenta each, Sz=0, seed 2",
                      "iterations": 150, "n_ev": 3,
                      "reorth": "partial" if args.batch_reorth else "every step"}}
    print(json.dumps(out), flush=True)
    return 0


def run_precision(args):
    """Config 2: the FP32-vector Lanczos against FP64 on the 6x5 triangular
    torus, all 30 momenta, 6 levels each.  Three forms per sector, on the GPU:
      * fp32: FP32 Krylov vectors and H*v, FP64 scalars (edg_solve_mixed);
      * fp64: the same algorithm with FP64 vectors, FP64 H*v and FP64
        arithmetic throughout (fp64_vectors) -- the reference point of every
        eigenvalue's error and of the speed-up, which then isolates precision;
      * plain: the reference's own algorithm (deflation, restarts; edg_solve_plain)
        in FP64, on a seeded sample of momenta, as a cross-check of the fp64
        levels and for its time."""
    import numpy as np
    import torch

    from ed_code_gb300 import lattice as L
    from ed_code_gb300.sector import GpuSector

    torch.cuda.init()
    spec = L.TorusSpec("triangular", 6, 5, Jz=0.8, Ch=0.2)
    moms = [(kx, ky) for kx in range(6) for ky in range(5)][: args.momenta]
    rows, t32, t64, t_build = [], 0.0, 0.0, 0.0
    for kx, ky in moms:
        t0 = time.perf_counter()
        sec = GpuSector(L.make_model(spec, 0, kx, ky))
        sec.build_targets()
        torch.cuda.synchronize()
        t_build += time.perf_counter() - t0
        t0 = time.perf_counter()
        r32 = sec.solve_mixed(n_ev=6, iterations=300, reorth_every=args.reorth, seed=1)
        t1 = time.perf_counter()
        r64 = sec.solve_mixed(n_ev=6, iterations=300, reorth_every=args.reorth, seed=1, fp64_vectors=True)
        t2 = time.perf_counter()
        t32 += t1 - t0
        t64 += t2 - t1
        e32, e64 = np.asarray(r32["eigs"]), np.asarray(r64["eigs"])
        k = min(len(e32), len(e64))
        rel = (np.abs(e32[:k] - e64[:k]) / np.abs(e64[:k])).tolist()
        rows.append({"k": [kx, ky], "n_p": sec.n_p, "fp64": e64.tolist(), "fp32": e32.tolist(), "rel_err": rel,
                     "fp32_residual_max": float(max(r32["residuals"])), "fp32_s": t1 - t0, "fp64_s": t2 - t1,
                     "reorth_steps_fp32_fp64": [r32["stats"]["reorth_steps"], r64["stats"]["reorth_steps"]]})
        sec.close()
    rng = np.random.default_rng(1)
    pick = [moms[int(i)] for i in rng.choice(len(moms), size=min(args.plain_sample, len(moms)), replace=False)]
    plain = []
    for kx, ky in pick:
        sec = GpuSector(L.make_model(spec, 0, kx, ky))
        sec.build_targets()
        eigs, dt = _plain(sec, 6)
        row = next(r for r in rows if r["k"] == [kx, ky])
        plain.append({"k": [kx, ky], "seconds": dt, "plain_fp64": [float(x) for x in eigs],
                      "fp64_vs_plain": _rel_err(row["fp64"], eigs), "fp32_vs_plain": _rel_err(row["fp32"], eigs)})
        sec.close()
    errs = [e for r in rows for e in r["rel_err"]]
    n = len(moms)
    out = {"metric": "precision form vs FP64 (same algorithm): solve time ratio", "mode": "precision",
           "value": t64 / t32, "unit": "x", "higher_is_better": True, "n_gpus": 1, "data": "synthetic",
           "fp32_seconds_per_sector": t32 / n, "fp64_seconds_per_sector": t64 / n,
           "sector_build_seconds_per_sector": t_build / n,
           "levels_compared": len(errs), "max_rel_err": max(errs), "levels_over_1e-9": sum(e > 1e-9 for e in errs),
           "max_fp32_residual": max(r["fp32_residual_max"] for r in rows),
           "plain_sample": plain,
           "plain_fp64_seconds_per_sector": float(np.mean([p["seconds"] for p in plain])) if plain else None,
           "speedup_vs_plain_algorithm": (float(np.mean([p["seconds"] for p in plain])) / (t32 / n)) if plain else None,
           "sectors": rows,
           "config": {"workload": "6x5 triangular, Delta=0.8, Jchi=0.2, Sz=0, all momenta", "iterations": 300,
                      "n_ev": 6, "reorth_every": args.reorth, "seed": 1}}
    print(json.dumps(out), flush=True)
    return 0


def run_solve36(args):
    """The large single sector: 300 FP32 Lanczos steps, 6 levels, FP64 residuals."""
    import torch

    from ed_code_gb300.sector import GpuSector

    torch.cuda.init()
    model = build_model("tri6x6_k00")
    t0 = time.perf_counter()
    sec = GpuSector(model)
    assert sec.build_targets()
    sec.tune(0)
    t_build = time.perf_counter() - t0
    t1 = time.perf_counter()
    r = sec.solve_mixed(n_ev=6, iterations=300, reorth_every=0, seed=4)  # 2 GB vectors: local form
    t_solve = time.perf_counter() - t1
    out = {"metric": "36-site sector solve", "mode": "solve36", "value": t_solve, "unit": "s",
           "higher_is_better": False, "n_gpus": 1, "data": "synthetic", "build_seconds": t_build,
           "eigs": [float(x) for x in r["eigs"]], "ritz": [float(x) for x in r["ritz"]],
           "residuals": [float(x) for x in r["residuals"]], "stats": r["stats"],
           "config": {"workload": "tri6x6_k00", "iterations": 300, "n_ev": 6,
                      "vectors": f"c64: {r['stats']['stored_vectors']} stored, the rest in a ring of resident vectors",
                      "seed": 4}}
    print(json.dumps(out), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="tri6x6_k00")
    ap.add_argument("--dtype", choices=["c64", "c128"], default="c64")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--matrix-free", action="store_true", help="do not store the searched targets")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-block", action="store_true", help="skip the 2- and 4-vector block H*v timing")
    ap.add_argument("--no-other-dtype", action="store_true",
                    help="skip timing the H*v in the other vector precision (FP64 for a c64 line)")
    ap.add_argument("--rows", default=None,
                    help="LANES,POLICY[,CTAS_PER_SM[,PIPELINED]]: fix the stored-row kernel instead of timing it")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--cpu-sectors", default="all",
                    help="CPU-baseline sectors timed beside the GPU: all, none, or names from oracle/time_reference.py")
    ap.add_argument("--ref-step-seconds", type=float, default=4.0)
    ap.add_argument("--mode", choices=["hv", "serve", "batch", "precision", "solve36"], default="hv",
                    help="hv: the headline H*v line; the others time the solver configurations")
    ap.add_argument("--requests", type=int, default=64)
    ap.add_argument("--rate", type=float, default=200.0)
    ap.add_argument("--res-tol", type=float, default=1e-6)
    ap.add_argument("--plain-per-size", type=int, default=2)
    ap.add_argument("--hamiltonians", type=int, default=64)
    ap.add_argument("--plain-sample", type=int, default=3)
    ap.add_argument("--momenta", type=int, default=30)
    ap.add_argument("--batch-shape", choices=["small", "tri7x4"], default="small",
                    help="batch: 4x4/5x4 Hamiltonians with all momenta, or 7x4 ones with --momenta momenta")
    ap.add_argument("--reorth", type=int, default=-1,
                    help="precision: -1 reorthogonalise partially (Simon's estimates; the default), k > 0 every k "
                         "steps, 0 locally against the last two vectors")
    ap.add_argument("--serve-tile", type=int, default=4096, help="serve: rows per tile of the batch kernels")
    ap.add_argument("--serve-tune", type=int, default=1, choices=[0, 1],
                    help="serve: time the batch tiles on the first requests (1) or keep --serve-tile (0)")
    ap.add_argument("--batch-reorth", type=int, default=1, choices=[0, 1],
                    help="serve/batch: reorthogonalise partially (1, the serving loop's default) or every step (0)")
    ap.add_argument("--ingest-ncu", metavar="CSV", default=None,
                    help="record the DRAM bytes per launch of --kernel from this ncu CSV in profiles/traffic.json "
                         "under --tag, and exit")
    ap.add_argument("--tag", default=None, help="--ingest-ncu: the record's key (hv_<mode>_<workload>_<dtype>)")
    ap.add_argument("--kernel", default="k_hv_csr", help="--ingest-ncu: kernel name substring")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="--ingest-ncu: units of a full launch / units of the captured launch")
    ap.add_argument("--note", default="", help="--ingest-ncu: how the capture was made")
    args = ap.parse_args()
    if args.ingest_ncu:
        if not args.tag:
            ap.error("--ingest-ncu needs --tag")
        print(json.dumps(ingest_ncu(args.ingest_ncu, args.tag, args.kernel, args.scale, args.note)))
        return 0
    if args.mode != "hv" and args.impl == "gb300":
        return {"serve": run_serve, "batch": run_batch, "precision": run_precision,
                "solve36": run_solve36}[args.mode](args)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, world, rank)
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    try:
        return run_device(args, world, rank, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
