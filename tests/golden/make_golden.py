"""Generate the golden fixtures from the reference itself.

Runs in a container where the reference sources are present: builds the
reference (``make -C oracle ref REF_SRC=...``: ED2 plus the table/sHv dump harness,
compiled from the read-only sources), writes one reference input file per
case with ``ed_code_gb300.lattice``, and records what the reference prints or
dumps:

* small sectors: every table (pblock_states, norm, rep_loc, state_ph, Ia, Ib)
  and sHv applied to seeded vectors;
* larger sectors: SHA-256 digests of the integer/exact tables, sampled table
  entries, and sHv checksums (sum, norm, projection on a second vector) plus
  sampled entries;
* eigenvalues printed by the reference driver ED2 (dense ``zheev`` path for
  n_p <= 10000, Lanczos above).

Output: tests/golden/<case>.npz and tests/golden/cases.json.
usage: python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from ed_code_gb300 import lattice as L  # noqa: E402
import oracle as O  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
ED2 = os.path.join(ROOT, "oracle", "_ref", "ED2")
FULL_TABLE_LIMIT = 20000      # store full tables up to this many configurations
N_SAMPLE = 4096               # sampled entries for larger sectors
VEC_SEEDS = (11, 12)


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def rng_relabel(n, seed):
    r = np.random.default_rng(seed)
    return [int(x) for x in r.permutation(n)]



# name -> (spec kwargs, [(Sz, kx, ky) or (Sz, kx, ky, kz)], run ED2?, ED2 kwargs)
CASES = {
    "sq4x4": (dict(lattice="square", Lx=4, Ly=4), [(0, 0, 0)], True, dict(num_eigenvalues=4)),
    "sq4x4_j2": (dict(lattice="square", Lx=4, Ly=4, Jz=0.7, J2=0.4), [(0, 2, 2), (0, 1, 0)], True,
                 dict(num_eigenvalues=3)),
    # Phases per bond direction (x: 0.7, y: -1.3), so H stays translation
    # invariant and Hermitian in the momentum basis.
    "sq4x4_phase_sz1": (dict(lattice="square", Lx=4, Ly=4, bond_phases=[0.7, -1.3] * 16), [(1, 1, 3)], True,
                        dict(num_eigenvalues=3)),
    "tri4x3": (dict(lattice="triangular", Lx=4, Ly=3, Jz=0.8, Ch=0.2),
               [(0, kx, ky) for kx in range(4) for ky in range(3)], True, dict(num_eigenvalues=4)),
    "tri4x3_chch": (dict(lattice="triangular", Lx=4, Ly=3, Jz=0.8, Ch=0.2, ChCh=0.3), [(0, 2, 1), (0, 0, 0)], True,
                    dict(num_eigenvalues=3)),
    "tri4x3_relabel": (dict(lattice="triangular", Lx=4, Ly=3, Jz=0.9, Ch=0.25, relabel=rng_relabel(12, 3)),
                       [(0, 1, 1), (1, 0, 2)], True, dict(num_eigenvalues=3)),
    # n_p ~ 9.2e3 takes the reference's dense zheev path, which needs about an hour
    # here, so this case records tables and sHv only.
    "tri5x4_j2": (dict(lattice="triangular", Lx=5, Ly=4, Jz=1.2, J2=0.3, Ch=0.25), [(0, 0, 0), (0, 2, 1)], False,
                  dict(num_eigenvalues=3)),
    "tri6x4_k10": (dict(lattice="triangular", Lx=6, Ly=4, Jz=0.8, Ch=0.2), [(0, 1, 0)], True,
                   dict(num_eigenvalues=2, iterations=120, ncycles=3, tol=1e-12)),
    "sq6x4_k00": (dict(lattice="square", Lx=6, Ly=4), [(0, 0, 0)], True,
                  dict(num_eigenvalues=4, iterations=200, ncycles=2, tol=1e-12)),
    # 3-D tori go through the reference's 3-D pConstruct_States and sHv.  Its
    # driver fixes dim = 2 (ED.cpp:69), so there is no ED2 run for them.
    "cub3x2x2": (dict(lattice="cubic", Lx=3, Ly=2, Lz=2, Jz=0.9, Ch=0.2), [(0, 0, 0, 0), (0, 1, 1, 1), (1, 2, 0, 1)],
                 False, dict(num_eigenvalues=3)),
    "cub4x2x2": (dict(lattice="cubic", Lx=4, Ly=2, Lz=2, Jz=1.1), [(0, 2, 1, 0), (0, 1, 0, 1)], False,
                 dict(num_eigenvalues=3)),
}


def parse_ed2(text: str):
    """Eigenvalues from the reference's 'Energies' table (Lanczos_sector.cpp:128-132)."""
    out = []
    lines = text.splitlines()
    try:
        start = next(i for i, l in enumerate(lines) if l.startswith("Energies"))
    except StopIteration:
        return out
    for l in lines[start + 1:]:
        parts = l.split()
        if len(parts) >= 7:
            try:
                out.append(float(parts[0]))
            except ValueError:
                break
    return out


def run_case(name: str, workdir: str) -> dict:
    spec_kw, sectors, want_ed2, ed2_kw = CASES[name]
    spec = L.TorusSpec(**spec_kw)
    store = {}
    meta = {"spec": {k: v for k, v in spec_kw.items()}, "sectors": []}
    for si, sec in enumerate(sectors):
        Sz, kx, ky = sec[:3]
        kz = sec[3] if len(sec) > 3 else 0
        extra = dict(kz=kz) if spec.lattice == "cubic" else {}
        tag = f"s{si}"
        d = os.path.join(workdir, f"{name}_{tag}")
        os.makedirs(d, exist_ok=True)
        text = L.input_file_text(spec, Sz, kx, ky, **extra, **ed2_kw)
        inp = os.path.join(d, "in.txt")
        with open(inp, "w") as f:
            f.write(text)
        model = L.make_model(spec, Sz, kx, ky, **extra)
        n_p_guess = O.OracleSector(model).n_p if model.T3 else O.sector_dim(model)
        vecs = [O.splitmix_vector(n_p_guess, s) for s in VEC_SEEDS]
        for k, v in enumerate(vecs):
            v.tofile(os.path.join(d, f"v{k}.c128"))
        subprocess.run([HARNESS, inp, d, "tables", str(len(vecs))], check=True, stdout=subprocess.DEVNULL)
        meta_line = open(os.path.join(d, "meta.txt")).read().split()
        n_sites, n_ones, L1, L2, _, _, n_p, n_cfg, bits_right = (int(x) for x in meta_line[:9])
        assert n_p == n_p_guess, (name, n_p, n_p_guess)
        states = np.fromfile(os.path.join(d, "states.i64"), np.int64)
        norm = np.fromfile(os.path.join(d, "norm.f64"), np.float64)
        rep_loc = np.fromfile(os.path.join(d, "rep_loc.i64"), np.int64)
        state_ph = np.fromfile(os.path.join(d, "state_ph.c128"), np.complex128)
        Ia = np.fromfile(os.path.join(d, "Ia.i64"), np.int64)
        Ib = np.fromfile(os.path.join(d, "Ib.i64"), np.int64)
        ws = [np.fromfile(os.path.join(d, f"w{k}.c128"), np.complex128) for k in range(len(vecs))]
        sm = {"Sz": Sz, "kx": kx, "ky": ky, "kz": kz, "L3": int(meta_line[10]), "n_sites": n_sites, "n_ones": n_ones, "L1": L1, "L2": L2, "n_p": n_p,
              "n_configs": n_cfg, "bits_right": bits_right, "vec_seeds": list(VEC_SEEDS),
              "sha_states": sha(states), "sha_norm": sha(norm), "sha_rep_loc": sha(rep_loc), "sha_Ia": sha(Ia),
              "sha_Ib": sha(Ib), "full": n_cfg <= FULL_TABLE_LIMIT}
        if n_cfg <= FULL_TABLE_LIMIT:
            store[f"{tag}_states"] = states
            store[f"{tag}_norm"] = norm
            store[f"{tag}_rep_loc"] = rep_loc
            store[f"{tag}_state_ph"] = state_ph
            store[f"{tag}_Ia"] = Ia
            store[f"{tag}_Ib"] = Ib
            for k, w in enumerate(ws):
                store[f"{tag}_w{k}"] = w
        else:
            r = np.random.default_rng(1000 + si)
            rows = np.sort(r.choice(n_p, size=min(N_SAMPLE, n_p), replace=False))
            cfg = np.sort(r.choice(n_cfg, size=min(N_SAMPLE, n_cfg), replace=False))
            store[f"{tag}_rows"] = rows
            store[f"{tag}_states_at_rows"] = states[rows]
            store[f"{tag}_norm_at_rows"] = norm[rows]
            store[f"{tag}_cfg"] = cfg
            store[f"{tag}_rep_loc_at_cfg"] = rep_loc[cfg]
            store[f"{tag}_state_ph_at_cfg"] = state_ph[cfg]
            for k, w in enumerate(ws):
                store[f"{tag}_w{k}_at_rows"] = w[rows]
                # checksums: sum, 2-norm^2, projection onto the other seeded vector
                other = vecs[(k + 1) % len(vecs)]
                store[f"{tag}_w{k}_sum"] = np.array([w.sum()])
                store[f"{tag}_w{k}_norm2"] = np.array([np.vdot(w, w).real])
                store[f"{tag}_w{k}_proj"] = np.array([np.vdot(other, w)])
        if want_ed2:
            out = os.path.join(d, "ed2_out.txt")
            subprocess.run([ED2, inp, out], check=True, env=dict(os.environ, OMP_NUM_THREADS=str(os.cpu_count())))
            eig = parse_ed2(open(out).read())
            sm["ed2_path"] = "dense" if n_p <= 10000 else "lanczos"
            sm["ed2_eigs"] = eig[:16]
            sm["ed2_kw"] = ed2_kw
        meta["sectors"].append(sm)
        print(f"{name} {tag}: n_p={n_p} n_cfg={n_cfg} eigs={sm.get('ed2_eigs', [])[:4]}", flush=True)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **store)
    return meta


def main(argv):
    names = argv or list(CASES)
    sys.path.insert(0, ROOT)
    import __graft_entry__ as G

    ref = G.reference_src()
    if not ref:
        raise SystemExit("the reference sources are not mounted (set EDG_REFERENCE_SRC to its src/ directory)")
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF_SRC={ref}"], check=True,
                   stdout=subprocess.DEVNULL)
    cases_path = os.path.join(HERE, "cases.json")
    allmeta = json.load(open(cases_path)) if os.path.exists(cases_path) else {}
    with tempfile.TemporaryDirectory() as tmp:
        for n in names:
            allmeta[n] = run_case(n, tmp)
    with open(cases_path, "w") as f:
        json.dump(allmeta, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main(sys.argv[1:])
