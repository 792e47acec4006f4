"""Generate the tridiagonal-eigensolve fixtures from the reference.

For a few sectors, the reference's own first Lanczos cycle (reference sHv and
BLAS-1 helpers, driven by oracle/ref_harness's T mode) runs m steps from a
seeded start vector and its T matrix is recorded.  For prefixes T_k of it the
fixture stores what the reference's tridiagonal step computes: zheev('V','U')
of the complex matrix it assembles (lanczos.cpp:271-286: complex alpha on the
diagonal, beta off it; Matrix_Functions.cpp:28-48), called through scipy's
bundled OpenBLAS -- the library the reference is linked against here.

Output: tests/golden/tridiag.npz.
usage: python tests/golden/make_tridiag.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np
import scipy.linalg as sl

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from ed_code_gb300 import lattice as L  # noqa: E402
import oracle as O  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
N_VECS = 8  # lowest eigenvectors stored per prefix

# name -> (spec kwargs, (Sz, kx, ky), Lanczos steps, start-vector seed, prefixes)
CASES = {
    "sq4x4": (dict(lattice="square", Lx=4, Ly=4), (0, 0, 0), 150, 21, (12, 60, 150)),
    "tri4x3_k11": (dict(lattice="triangular", Lx=4, Ly=3, Jz=0.8, Ch=0.2), (0, 1, 1), 60, 22, (8, 30, 60)),
    "sq6x4_k00": (dict(lattice="square", Lx=6, Ly=4), (0, 0, 0), 200, 23, (40, 120, 200)),
    "tri6x4_k10": (dict(lattice="triangular", Lx=6, Ly=4, Jz=0.8, Ch=0.2), (0, 1, 0), 300, 24, (100, 300)),
}


def zheev_lowest(alpha: np.ndarray, beta: np.ndarray, k: int):
    """The reference's T_k and zheev('V','U') on it (lower=False: UPLO 'U')."""
    T = np.zeros((k, k), np.complex128)
    T[np.arange(k), np.arange(k)] = alpha[:k]
    for j in range(k - 1):
        T[j, j + 1] = beta[j + 1]
        T[j + 1, j] = beta[j + 1]
    w, V = sl.eigh(T, lower=False, driver="ev")
    return w, V[:, : min(N_VECS, k)]


def main():
    if not os.path.exists(HARNESS):
        raise SystemExit("build the reference first: make -C oracle ref REF_SRC=<reference src/>")
    store = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, (spec_kw, (Sz, kx, ky), m, seed, prefixes) in CASES.items():
            spec = L.TorusSpec(**spec_kw)
            d = os.path.join(tmp, name)
            os.makedirs(d)
            inp = os.path.join(d, "in.txt")
            with open(inp, "w") as f:
                f.write(L.input_file_text(spec, Sz, kx, ky))
            n_p = O.sector_dim(L.make_model(spec, Sz, kx, ky))
            O.splitmix_vector(n_p, seed).tofile(os.path.join(d, "vT.c128"))
            subprocess.run([HARNESS, inp, d, "tables", "0", "1", str(m)], check=True, stdout=subprocess.DEVNULL)
            raw = np.fromfile(os.path.join(d, "T.f64"), np.float64)
            alpha = raw[: 2 * m].view(np.complex128)
            beta = raw[2 * m:]
            assert len(alpha) == m and len(beta) == m + 1, (name, raw.shape)
            store[f"{name}_alpha"] = alpha
            store[f"{name}_beta"] = beta
            store[f"{name}_prefixes"] = np.array(prefixes)
            for k in prefixes:
                w, V = zheev_lowest(alpha, beta, k)
                store[f"{name}_k{k}_eigs"] = w
                store[f"{name}_k{k}_vecs"] = V
            print(f"{name}: n_p={n_p} m={m} lowest={store[f'{name}_k{prefixes[-1]}_eigs'][:3]}", flush=True)
    np.savez_compressed(os.path.join(HERE, "tridiag.npz"), **store)


if __name__ == "__main__":
    main()
