"""Generate the observables fixture from the reference's analysis programs.

Runs where the reference sources are present (make -C oracle ref analysis
REF_SRC=...).  The reference driver ED2 diagonalises one sector with
Find_Vectors=1 and writes its two lowest momentum eigenvectors (_pEV files,
Lanczos_sector.cpp:140-197); the reference's analysis programs pspincorr and
pchirality (analysis/src) read them, unwrap them (Unwrap_pState) and print
<bra|Sz_i Sz_j|ket>, <bra|SxSx+SySy|ket> on the pairs of each triangle and the
chirality of the triangle list.  The fixture keeps the eigenvectors, the
triangles and the printed values.

Two details of the reference bound the comparison: the _pEV files carry px,
py with six significant digits (the stream's default precision), so the
files are rewritten here with them in full before the analysis reads them;
and the analysis prints its results with six significant digits, the
precision the fixture is compared at.  The sector is 4x3 triangular at
k = (1, 1): no state there has a stabiliser, so the reference's unwrap (which
sums each orbit over all translations) is normalised like the momentum basis.

Output: tests/golden/observables.npz.
usage: python tests/golden/make_observables.py
"""
from __future__ import annotations

import math
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from ed_code_gb300 import lattice as L  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")
SPEC = dict(lattice="triangular", Lx=4, Ly=3, Jz=0.8, Ch=0.2)
SECTOR = (0, 1, 1)
TRIANGLES = 3  # the first triangles of the lattice's list


def parse_pev(path):
    lines = open(path).read().splitlines()
    k = next(i for i, l in enumerate(lines) if l.startswith("pblock_states"))
    st, nrm, c = [], [], []
    for l in lines[k + 1:]:
        p = l.split()
        if len(p) < 3:
            continue
        m = re.match(r"\(([-0-9.eE+]+),([-0-9.eE+]+)\)", p[2])
        st.append(int(p[0]))
        nrm.append(float(p[1]))
        c.append(complex(float(m.group(1)), float(m.group(2))))
    return np.array(st, np.int64), np.array(nrm), np.array(c), lines[:k + 2]


def exact_norm(norm, n_trans):
    """The norms sqrt(L1 L2 / lid) in full (the reference prints the first
    row's with six digits): each value snapped to the nearest such root."""
    cand = np.array([math.sqrt(n_trans / d) for d in range(1, n_trans + 1) if n_trans % d == 0])
    return cand[np.argmin(np.abs(cand[None, :] - np.asarray(norm)[:, None]), axis=1)]


def write_pev(path, head, states, norm, coeff, n_p, px, py):
    """The file as the reference writes it, with px, py and the norms in full."""
    with open(path, "w") as f:
        i = head.index(next(l for l in head if l.startswith("np")))
        f.write("\n".join(head[:i + 1]) + "\n")
        f.write(f"{n_p}\t\t{px!r}\t\t{py!r}\n\n\npblock_states \t\t Norm \t\t\t v_coeff\n\n")
        for s, nr, c in zip(states, norm, coeff):
            f.write(f"{s}\t\t\t{float(nr)!r}\t\t\t({c.real:.15f},{c.imag:.15f})\n")


def cplx(s):
    m = re.search(r"\(([-0-9.eE+]+),([-0-9.eE+]+)\)", s)
    return complex(float(m.group(1)), float(m.group(2)))


def main():
    for exe in ("ED2", "pspincorr", "pchirality"):
        if not os.path.exists(os.path.join(REF, exe)):
            raise SystemExit("build the reference first: make -C oracle ref analysis REF_SRC=<reference src/>")
    spec = L.TorusSpec(**SPEC)
    Sz, kx, ky = SECTOR
    model = L.make_model(spec, Sz, kx, ky)
    tris = [tuple(t) for t in spec.triangles()[:TRIANGLES]]
    store = {}
    with tempfile.TemporaryDirectory() as tmp:
        inp = os.path.join(tmp, "in.txt")
        vec = os.path.join(tmp, "vec")
        text = L.input_file_text(spec, Sz, kx, ky, num_eigenvalues=2, find_vectors=True)
        with open(inp, "w") as f:
            f.write(text + "Unwrap_pVector=0\n" + f"Vector_File_Path={vec}\n")
        subprocess.run([os.path.join(REF, "ED2"), inp, os.path.join(tmp, "ed2.txt")], check=True,
                       stdout=subprocess.DEVNULL)
        L1, L2 = spec.Lx, spec.Ly
        px, py = 2 * kx * math.pi / L1, 2 * ky * math.pi / L2
        vecs = []
        for q in range(2):
            st, nrm, c, head = parse_pev(f"{vec}_pEV{q}.txt")
            nrm = exact_norm(nrm, L1 * L2)
            write_pev(os.path.join(tmp, f"full_pEV{q}.txt"), head, st, nrm, c, len(st), px, py)
            vecs.append(c)
            store["states"] = st
        store["vec0"], store["vec1"] = vecs
        store["triangles"] = np.array(tris, np.int64)
        T1, T2 = L.translations(spec.Lx, spec.Ly)
        tri_txt = "Triangles=[" + ",".join(f"[{a},{b},{c}]" for a, b, c in tris) + "]"
        for ket, bra in ((1, 1), (1, 2), (2, 1)):
            ana = os.path.join(tmp, f"ana_{ket}{bra}.txt")
            with open(ana, "w") as f:
                f.write(f"N={spec.n_sites}\nSz={Sz}\nT1=[" + ",".join(map(str, T1)) + "]\nT2=[" +
                        ",".join(map(str, T2)) + f"]\n{tri_txt}\nev1={ket}\nev2={bra}\n"
                        f"pEV1_file={os.path.join(tmp, 'full_pEV0.txt')}\n"
                        f"pEV2_file={os.path.join(tmp, 'full_pEV1.txt')}\n")
            out = os.path.join(tmp, f"corr_{ket}{bra}.txt")
            subprocess.run([os.path.join(REF, "pspincorr"), ana, out], check=True, stdout=subprocess.DEVNULL)
            zz, xy = [], []
            for line in open(out):
                m = re.match(r"Sz \((\d+)\) Sz \((\d+)\) = (.*)", line.strip())
                if m:
                    zz.append((int(m.group(1)), int(m.group(2)), cplx(m.group(3))))
                m = re.match(r"Sp \((\d+)\) Sm \((\d+)\) = (.*)", line.strip())
                if m:
                    xy.append((int(m.group(1)), int(m.group(2)), cplx(m.group(3))))
            store[f"szsz_{ket}{bra}"] = np.array([[a, b, v.real, v.imag] for a, b, v in zz])
            store[f"xy_{ket}{bra}"] = np.array([[a, b, v.real, v.imag] for a, b, v in xy])
        # pchirality: psi1 = pEV1 (ket), psi2 = pEV2 (bra); both files are the
        # level wanted for an expectation value
        for ket, bra in ((0, 0), (0, 1)):
            ana = os.path.join(tmp, f"chi_{ket}{bra}.txt")
            with open(ana, "w") as f:
                f.write(f"N={spec.n_sites}\nSz={Sz}\nT1=[" + ",".join(map(str, T1)) + "]\nT2=[" +
                        ",".join(map(str, T2)) + f"]\n{tri_txt}\n"
                        f"pEV1_file={os.path.join(tmp, f'full_pEV{ket}.txt')}\n"
                        f"pEV2_file={os.path.join(tmp, f'full_pEV{bra}.txt')}\n")
            out = os.path.join(tmp, f"chi_out_{ket}{bra}.txt")
            subprocess.run([os.path.join(REF, "pchirality"), ana, out], check=True, stdout=subprocess.DEVNULL)
            txt = open(out).read()
            m = re.search(r"Expectation value of chirality operator is = (\([^)]*\))", txt)
            store[f"chirality_{ket}{bra}"] = np.array([cplx(m.group(1))])
    np.savez_compressed(os.path.join(HERE, "observables.npz"), **store)
    print({k: v.shape for k, v in store.items()})


if __name__ == "__main__":
    main()
