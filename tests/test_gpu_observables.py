"""Observables between momentum eigenvectors against the reference's own
operator definitions (chirality_exp.cpp: szsz_op, sxsxsysy_op, ch_op, and
pchirality.cpp's factor i) evaluated in the fixed-Sz basis after unwrapping."""
import cmath

import numpy as np
import pytest

from conftest import golden_model

pytestmark = pytest.mark.gpu


def unwrap(model, states, norm, coeff):
    """Fixed-Sz amplitudes of a momentum vector: each representative's orbit
    walked in the reference's order (Unwrap_pState, Momentum_Basis.cpp:978-1037)
    with its phases; a state reached lid times is divided by lid so that the
    result is normalised like the momentum basis itself."""
    from ed_code_gb300 import observables

    T1, T2 = model.T1, model.T2
    G = observables.translations(model)
    L1 = 1
    s = T1[0]
    while s != 0:
        s, L1 = T1[s], L1 + 1
    L2 = len(G) // L1
    px, py = 2 * np.pi * model.kx / L1, 2 * np.pi * model.ky / L2
    ex, ey = cmath.exp(-1j * px), cmath.exp(-1j * py)

    def tr(v, T):
        out = 0
        for i in range(model.n_sites):
            if (v >> i) & 1:
                out |= 1 << T[i]
        return out

    psi = {}
    for r, nr, c in zip(states, norm, coeff):
        loc = {}
        v, ph = int(r), 1.0 + 0j
        loc[v] = loc.get(v, 0) + c * ph / nr
        for x in range(L1):
            if x > 0:
                v, ph = tr(v, T1), ph * ex
                loc[v] = loc.get(v, 0) + c * ph / nr
            for _ in range(1, L2):
                v, ph = tr(v, T2), ph * ey
                loc[v] = loc.get(v, 0) + c * ph / nr
        lid = round(L1 * L2 / nr ** 2)
        for k, a in loc.items():
            psi[k] = psi.get(k, 0) + a / lid
    return psi


def bit(c, i):
    return (c >> i) & 1


def szsz(psi1, psi2, i, j):
    return sum((bit(c, i) - 0.5) * (bit(c, j) - 0.5) * np.conj(psi2.get(c, 0)) * a for c, a in psi1.items())


def sxsx(psi1, psi2, i, j):
    s = 0
    for c, a in psi1.items():
        if bit(c, i) != bit(c, j):
            s += np.conj(psi2.get(c ^ ((1 << i) | (1 << j)), 0)) * a
    return 0.5 * s


def ch_op(psi1, psi2, i, j, k):
    s = 0
    for c, a in psi1.items():
        if bit(c, i) != bit(c, j):
            sgn = 1 if bit(c, k) else -1
            t = c ^ ((1 << i) | (1 << j))
            s += (-0.25 if bit(c, j) == 0 else 0.25) * sgn * np.conj(psi2.get(t, 0)) * a
    return s


@pytest.fixture(scope="module")
def states(cuda_device):
    from ed_code_gb300 import sector

    model = golden_model("tri4x3", 0)
    sec = sector.GpuSector(model)
    eigs, vecs, _ = sec.solve_plain(n_ev=2, want_vectors=True)
    reps, norm, _ = sec.basis()
    return model, eigs, vecs, reps, norm


def test_spin_correlations_and_chirality(states):
    from ed_code_gb300 import observables as Ob

    model, eigs, vecs, reps, norm = states
    psi0 = unwrap(model, reps, norm, vecs[0])
    psi1 = unwrap(model, reps, norm, vecs[1])
    assert abs(sum(abs(a) ** 2 for a in psi0.values()) - 1) < 1e-12
    pairs = [(0, 1), (0, 5), (2, 7), (3, 11)]
    got = Ob.spin_correlations(model, pairs, vecs[0])
    mixed = Ob.spin_correlations(model, pairs, vecs[1], bra=vecs[0])
    for (i, j) in pairs:
        assert abs(got[(i, j)]["SzSz"] - szsz(psi0, psi0, i, j)) < 1e-12
        assert abs(got[(i, j)]["SxSx+SySy"] - sxsx(psi0, psi0, i, j)) < 1e-12
        assert abs(mixed[(i, j)]["SzSz"] - szsz(psi1, psi0, i, j)) < 1e-12
        assert abs(mixed[(i, j)]["SxSx+SySy"] - sxsx(psi1, psi0, i, j)) < 1e-12
    tris = [(t.i, t.j, t.k) for t in model.ch_list[::3]]
    ref = 0
    for (i, j, k) in tris:
        ref += ch_op(psi0, psi0, i, j, k) + ch_op(psi0, psi0, j, k, i) + ch_op(psi0, psi0, k, i, j)
    assert abs(Ob.chirality(model, tris, vecs[0]) - 1j * ref) < 1e-12
    # the energy from the bond correlations and the chirality
    e = 0
    corr = Ob.spin_correlations(model, [(b.x, b.y) for b in model.adj_list], vecs[0])
    for b in model.adj_list:
        c = corr[(b.x, b.y)]
        e += b.J * (c["SxSx+SySy"] + model.Jz * c["SzSz"])
    e -= model.Ch * Ob.chirality(model, tris, vecs[0])
    assert abs(e - eigs[0]) < 1e-10 * abs(eigs[0])


def test_observables_match_the_reference_analysis_programs(cuda_device):
    """Pinned to the reference's own analysis programs: pspincorr and
    pchirality (analysis/src, compiled from the reference's sources) read the
    two lowest eigenvectors ED2 wrote for the 4x3 triangular sector at k=(1,1)
    and printed <bra|Sz_i Sz_j|ket>, <bra|SxSx+SySy|ket> and the chirality
    (tests/golden/make_observables.py).  They print six significant digits,
    which sets the tolerance."""
    import os

    from ed_code_gb300 import lattice as L
    from ed_code_gb300 import observables
    from ed_code_gb300.sector import GpuSector

    fix = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "observables.npz"))
    model = L.make_model(L.TorusSpec("triangular", 4, 3, Jz=0.8, Ch=0.2), 0, 1, 1)
    sec = GpuSector(model)
    states, _, _ = sec.basis()
    assert np.array_equal(states, fix["states"])
    sec.close()
    vec = [fix["vec0"] / np.linalg.norm(fix["vec0"]), fix["vec1"] / np.linalg.norm(fix["vec1"])]

    def close(got, want):
        assert abs(got - want) <= 1e-5 * abs(want) + 2e-6, (got, want)

    for tag, (ket, bra) in {"11": (0, 0), "12": (0, 1), "21": (1, 0)}.items():
        zz, xy = fix[f"szsz_{tag}"], fix[f"xy_{tag}"]
        pairs = sorted({(int(a), int(b)) for a, b, _, _ in zz})
        res = observables.spin_correlations(model, pairs, ket=vec[ket], bra=vec[bra])
        for a, b, re, im in zz:
            close(res[(int(a), int(b))]["SzSz"], complex(re, im))
        for a, b, re, im in xy:
            close(res[(int(a), int(b))]["SxSx+SySy"], complex(re, im))
    tris = [tuple(int(x) for x in t) for t in fix["triangles"]]
    for tag, (ket, bra) in {"00": (0, 0), "01": (0, 1)}.items():
        close(observables.chirality(model, tris, ket=vec[ket], bra=vec[bra]), complex(fix[f"chirality_{tag}"][0]))
