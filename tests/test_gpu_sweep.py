"""All-sectors sweep against the reference's eigenvalues (ED2, Sz=0, every
momentum of the 4x3 triangular torus) and the oracle's dense spectra (Sz>0)."""
import numpy as np
import pytest

from conftest import golden_cases

import oracle as O

pytestmark = pytest.mark.gpu


def test_sweep_every_sector(cuda_device):
    from ed_code_gb300 import lattice as L
    from ed_code_gb300 import sweep as W

    spec = L.TorusSpec("triangular", 4, 3, Jz=0.8, Ch=0.2)
    levels = W.sweep(spec, n_ev=3, max_iterations=120, res_tol=1e-6)
    E = np.array([q.En for q in levels])
    assert np.all(np.diff(E) >= -1e-15)
    # every (Sz >= 0, k) sector that has states contributed
    assert {(q.Sz, q.kx, q.ky) for q in levels if q.Sz == 0} == {(0.0, kx, ky) for kx in range(4) for ky in range(3)}
    assert max(q.Sz for q in levels) == 6.0
    # Sz = 0 against the reference's ED2, sector by sector (levels counted once)
    gold = golden_cases()["tri4x3"]["sectors"]
    for g in gold:
        got = sorted(q.En for q in levels if q.Sz == 0 and (q.kx, q.ky) == (g["kx"], g["ky"]))
        ref = []
        for x in g["ed2_eigs"]:
            if not ref or abs(x - ref[-1]) > 1e-9 * abs(x):
                ref.append(x)
        assert len(got) == 3
        np.testing.assert_allclose(got, ref[:3], rtol=1e-9)
    # Sz = 1 and Sz = 2 against the oracle's dense spectra
    for Sz in (1.0, 2.0):
        for kx, ky in [(0, 0), (1, 2), (3, 1)]:
            m = L.make_model(spec, Sz, kx, ky)
            ev = np.linalg.eigvalsh(O.OracleSector(m).dense())
            ref = []
            for x in ev:
                if not ref or abs(x - ref[-1]) > 1e-9 * abs(x):
                    ref.append(x)
            got = sorted(q.En for q in levels if q.Sz == Sz and (q.kx, q.ky) == (kx, ky))
            n = min(len(got), 3)
            np.testing.assert_allclose(got[:n], ref[:n], rtol=1e-9)
    # the ids keep the collection order; the ground state comes first
    assert sorted(q.id for q in levels) == list(range(len(levels)))
    assert levels[0].En == E.min()
    txt = W.table(levels, 12, 0.8, 0.0)
    assert txt.count("\n") >= len(levels)
