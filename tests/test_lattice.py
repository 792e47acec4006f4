"""Torus generators and the parser mirror of the reference input format."""
import numpy as np
import pytest

from ed_code_gb300 import lattice as L


@pytest.mark.parametrize("lat,Lx,Ly,nb,ntri", [("square", 4, 4, 32, 0), ("triangular", 6, 5, 90, 60),
                                               ("triangular", 6, 6, 108, 72), ("triangular", 5, 4, 60, 40)])
def test_torus_counts(lat, Lx, Ly, nb, ntri):
    spec = L.TorusSpec(lat, Lx, Ly, Ch=0.2 if lat == "triangular" else 0.0)
    m = L.make_model(spec)
    assert m.n_sites == Lx * Ly
    assert len(m.adj_list) == nb
    assert len(m.ch_list) == 3 * ntri
    assert sorted(m.T1) == list(range(Lx * Ly)) and sorted(m.T2) == list(range(Lx * Ly))


def test_nnn_bond_counts():
    assert len(L.make_model(L.TorusSpec("square", 4, 4, J2=0.3)).adj_list) == 64
    assert len(L.make_model(L.TorusSpec("triangular", 5, 4, J2=0.3, Ch=0.1)).adj_list) == 120


def test_triangles_are_counter_clockwise():
    """Cross product of the two edges from the first vertex is positive (a2 at 60 degrees)."""
    a1, a2 = np.array([1.0, 0.0]), np.array([0.5, np.sqrt(3) / 2])
    for x, y in [(0, 0), (2, 1)]:
        for tri in ([(x, y), (x + 1, y), (x, y + 1)], [(x + 1, y), (x + 1, y + 1), (x, y + 1)]):
            p = [i * a1 + j * a2 for i, j in tri]
            e1, e2 = p[1] - p[0], p[2] - p[0]
            assert e1[0] * e2[1] - e1[1] * e2[0] > 0


def test_chirality_entries_are_cyclic_and_phase_from_bond():
    spec = L.TorusSpec("triangular", 4, 3, Ch=0.2, bond_phases=[0.3, -0.5, 1.1] * 12)
    m = L.make_model(spec)
    t1, t2, t3 = m.ch_list[0:3]
    assert (t2.i, t2.j, t2.k) == (t1.j, t1.k, t1.i)
    assert (t3.i, t3.j, t3.k) == (t1.k, t1.i, t1.j)
    # the phase of entry (i,j,k) is the phase of bond i-j as seen from i
    bond = {(b.x, b.y): b.expphase for b in m.adj_list}
    for t in m.ch_list:
        e = bond.get((t.i, t.j), None)
        e = e if e is not None else bond[(t.j, t.i)].conjugate()
        assert abs(t.expphase - e) < 1e-15


def test_parser_reads_sector_and_solver_keys():
    text = L.input_file_text(L.TorusSpec("square", 4, 4), Sz=1, kx=2, ky=3, num_eigenvalues=5, tol=1e-9,
                             iterations=77, ncycles=4)
    m = L.parse_input_text(text)
    assert (m.Sz, m.kx, m.ky, m.num_eigenvalues) == (1.0, 2, 3, 5)
    assert (m.tol, m.lanczos_iterations, m.lanczos_ncycles) == (1e-9, 77, 4)
    assert m.n_ones == 9


def test_parser_rejects_mismatched_translations():
    with pytest.raises(ValueError):
        L.parse_input_text("T1=[1,0]\nT2=[0]\n")


def test_bowties_only_when_triangles_neighbour():
    m = L.make_model(L.TorusSpec("triangular", 4, 3, Ch=0.2, ChCh=0.1))
    ntri = len(m.ch_list) // 3
    assert len(m.chch_list) % 9 == 0 and 0 < len(m.chch_list) <= 9 * ntri * (ntri - 1)


def test_cubic_torus_round_trip():
    spec = L.TorusSpec("cubic", 4, 2, Lz=3, Jz=0.9, Ch=0.2)
    m = L.make_model(spec, 1, 2, 1, kz=2)
    assert m.n_sites == 24 and m.kz == 2 and (m.kx, m.ky, m.Sz) == (2, 1, 1.0)
    T1, T2, T3 = L.translations3(4, 2, 3)
    assert (m.T1, m.T2, m.T3) == (T1, T2, T3)
    # every site has 6 neighbours on a 4x2x3 torus, the y direction (length 2) counting once
    assert len(m.adj_list) == 24 * 3 - 24 // 2
    assert len(m.ch_list) == 3 * 24
    text = L.input_file_text(spec, 1, 2, 1, kz=2)
    assert "T3=[" in text and "kz=2" in text
    assert L.parse_input_text(text).T3 == T3
    assert "T3=" not in L.input_file_text(L.TorusSpec("square", 4, 4))
