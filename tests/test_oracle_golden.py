"""The CPU restatement (oracle/) against the reference's own outputs.

The fixtures in tests/golden/ were produced by the reference compiled from its
sources (tests/golden/make_golden.py).  These tests pin the oracle before it is
used as the checker of the GPU library.
"""
import hashlib

import numpy as np
import pytest

from conftest import all_golden_sectors, golden_arrays, golden_cases, golden_model

import oracle as O


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("name,idx", all_golden_sectors(max_configs=3_000_000))
def test_oracle_tables_match_reference(name, idx):
    meta = golden_cases()[name]["sectors"][idx]
    model = golden_model(name, idx)
    sec = O.OracleSector(model)
    assert sec.n_p == meta["n_p"]
    assert (sec.L1, sec.L2) == (meta["L1"], meta["L2"])
    assert sec.bits_right == meta["bits_right"]
    # integer tables: bit-exact
    assert sha(sec.states) == meta["sha_states"]
    assert sha(sec.rep_loc) == meta["sha_rep_loc"]
    assert sha(sec.Ia) == meta["sha_Ia"]
    assert sha(sec.Ib) == meta["sha_Ib"]
    # norms are correctly rounded sqrt of integers: bit-exact too
    assert sha(sec.norm) == meta["sha_norm"]
    g = golden_arrays(name)
    tag = f"s{idx}"
    if meta["full"]:
        np.testing.assert_array_equal(sec.state_ph, g[f"{tag}_state_ph"])
    else:
        cfg = g[f"{tag}_cfg"]
        np.testing.assert_allclose(sec.state_ph[cfg], g[f"{tag}_state_ph_at_cfg"], rtol=0, atol=1e-15)


@pytest.mark.parametrize("name,idx", all_golden_sectors(max_configs=3_000_000))
def test_oracle_hv_matches_reference(name, idx):
    meta = golden_cases()[name]["sectors"][idx]
    model = golden_model(name, idx)
    sec = O.OracleSector(model)
    g = golden_arrays(name)
    tag = f"s{idx}"
    for k, seed in enumerate(meta["vec_seeds"]):
        v = O.splitmix_vector(sec.n_p, seed)
        w = sec.hv(v)
        if meta["full"]:
            ref = g[f"{tag}_w{k}"]
            np.testing.assert_allclose(w, ref, rtol=0, atol=1e-13 * max(1.0, np.abs(ref).max()))
        else:
            rows = g[f"{tag}_rows"]
            ref = g[f"{tag}_w{k}_at_rows"]
            np.testing.assert_allclose(w[rows], ref, rtol=0, atol=1e-12)
            other = O.splitmix_vector(sec.n_p, meta["vec_seeds"][(k + 1) % len(meta["vec_seeds"])])
            assert abs(w.sum() - g[f"{tag}_w{k}_sum"][0]) < 1e-9 * np.sqrt(sec.n_p)
            assert abs(np.vdot(w, w).real - g[f"{tag}_w{k}_norm2"][0]) < 1e-10 * g[f"{tag}_w{k}_norm2"][0]
            assert abs(np.vdot(other, w) - g[f"{tag}_w{k}_proj"][0]) < 1e-9 * np.sqrt(sec.n_p)


@pytest.mark.parametrize("name,idx", [(n, i) for n, i in all_golden_sectors(max_configs=20000)])
def test_oracle_dense_spectrum_matches_reference(name, idx):
    """The reference's dense path (makeH + zheev, n_p <= 10000) printed these eigenvalues."""
    meta = golden_cases()[name]["sectors"][idx]
    if "ed2_eigs" not in meta or meta["n_p"] > 2000:
        pytest.skip("no dense reference spectrum for this sector")
    sec = O.OracleSector(golden_model(name, idx))
    H = sec.dense()
    assert np.abs(H - H.conj().T).max() < 1e-13
    ev = np.linalg.eigvalsh(H)
    ref = np.array(meta["ed2_eigs"])
    np.testing.assert_allclose(ev[: len(ref)], ref, rtol=0, atol=1e-11)


def test_oracle_sector_dim_formula():
    """The character count of the dimension agrees with enumeration."""
    for name, idx in all_golden_sectors():
        meta = golden_cases()[name]["sectors"][idx]
        assert O.sector_dim(golden_model(name, idx)) == meta["n_p"]


def test_oracle_hv_rows_match_tables():
    """Row mode (orbit walk + binary search, used where tables do not fit) equals table mode."""
    for name, idx in [("tri4x3_chch", 0), ("sq4x4_phase_sz1", 0), ("tri4x3_relabel", 1), ("tri5x4_j2", 1)]:
        model = golden_model(name, idx)
        sec = O.OracleSector(model)
        v = O.splitmix_vector(sec.n_p, 5)
        w = sec.hv(v)
        rows = np.arange(0, sec.n_p, 7)
        wr = O.hv_rows(model, sec.states, sec.lid, v, rows)
        np.testing.assert_allclose(wr, w[rows], rtol=0, atol=1e-13)


def test_splitmix_vector_is_deterministic():
    a = O.splitmix_vector(1000, 3)
    b = O.splitmix_vector(1000, 3)
    assert np.array_equal(a, b)
    assert np.abs(a.real).max() <= 1 and np.abs(a.imag).max() <= 1
    assert not np.array_equal(a, O.splitmix_vector(1000, 4))


def test_listless_rows_equal_list_rows():
    """The list-free row mode (used where the representative list cannot be
    built on the host) gives the same rows as the list mode with the same v."""
    from ed_code_gb300 import lattice as L

    for spec, sec in [(L.TorusSpec("triangular", 4, 3, Jz=0.9, Ch=0.3), (0, 1, 2)),
                      (L.TorusSpec("square", 4, 4, Jz=1.1, J2=0.4), (1, 1, 3))]:
        model = L.make_model(spec, *sec)
        reps, lid = O.build_reps(model)
        v = O.value_vector(reps, 99)
        rows = np.arange(0, len(reps), 3)
        a = O.hv_rows(model, reps, lid, v, rows)
        b = O.hv_rows_listless(model, reps[rows], lid[rows], 99)
        assert np.array_equal(a, b)
        # the rank-lookup stand-in of the reference arm (a binary search in a
        # sorted array of the list's size) costs time but changes no value
        probe = O.sorted_probe(len(reps), int(reps.min()), int(reps.max()) + 1)
        assert len(probe) == len(reps) and np.all(np.diff(probe) > 0) and probe[0] >= reps.min()
        c = O.hv_rows_listless(model, reps[rows], lid[rows], 99, probe=probe)
        assert np.array_equal(a, c)
        s, sl = O.sample_reps(model, 50, seed=5)
        assert len(s) == 50 and np.all(np.isin(s, reps))
        assert np.array_equal(sl, lid[np.searchsorted(reps, s)])
