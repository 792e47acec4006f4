"""Host side of bench.py (no GPU): the workloads it names, the DRAM traffic it
reads from the committed ncu summary, and the algorithmic bytes it divides
by, recomputed here from the formula the design notes state."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_traffic_of_the_headline_kernel_comes_from_the_profile():
    t = bench.profile_traffic("hv_stored-rows_tri6x6_k00_c64")
    assert t is not None and t == 271603818752.0
    assert bench.profile_traffic("no-such-profile") is None


def test_measured_peak_is_a_bandwidth():
    peak, kind = bench.measured_peak_hbm()
    assert kind in ("measured", "fallback") and 1000.0 < peak < 20000.0


def test_headline_workload_is_the_36_site_sector():
    from ed_code_gb300 import lattice as L

    import oracle as O

    model = bench.build_model("tri6x6_k00")
    assert model.n_sites == 36 and len(model.adj_list) == 108
    assert (model.kx, model.ky) == (0, 0) and model.Jz == 1.0 and model.Ch == 0.15
    assert O.sector_dim(model) == 252091362
    assert isinstance(model, L.Model)


def test_stored_row_algorithmic_bytes_at_36_sites():
    """n_p(2S+1) + nnz(S+E) + 8(n_p+1) + 8 n_p + n_p(2S+1) with S = 8 (complex64)
    and E = 4 (packed entries) is the 180,627,150,524 B the bench reports."""
    n_p, nnz, S, E = 252091362, 14001881868, 8, 4
    B = n_p * (2 * S + 1) + nnz * (S + E) + 8 * (n_p + 1) + 8 * n_p + n_p * (2 * S + 1)
    assert B == 180627150524


@pytest.mark.parametrize("argv", [["--mode", "gather-peak", "--hint", "2"], ["--serve-tile", "x"]])
def test_bad_arguments_are_rejected(argv, monkeypatch):
    monkeypatch.setattr(sys, "argv", ["bench.py"] + argv)
    with pytest.raises(SystemExit):
        bench.main()
