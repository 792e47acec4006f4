"""Host side of bench.py (no GPU): the workloads it names, the DRAM traffic it
reads from profiles/traffic.json (written from ncu CSV logs by
`bench.py --ingest-ncu`), and the algorithmic bytes it divides by,
recomputed here from the formula the design notes state."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_traffic_of_the_headline_kernel_comes_from_the_data_file():
    t = bench.profile_traffic("hv_stored-rows_tri6x6_k00_c64")
    assert t is not None and 1e11 < t < 1e12
    assert bench.profile_traffic("no-such-profile") is None


_METRICS_CSV = """==PROF== Connected to process 1
"ID","Process ID","Process Name","Host Name","Kernel Name","Context","Stream","Block Size","Grid Size","Device","CC","Section Name","Metric Name","Metric Unit","Metric Value"
"0","1","python","h","void edg::k_hv_csr<float, 8>(int)","1","7","(256, 1, 1)","(304, 1, 1)","0","10.3","Command line profiler metrics","dram__bytes_read.sum","Gbyte","2.50"
"0","1","python","h","void edg::k_hv_csr<float, 8>(int)","1","7","(256, 1, 1)","(304, 1, 1)","0","10.3","Command line profiler metrics","dram__bytes_write.sum","Mbyte","500.00"
"0","1","python","h","void edg::k_hv_csr<float, 8>(int)","1","7","(256, 1, 1)","(304, 1, 1)","0","10.3","Command line profiler metrics","gpu__time_duration.sum","msecond","1.00"
"1","1","python","h","void edg::k_u_scale<float>(int)","1","7","(256, 1, 1)","(304, 1, 1)","0","10.3","Command line profiler metrics","dram__bytes_read.sum","Gbyte","9.00"
"2","1","python","h","void edg::k_hv_csr<float, 8>(int)","1","7","(256, 1, 1)","(304, 1, 1)","0","10.3","Command line profiler metrics","dram__bytes_read.sum","Gbyte","3.50"
"2","1","python","h","void edg::k_hv_csr<float, 8>(int)","1","7","(256, 1, 1)","(304, 1, 1)","0","10.3","Command line profiler metrics","dram__bytes_write.sum","Mbyte","500.00"
"""


def test_ingest_ncu_averages_launches_and_scales(tmp_path, monkeypatch):
    csv = tmp_path / "dram.csv"
    csv.write_text(_METRICS_CSV)
    out = tmp_path / "traffic.json"
    monkeypatch.setattr(bench, "TRAFFIC_FILE", str(out))
    rec = bench.ingest_ncu(str(csv), "t1", "k_hv_csr", 2.0, "test")
    assert rec["launches"] == 2 and rec["captured_bytes_per_launch"] == pytest.approx(3.5e9)
    assert rec["dram_bytes_per_launch"] == pytest.approx(7.0e9)
    assert bench.profile_traffic("t1") == pytest.approx(7.0e9)
    with pytest.raises(SystemExit):
        bench.ingest_ncu(str(csv), "t2", "no_such_kernel", 1.0, "")


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


@pytest.mark.parametrize("argv", [["--mode", "gather-peak"], ["--serve-tile", "x"], ["--ingest-ncu", "x.csv"]])
def test_bad_arguments_are_rejected(argv, monkeypatch):
    monkeypatch.setattr(sys, "argv", ["bench.py"] + argv)
    with pytest.raises(SystemExit):
        bench.main()


def test_roofline_record_by_both_byte_counts():
    """frac by the kernel's bytes, base_frac by the problem's own bytes, and
    traffic over the kernel's bytes, all against the same peak."""
    r = bench.roofline_record(180.6e9, 118.3e9, 60.4, 6673.5, "measured", 272.6e9)
    assert r["achieved"] == pytest.approx(180.6e9 / 0.0604 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / 6673.5)
    assert r["base_frac"] == pytest.approx(118.3e9 / 0.0604 / 1e9 / 6673.5)
    assert r["traffic_over_algorithmic"] == pytest.approx(272.6 / 180.6)
    assert bench.roofline_record(1e9, 1e9, 1.0, 1000.0, "fallback", None)["traffic_over_algorithmic"] is None
