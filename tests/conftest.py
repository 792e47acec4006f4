"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on CPU."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libedgpu.so")
    config.addinivalue_line("markers", "slow: long-running")


def golden_cases():
    with open(os.path.join(GOLDEN, "cases.json")) as f:
        return json.load(f)


def golden_arrays(name):
    return np.load(os.path.join(GOLDEN, f"{name}.npz"))


def golden_model(name, sector_index):
    """lattice.Model of a golden case's sector, built the way the fixture script built it."""
    from ed_code_gb300 import lattice as L

    meta = golden_cases()[name]
    s = meta["sectors"][sector_index]
    spec = L.TorusSpec(**meta["spec"])
    extra = dict(kz=s.get("kz", 0)) if spec.lattice == "cubic" else {}
    return L.make_model(spec, s["Sz"], s["kx"], s["ky"], **extra)


def all_golden_sectors(max_configs=None, full_only=False):
    out = []
    for name, meta in sorted(golden_cases().items()):
        for i, s in enumerate(meta["sectors"]):
            if full_only and not s["full"]:
                continue
            if max_configs is not None and s["n_configs"] > max_configs:
                continue
            out.append((name, i))
    return out


@pytest.fixture(scope="session")
def cuda_device():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
