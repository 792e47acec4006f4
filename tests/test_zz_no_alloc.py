"""edg_hv_noalloc, the H*v entry point that allocates no device memory.

It is meant for callers whose own allocator holds the device's free memory,
or whose loop cannot afford the device synchronisation of cudaMalloc/cudaFree.
Its u = v/norm scratch is a fixed 16 MiB array in the library's device image
shared by every call, so the checks below run it twice in a row on the same
stream (the second call reuses what the first left in the array), then on a
smaller sector, and compare each result with edg_hv on the same input: 1e-13
relative to max|w| in FP64, 2e-5 in FP32, the tolerances of the other H*v
parity tests.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import golden_model

pytestmark = pytest.mark.gpu

TOL = {"complex128": 1e-13, "complex64": 2e-5}


@pytest.fixture(scope="module")
def sectors(cuda_device):
    from ed_code_gb300 import lattice as L
    from ed_code_gb300 import sector

    big = sector.GpuSector(golden_model("sq6x4_k00", 0))  # 112,800 states
    small = sector.GpuSector(L.make_model(L.TorusSpec("triangular", 5, 4, Jz=1.1, J2=0.3, Ch=0.2), 0, 2, 1))
    assert big.build_targets() and small.build_targets()
    return big, small


def _hv(fn, sec, v, w, stream):
    from ed_code_gb300 import _native as N
    import torch

    code = N.EDG_C128 if v.dtype == torch.complex128 else N.EDG_C64
    N.check(fn(sec._h, C.c_void_p(v.data_ptr()), C.c_void_p(w.data_ptr()), code, C.c_void_p(stream)))


def _rand(n, dtype, seed):
    import torch

    g = torch.Generator(device="cuda").manual_seed(seed)
    return torch.randn(n, dtype=dtype, device="cuda", generator=g)


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_noalloc_matches_edg_hv_on_consecutive_calls(sectors, dtype):
    import torch
    from ed_code_gb300 import _native as N

    lib = N.lib()
    tdt = getattr(torch, dtype)
    st = torch.cuda.current_stream().cuda_stream
    big, small = sectors
    cases = [(big, 11), (big, 12), (small, 13), (small, 14)]
    vs = [_rand(sec.n_p, tdt, seed) for sec, seed in cases]
    # the four calls are enqueued back to back, with no synchronisation between them
    outs = [torch.empty_like(v) for v in vs]
    for (sec, _), v, w in zip(cases, vs, outs):
        _hv(lib.edg_hv_noalloc, sec, v, w, st)
    refs = [torch.empty_like(v) for v in vs]
    for (sec, _), v, w in zip(cases, vs, refs):
        _hv(lib.edg_hv, sec, v, w, st)
    torch.cuda.synchronize()
    for w, ref in zip(outs, refs):
        a, b = w.cpu().numpy().astype(np.complex128), ref.cpu().numpy().astype(np.complex128)
        assert np.isfinite(a).all()
        assert np.abs(a - b).max() / max(1.0, np.abs(b).max()) <= TOL[dtype]


@pytest.mark.parametrize("dtype", ["complex128", "complex64"])
def test_noalloc_reads_both_entry_formats(cuda_device, monkeypatch, dtype):
    """Stored rows come packed (column and value id in one u32) or split (two
    arrays, EDG_ROW_FORMAT=split): the call reads either."""
    import torch
    from ed_code_gb300 import _native as N
    from ed_code_gb300 import sector

    lib = N.lib()
    tdt = getattr(torch, dtype)
    st = torch.cuda.current_stream().cuda_stream
    monkeypatch.setenv("EDG_ROW_FORMAT", "split")
    split = sector.GpuSector(golden_model("tri6x4_k10", 0))
    assert split.build_targets() and split.info["entry_bytes"] == 6
    monkeypatch.delenv("EDG_ROW_FORMAT")
    packed = sector.GpuSector(golden_model("tri6x4_k10", 0))
    assert packed.build_targets() and packed.info["entry_bytes"] == 4
    v = _rand(split.n_p, tdt, 21)
    outs = {}
    for name, sec in (("split", split), ("packed", packed)):
        w = torch.empty_like(v)
        _hv(lib.edg_hv_noalloc, sec, v, w, st)
        ref = torch.empty_like(v)
        _hv(lib.edg_hv, sec, v, ref, st)
        torch.cuda.synchronize()
        a, b = w.cpu().numpy().astype(np.complex128), ref.cpu().numpy().astype(np.complex128)
        assert np.abs(a - b).max() / max(1.0, np.abs(b).max()) <= TOL[dtype], name
        outs[name] = a
    assert np.array_equal(outs["split"], outs["packed"])


def test_noalloc_rejects_what_it_cannot_serve(cuda_device):
    import torch
    from ed_code_gb300 import _native as N
    from ed_code_gb300 import lattice as L
    from ed_code_gb300 import sector

    lib = N.lib()
    st = torch.cuda.current_stream().cuda_stream
    # about 5.2 million states: more than the fixed scratch holds in either precision
    large = sector.GpuSector(L.make_model(L.TorusSpec("triangular", 6, 5, Jz=0.8, Ch=0.2), 0, 2, 3))
    assert large.n_p > 2_097_152
    v = torch.zeros(large.n_p, dtype=torch.complex64, device="cuda")
    w = torch.empty_like(v)
    with pytest.raises(N.EdgError, match="at most 2097152 complex64"):
        _hv(lib.edg_hv_noalloc, large, v, w, st)
    large.close()
    # a sector without stored rows
    plain = sector.GpuSector(golden_model("tri4x3", 0))
    v = torch.zeros(plain.n_p, dtype=torch.complex128, device="cuda")
    w = torch.empty_like(v)
    with pytest.raises(N.EdgError, match="stored rows"):
        _hv(lib.edg_hv_noalloc, plain, v, w, st)
