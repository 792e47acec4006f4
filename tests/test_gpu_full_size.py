"""The headline benchmark's sector at full size: 6x6 triangular torus, N=36,
J1=1, Delta=1, Jchi=0.15, Sz=0, k=Gamma, 252,091,362 states.

The reference cannot build this sector (its per-configuration tables would
take about 217 GB), so the checks are size-independent properties and rows
sampled from the oracle's tableless row formula:
  * the dimension equals the oracle's independent character count;
  * the basis is strictly ascending and sampled rows are allowed
    representatives with the oracle's stabiliser count;
  * H*v on sampled rows equals the oracle's rows: the matrix-free kernel in
    FP32, the stored rows in FP64 and in FP32 with the benchmark's kernel
    configuration (8 lanes, 2 CTAs per SM, pipelined);
  * Hermiticity, <u|Hv> = conj(<v|Hu>), over the whole sector in FP64.
Tolerances as in the parity tests: 1e-13 (FP64) and 2e-5 (FP32) of max|w|.
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-13
FP32_TOL = 2e-5


def test_36_site_sector_at_full_size(cuda_device):
    import torch
    from ed_code_gb300 import lattice as L
    from ed_code_gb300 import sector

    model = L.make_model(L.TorusSpec("triangular", 6, 6, Jz=1.0, Ch=0.15), 0, 0, 0)
    sec = sector.GpuSector(model)
    assert sec.n_p == O.sector_dim(model) == 252091362
    states, norm, _ = sec.basis()
    assert np.all(np.diff(states) > 0)
    lid = np.rint(model.n_sites / norm.astype(np.float64) ** 2).astype(np.int32)
    del norm
    rng = np.random.default_rng(36)
    rows = np.sort(rng.choice(sec.n_p, size=256, replace=False))
    for r in rows[:32]:
        assert O.allowed_rep(model, int(states[r])) == lid[r]

    dev = torch.device("cuda", 0)
    v = torch.empty(sec.n_p, dtype=torch.complex128, device=dev)
    sector.fill_random(v, 11)
    v_host = v.cpu().numpy()
    ref = O.hv_rows(model, states, lid, v_host, rows)
    del states, lid
    scale = max(1.0, np.abs(ref).max())
    idx = torch.from_numpy(rows).to(dev)

    v32 = v.to(torch.complex64)
    w32 = torch.empty_like(v32)
    sec.hv(v32, w32)  # matrix-free
    assert np.abs(w32[idx].cpu().numpy() - ref).max() / scale <= FP32_TOL

    assert sec.build_targets() and sec.info["entry_bytes"] == 4
    w = torch.empty_like(v)
    sec.hv(v, w)
    assert np.abs(w[idx].cpu().numpy() - ref).max() / scale <= FP64_TOL
    sec.set_rows(8, 2, 2, 1)
    sec.hv(v32, w32)
    assert np.abs(w32[idx].cpu().numpy() - ref).max() / scale <= FP32_TOL
    del v32, w32

    u = torch.empty_like(v)
    sector.fill_random(u, 12)
    hu = torch.empty_like(v)
    sec.hv(u, hu)
    lhs = torch.vdot(u, w).item()
    rhs = np.conj(torch.vdot(v, hu).item())
    assert abs(lhs - rhs) <= 1e-11 * np.sqrt(sec.n_p) * scale, (lhs, rhs)
