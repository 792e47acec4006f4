"""The device tridiagonal eigensolve against the reference's zheev.

tests/golden/tridiag.npz holds Lanczos T matrices recorded from the
reference's own recurrence (reference sHv and BLAS-1 helpers, no
reorthogonalisation, so converged levels repeat as near-copies) and, for
prefixes T_k, the eigenpairs zheev('V','U') returns for the complex matrix the
reference assembles (lanczos.cpp:271-286) -- through the OpenBLAS the
reference is linked against (make_tridiag.py).  The device kernels
(edg_tridiag_lowest: multisection bisection, inverse iteration, FP64) must
agree to 1e-12 relative in the eigenvalues; eigenvectors are compared where
the eigenvalue is isolated, and by residual everywhere.  With the copy filter
the kept Ritz values must be those a restatement of the Cullum-Willoughby
test picks from zheev's spectra of T and T-hat.
"""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = np.load(os.path.join(HERE, "golden", "tridiag.npz"))
CASES = sorted({k.rsplit("_alpha", 1)[0] for k in FIX.files if k.endswith("_alpha")})
EIG_TOL = 1e-12


def _cases():
    for name in CASES:
        for k in FIX[f"{name}_prefixes"]:
            yield name, int(k)


def _t(name, k):
    alpha, beta = FIX[f"{name}_alpha"], FIX[f"{name}_beta"]
    d = np.ascontiguousarray(alpha[:k].real)
    e = np.zeros(k)
    e[1:] = beta[1:k]
    return d, e


def _device(d, e, k, filt):
    from ed_code_gb300 import _native as N

    m = len(d)
    eigs = np.zeros(k)
    vecs = np.zeros((k, m))
    n = C.c_int(0)
    N.check(N.lib().edg_tridiag_lowest(d.ctypes.data, e.ctypes.data, m, k, int(filt), eigs.ctypes.data,
                                       vecs.ctypes.data, C.byref(n)))
    return eigs[: n.value], vecs[: n.value]


def _dense(d, e):
    m = len(d)
    T = np.diag(d)
    T[np.arange(m - 1), np.arange(1, m)] = e[1:]
    T[np.arange(1, m), np.arange(m - 1)] = e[1:]
    return T


@pytest.mark.parametrize("name,k", list(_cases()))
def test_eigenpairs_match_zheev(cuda_device, name, k):
    d, e = _t(name, k)
    ref_w, ref_v = FIX[f"{name}_k{k}_eigs"], FIX[f"{name}_k{k}_vecs"]
    nv = ref_v.shape[1]
    w, V = _device(d, e, nv, False)
    assert len(w) == nv
    err = np.abs(w - ref_w[:nv]) / np.maximum(1.0, np.abs(ref_w[:nv]))
    assert err.max() <= EIG_TOL, (name, k, err.max())
    T = _dense(d, e)
    scale = np.abs(T).sum(axis=1).max()
    for q in range(nv):
        y = V[q]
        assert abs(np.linalg.norm(y) - 1.0) <= 1e-12
        assert np.linalg.norm(T @ y - w[q] * y) <= 1e-10 * scale
        gap = np.min(np.abs(np.delete(ref_w, q) - ref_w[q])) if len(ref_w) > 1 else np.inf
        if gap > 1e-6 * scale:  # an isolated eigenvalue: its eigenvector is unique up to a phase
            assert abs(np.vdot(ref_v[:, q], y)) >= 1 - 1e-10, (name, k, q)


def _cw_restatement(th, hat, scale, want):
    kept = []
    tol_c, tol_h = 1e-7 * scale, 1e-10 * scale
    for k in range(len(th)):
        if len(kept) >= want:
            break
        prev_close = k > 0 and abs(th[k] - th[k - 1]) < tol_c
        next_close = k + 1 < len(th) and abs(th[k + 1] - th[k]) < tol_c
        in_hat = np.any(np.abs(hat - th[k]) < tol_h)
        if in_hat and not prev_close and not next_close:
            continue
        if prev_close:
            continue
        kept.append(th[k])
    return np.array(kept)


@pytest.mark.parametrize("name", CASES)
def test_copy_filter_matches_zheev_spectra(cuda_device, name):
    import scipy.linalg as sl

    k = int(FIX[f"{name}_prefixes"][-1])
    d, e = _t(name, k)
    T = _dense(d, e)
    scale = max(1.0, np.abs(T).sum(axis=1).max())
    th = FIX[f"{name}_k{k}_eigs"][: min(72, k)]
    hat = sl.eigh(T[1:, 1:].astype(np.complex128), lower=False, driver="ev", eigvals_only=True)[: min(k - 1, len(th) + 2)]
    want = min(8, k)
    ref = _cw_restatement(th, hat, scale, want)
    got, V = _device(d, e, want, True)
    assert len(got) == len(ref) >= 1, (got, ref)
    assert np.max(np.abs(got - ref) / np.maximum(1.0, np.abs(ref))) <= EIG_TOL
    for q in range(len(got)):
        assert np.linalg.norm(T @ V[q] - got[q] * V[q]) <= 1e-10 * scale


def test_bad_arguments_are_rejected(cuda_device):
    from ed_code_gb300 import _native as N

    d = np.zeros(4)
    out = np.zeros(4)
    n = C.c_int(0)
    lib = N.lib()
    assert lib.edg_tridiag_lowest(d.ctypes.data, d.ctypes.data, 4, 0, 0, out.ctypes.data, None, C.byref(n)) != 0
    assert lib.edg_tridiag_lowest(d.ctypes.data, d.ctypes.data, 4, 5, 0, out.ctypes.data, None, C.byref(n)) != 0
    assert lib.edg_tridiag_lowest(d.ctypes.data, None, 4, 1, 0, out.ctypes.data, None, C.byref(n)) != 0
    # a 1x1 matrix needs no off-diagonal
    N.check(lib.edg_tridiag_lowest(np.array([2.5]).ctypes.data, None, 1, 1, 0, out.ctypes.data, None, C.byref(n)))
    assert n.value == 1 and out[0] == 2.5
