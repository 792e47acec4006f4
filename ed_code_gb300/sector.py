"""Python side of the GPU sector: the reference's sector surface over the C ABI.

``GpuSector(model)`` is what ``sector_lanczos`` (Lanczos_sector.cpp:15-198)
builds before it diagonalises: the (Sz, kx, ky) momentum basis, here built
and kept on the GPU.  ``sHv`` mirrors the reference's ``sHv`` (H_v.cpp:192;
H_v.h:36-57): host vectors in, host vector out.  ``hv`` applies H to CUDA
tensors already on the device.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Tuple

import numpy as np

from . import _native as N
from .lattice import Model


def _model_struct(model: Model):
    """edg_model for a lattice.Model; returns (struct, keep-alive list)."""
    n = model.n_sites
    T1 = (C.c_int * n)(*model.T1)
    T2 = (C.c_int * n)(*model.T2)
    bonds = (N.edg_bond * max(1, len(model.adj_list)))(
        *[N.edg_bond(b.x, b.y, b.J, b.expphase.real, b.expphase.imag) for b in model.adj_list])
    tris = (N.edg_triangle * max(1, len(model.ch_list)))(
        *[N.edg_triangle(t.i, t.j, t.k, t.expphase.real, t.expphase.imag) for t in model.ch_list])
    # the library ignores the bowties when ChCh is 0, so they are not copied then
    chch = model.chch_list if abs(model.ChCh) > 1e-16 else []
    bows = (N.edg_bowtie * max(1, len(chch)))(*[N.edg_bowtie(b.x, b.y, b.z, b.p, b.q, b.r) for b in chch])
    T3 = (C.c_int * n)(*model.T3) if getattr(model, "T3", None) else None
    m = N.edg_model(n, T1, T2, model.Jz, bonds, len(model.adj_list), model.Ch, tris, len(model.ch_list),
                    model.ChCh, bows, len(chch), T3)
    return m, [T1, T2, T3, bonds, tris, bows]


class GpuSector:
    """One (Sz, kx, ky) sector resident on the current CUDA device."""

    def __init__(self, model: Model, n_ones: Optional[int] = None):
        self.model = model
        self.n_ones = model.n_ones if n_ones is None else int(n_ones)
        m, self._keep = _model_struct(model)
        h = C.c_void_p()
        if getattr(model, "T3", None):
            N.check(N.lib().edg_sector_create3(C.byref(m), self.n_ones, int(model.kx), int(model.ky), int(model.kz),
                                               C.byref(h)))
        else:
            N.check(N.lib().edg_sector_create(C.byref(m), self.n_ones, int(model.kx), int(model.ky), C.byref(h)))
        self._h = h
        info = N.edg_sector_info()
        N.check(N.lib().edg_sector_get_info(self._h, C.byref(info)))
        self.info = {f: getattr(info, f) for f, _ in N.edg_sector_info._fields_}
        self.n_p = int(info.n_p)

    def refresh_info(self) -> None:
        info = N.edg_sector_info()
        N.check(N.lib().edg_sector_get_info(self._h, C.byref(info)))
        self.info = {f: getattr(info, f) for f, _ in N.edg_sector_info._fields_}

    def build_targets(self, max_bytes: int = 0) -> bool:
        """Keep the searched targets in HBM (edg_sector_build_targets).
        Returns False, leaving the sector matrix-free, when they do not fit."""
        rc = N.lib().edg_sector_build_targets(self._h, int(max_bytes))
        if rc == 5:  # EDG_ERR_NOMEM
            return False
        N.check(rc)
        self.refresh_info()
        return True

    def tune(self, lanes_per_row: int = 0):
        """Choose the lanes per stored row and the cache policy of its loads by
        timing them on this sector (0: all lane counts; 8/16/32: that count).
        Returns (lanes, [best ms for 8, 16, 32], -1 where not timed); the
        choices are also in ``info["lanes_per_row"]``, ``info["cache_policy"]``,
        ``info["ctas_per_sm"]`` and ``info["pipelined"]``."""
        ch = C.c_int()
        ms = np.zeros(3, np.float64)
        N.check(N.lib().edg_sector_tune(self._h, int(lanes_per_row), C.byref(ch), ms.ctypes.data))
        self.refresh_info()
        return ch.value, ms

    def set_rows(self, lanes_per_row: int, cache_policy: int, ctas_per_sm: int = 0, pipelined: int = 0) -> None:
        """Fix the stored-row kernel's lanes per row (8/16/32), cache policy (1/2),
        CTAs per SM (0: as many as fit) and pipelining (0/1)."""
        N.check(N.lib().edg_sector_set_rows(self._h, int(lanes_per_row), int(cache_policy), int(ctas_per_sm),
                                            int(pipelined)))
        self.refresh_info()

    def free_targets(self) -> None:
        N.check(N.lib().edg_sector_free_targets(self._h))
        self.refresh_info()

    # -- basis tables ------------------------------------------------------
    def basis(self) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
        """(pblock_states, norm, norm_inv) as pConstruct_States returns them."""
        st = np.empty(self.n_p, np.int64)
        nr = np.empty(self.n_p, np.float64)
        ni = np.empty(self.n_p, np.float64)
        N.check(N.lib().edg_sector_copy_basis(self._h, st.ctypes.data, nr.ctypes.data, ni.ctypes.data))
        return st, nr, ni

    def lin_tables(self) -> Tuple[np.ndarray, np.ndarray, int]:
        nh = 1 << (self.model.n_sites // 2)
        Ia = np.empty(nh, np.int64)
        Ib = np.empty(nh, np.int64)
        br = C.c_int64()
        N.check(N.lib().edg_sector_copy_lin_tables(self._h, Ia.ctypes.data, Ib.ctypes.data, C.byref(br)))
        return Ia, Ib, int(br.value)

    def config_tables(self, max_configs: int = 1 << 26):
        """(rep_loc, state_ph, lxly) over all C(N, n_up) configurations."""
        nc = int(self.info["n_configs"])
        rl = np.empty(nc, np.int64)
        ph = np.empty(nc, np.complex128)
        lxly = np.empty((nc, 2), np.int32)
        N.check(N.lib().edg_sector_copy_config_tables(self._h, int(max_configs), rl.ctypes.data, ph.ctypes.data,
                                                      lxly.ctypes.data))
        return rl, ph, lxly

    # -- H*v -----------------------------------------------------------------
    def sHv(self, v: np.ndarray, dtype=np.complex128) -> np.ndarray:
        """w = H v with host arrays (copies in and out inside the call)."""
        dt = np.dtype(dtype)
        if dt not in (np.complex128, np.complex64):
            raise TypeError("dtype must be complex128 or complex64")
        v = np.ascontiguousarray(v, dtype=dt)
        if v.shape != (self.n_p,):
            raise ValueError(f"v must have shape ({self.n_p},)")
        w = np.empty_like(v)
        code = N.EDG_C128 if dt == np.complex128 else N.EDG_C64
        N.check(N.lib().edg_hv_host(self._h, v.ctypes.data, w.ctypes.data, code))
        return w

    def hv(self, v, w, stream=None) -> None:
        """w = H v on CUDA tensors (complex128 or complex64, n_p entries)."""
        import torch

        if v.dtype not in (torch.complex128, torch.complex64) or w.dtype != v.dtype:
            raise TypeError("v and w must both be complex128 or both complex64")
        if not (v.is_cuda and w.is_cuda and v.is_contiguous() and w.is_contiguous()):
            raise ValueError("v and w must be contiguous CUDA tensors")
        if v.numel() != self.n_p or w.numel() != self.n_p:
            raise ValueError(f"v and w must have {self.n_p} entries")
        code = N.EDG_C128 if v.dtype == torch.complex128 else N.EDG_C64
        st = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
        N.check(N.lib().edg_hv(self._h, C.c_void_p(v.data_ptr()), C.c_void_p(w.data_ptr()), code, C.c_void_p(st)))

    def solve_plain(self, n_ev: int = 2, iterations: int = 100, ncycles: int = 10, tol: float = 1e-11,
                    seed: int = 0, dense_threshold: int = 10000, want_vectors: bool = False, log=None):
        """The sector eigensolver of sector_lanczos in FP64 (lanczos_evecs, or
        exact_evecs for n_p <= dense_threshold).  Returns (eigs, evecs, stats)."""
        dense = dense_threshold >= 0 and self.n_p <= dense_threshold
        cap = self.n_p if dense else min(n_ev, self.n_p)
        eigs = np.empty(cap, np.float64)
        nvec = (min(n_ev, self.n_p) if want_vectors else 0)
        evecs = np.empty((nvec, self.n_p), np.complex128) if nvec else None
        cb = N.LOG_FN(lambda ctx, line: log(line.decode())) if log else N.LOG_FN()
        opts = N.edg_solver_opts(int(n_ev), int(iterations), int(ncycles), float(tol), int(seed),
                                 int(dense_threshold), cb, None)
        n_out = C.c_int64()
        st = N.edg_solver_stats()
        N.check(N.lib().edg_solve_plain(self._h, C.byref(opts), eigs.ctypes.data, cap, C.byref(n_out),
                                        evecs.ctypes.data if nvec else None, nvec, C.byref(st)))
        stats = {f: getattr(st, f) for f, _ in N.edg_solver_stats._fields_}
        return eigs[: n_out.value], evecs, stats

    def solve_mixed(self, n_ev: int = 6, iterations: int = 300, reorth_every: int = 1, seed: int = 1,
                    want_vectors: bool = False, fp64_vectors: bool = False):
        """Lowest eigenvalues with FP32 Krylov vectors (edg_solve_mixed); with
        fp64_vectors the same algorithm in FP64 throughout.  reorth_every: k > 0
        full reorthogonalisation every k steps, -1 partial (where Simon's
        estimates call for it), 0 local only.
        Returns dict(eigs, ritz, residuals, evecs, stats)."""
        k = min(n_ev, 32)
        eigs = np.empty(k, np.float64)
        ritz = np.empty(k, np.float64)
        res = np.empty(k, np.float64)
        evecs = np.empty((k, self.n_p), np.complex128) if want_vectors else None
        opts = N.edg_mixed_opts(int(n_ev), int(iterations), int(reorth_every), int(seed), int(bool(want_vectors)),
                                int(bool(fp64_vectors)))
        n_out = C.c_int64()
        st = N.edg_mixed_stats()
        N.check(N.lib().edg_solve_mixed(self._h, C.byref(opts), eigs.ctypes.data, ritz.ctypes.data, res.ctypes.data,
                                        C.byref(n_out), evecs.ctypes.data if want_vectors else None, C.byref(st)))
        n = n_out.value
        return {"eigs": eigs[:n], "ritz": ritz[:n], "residuals": res[:n],
                "evecs": evecs[:n] if want_vectors else None,
                "stats": {f: getattr(st, f) for f, _ in N.edg_mixed_stats._fields_}}

    def hv_block(self, v, w, stream=None) -> None:
        """W = H V for torch tensors of shape (n_p, 2) or (n_p, 4) (the vectors
        interleaved by row), on the device (edg_hv_block)."""
        nv = int(v.shape[1])
        code = N.EDG_C128 if v.dtype == __import__("torch").complex128 else N.EDG_C64
        st = stream.cuda_stream if stream is not None else 0
        N.check(N.lib().edg_hv_block(self._h, C.c_void_p(v.data_ptr()), C.c_void_p(w.data_ptr()), nv, code,
                                     C.c_void_p(st)))

    def count_offdiag(self) -> int:
        n = C.c_int64()
        N.check(N.lib().edg_count_offdiag(self._h, C.byref(n)))
        return int(n.value)

    def algorithmic_bytes(self, elem_bytes: int, nnz_off: Optional[int] = None) -> int:
        """Bytes one H*v must move at minimum.  Matrix-free: per row the
        representative (8), the stabiliser byte (1), v_i and w_i; per
        off-diagonal target one v_j.  Stored rows: see the comment below."""
        if nnz_off is None:
            nnz_off = self.count_offdiag()
        S = elem_bytes
        if self.info.get("n_targets", 0):
            # stored rows: v_i, stabiliser byte, w_i; per nonzero its entry
            # (4 bytes packed, 6 split) and one u_j; row offsets and diagonal;
            # the u pass
            nnz = self.info["n_targets"]
            entry = self.info.get("entry_bytes") or 6
            return (self.n_p * (2 * S + 1) + nnz * (S + entry) + 8 * (self.n_p + 1) + 8 * self.n_p
                    + self.n_p * (2 * S + 1))
        return self.n_p * (8 + 1 + 2 * S) + nnz_off * S

    def algorithmic_bytes_block(self, elem_bytes: int, nnz_off: Optional[int], nv: int) -> int:
        """Bytes one block H*v on nv vectors must move (stored rows): the
        entries, row offsets and diagonal once; per vector v_i, w_i, one u_j
        per nonzero and the u pass; the stabiliser byte twice (u pass, row)."""
        S = elem_bytes
        nnz = self.info.get("n_targets", 0)
        entry = self.info.get("entry_bytes") or 6
        return (nnz * entry + 8 * (self.n_p + 1) + 8 * self.n_p + 2 * self.n_p
                + nv * (self.n_p * 2 * S + nnz * S + self.n_p * 2 * S))

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().edg_sector_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fill_random(t, seed: int, stream=None) -> None:
    """Fill a complex CUDA tensor with the splitmix64 test vector for `seed`."""
    import torch

    code = N.EDG_C128 if t.dtype == torch.complex128 else N.EDG_C64
    st = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
    N.check(N.lib().edg_fill_random(C.c_void_p(t.data_ptr()), t.numel(), code, int(seed), C.c_void_p(st)))
