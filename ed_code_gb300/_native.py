"""ctypes binding of libedgpu.so (include/edgpu.h).

The library is the product: there is no CPU fallback.  Loading fails loudly
when libedgpu.so has not been built (``python -m ed_code_gb300.build``), and
every call raises :class:`EdgError` with the library's message on failure.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libedgpu.so")

EDG_OK = 0
EDG_ERR = {
    1: "EDG_ERR_INVALID", 2: "EDG_ERR_MOMENTUM", 3: "EDG_ERR_EMPTY", 4: "EDG_ERR_CUDA", 5: "EDG_ERR_NOMEM",
    6: "EDG_ERR_UNSUPPORTED", 7: "EDG_ERR_NOT_CONVERGED", 8: "EDG_ERR_CANCELLED",
}
EDG_C128 = 0
EDG_C64 = 1


class EdgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{EDG_ERR.get(code, code)}: {msg}")
        self.code = code


class edg_bond(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int), ("J", C.c_double), ("re", C.c_double), ("im", C.c_double)]


class edg_triangle(C.Structure):
    _fields_ = [("i", C.c_int), ("j", C.c_int), ("k", C.c_int), ("re", C.c_double), ("im", C.c_double)]


class edg_bowtie(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("x", "y", "z", "p", "q", "r")]


class edg_model(C.Structure):
    _fields_ = [
        ("n_sites", C.c_int), ("T1", C.POINTER(C.c_int)), ("T2", C.POINTER(C.c_int)), ("lambda_", C.c_double),
        ("bonds", C.POINTER(edg_bond)), ("n_bonds", C.c_int), ("Ch", C.c_double),
        ("triangles", C.POINTER(edg_triangle)), ("n_triangles", C.c_int), ("ChCh", C.c_double),
        ("bowties", C.POINTER(edg_bowtie)), ("n_bowties", C.c_int), ("T3", C.POINTER(C.c_int)),
    ]


class edg_sector_info(C.Structure):
    _fields_ = [
        ("n_sites", C.c_int), ("n_ones", C.c_int), ("L1", C.c_int), ("L2", C.c_int), ("kx", C.c_int),
        ("ky", C.c_int), ("torus", C.c_int), ("n_groups", C.c_int), ("n_p", C.c_int64), ("n_configs", C.c_int64),
        ("device_bytes", C.c_int64), ("n_targets", C.c_int64), ("lanes_per_row", C.c_int),
        ("cache_policy", C.c_int), ("L3", C.c_int), ("kz", C.c_int),
        ("entry_bytes", C.c_int), ("n_values", C.c_int), ("ctas_per_sm", C.c_int), ("pipelined", C.c_int),
    ]


class edg_batch_opts(C.Structure):
    _fields_ = [("tile_rows", C.c_int), ("lanes_per_row", C.c_int), ("check_every", C.c_int), ("reorth", C.c_int)]


class edg_batch_request(C.Structure):
    _fields_ = [("n_ev", C.c_int), ("max_iterations", C.c_int), ("tol", C.c_double), ("seed", C.c_uint64),
                ("tag", C.c_int64)]


class edg_batch_result(C.Structure):
    _fields_ = [("tag", C.c_int64), ("status", C.c_int), ("n_found", C.c_int), ("iterations", C.c_int),
                ("converged", C.c_int), ("reorth_steps", C.c_int), ("reserved", C.c_int),
                ("eigs", C.c_double * 32), ("ritz", C.c_double * 32),
                ("residuals", C.c_double * 32)]


LOG_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_char_p)


class edg_solver_opts(C.Structure):
    _fields_ = [
        ("n_ev", C.c_int), ("iterations", C.c_int), ("ncycles", C.c_int), ("tol", C.c_double),
        ("seed", C.c_uint64), ("dense_threshold", C.c_int64), ("log_fn", LOG_FN), ("log_ctx", C.c_void_p),
    ]


class edg_solver_stats(C.Structure):
    _fields_ = [
        ("path", C.c_int), ("hv_calls", C.c_int64), ("hv_seconds", C.c_double), ("ortho_seconds", C.c_double),
        ("total_seconds", C.c_double),
    ]


class edg_mixed_opts(C.Structure):
    _fields_ = [("n_ev", C.c_int), ("iterations", C.c_int), ("reorth_every", C.c_int), ("seed", C.c_uint64),
                ("want_vectors", C.c_int), ("fp64_vectors", C.c_int)]


class edg_mixed_stats(C.Structure):
    _fields_ = [("hv_calls", C.c_int64), ("hv_seconds", C.c_double), ("total_seconds", C.c_double),
                ("passes", C.c_int), ("stored_vectors", C.c_int), ("reorth_steps", C.c_int)]


# name -> (restype, argtypes); every exported symbol of include/edgpu.h
SIGNATURES = {
    "edg_last_error": (C.c_char_p, []),
    "edg_abi_version": (C.c_int, []),
    "edg_sector_create": (C.c_int, [C.POINTER(edg_model), C.c_int, C.c_int, C.c_int, C.POINTER(C.c_void_p)]),
    "edg_sector_create3": (C.c_int, [C.POINTER(edg_model), C.c_int, C.c_int, C.c_int, C.c_int,
                                     C.POINTER(C.c_void_p)]),
    "edg_sector_destroy": (C.c_int, [C.c_void_p]),
    "edg_sector_get_info": (C.c_int, [C.c_void_p, C.POINTER(edg_sector_info)]),
    "edg_sector_copy_basis": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "edg_sector_copy_lin_tables": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int64)]),
    "edg_sector_copy_config_tables": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]),
    "edg_hv": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "edg_hv_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "edg_sector_set_rows": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]),
    "edg_batch_create": (C.c_int, [C.POINTER(edg_batch_opts), C.POINTER(C.c_void_p)]),
    "edg_batch_destroy": (C.c_int, [C.c_void_p]),
    "edg_batch_footprint": (C.c_int, [C.c_void_p, C.POINTER(edg_batch_request), C.POINTER(C.c_int64)]),
    "edg_batch_add": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(edg_batch_request)]),
    "edg_batch_step": (C.c_int, [C.c_void_p, C.c_int]),
    "edg_batch_poll": (C.c_int, [C.c_void_p, C.POINTER(edg_batch_result), C.c_int, C.POINTER(C.c_int)]),
    "edg_batch_timers": (C.c_int, [C.c_void_p, C.c_void_p]),
    "edg_batch_cancel": (C.c_int, [C.c_void_p, C.c_int64]),
    "edg_batch_tune": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_void_p]),
    "edg_batch_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "edg_hv_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "edg_hv_block": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
    "edg_count_offdiag": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "edg_fill_random": (C.c_int, [C.c_void_p, C.c_int64, C.c_int, C.c_uint64, C.c_void_p]),
    "edg_tridiag_lowest": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                     C.POINTER(C.c_int)]),
    "edg_sector_build_targets": (C.c_int, [C.c_void_p, C.c_int64]),
    "edg_sector_free_targets": (C.c_int, [C.c_void_p]),
    "edg_sector_tune": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.c_void_p]),
    "edg_solve_plain": (C.c_int, [C.c_void_p, C.POINTER(edg_solver_opts), C.c_void_p, C.c_int64,
                                  C.POINTER(C.c_int64), C.c_void_p, C.c_int64, C.POINTER(edg_solver_stats)]),
    "edg_solve_mixed": (C.c_int, [C.c_void_p, C.POINTER(edg_mixed_opts), C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.POINTER(C.c_int64), C.c_void_p, C.POINTER(edg_mixed_stats)]),
}

_lib: Optional[C.CDLL] = None


def lib() -> C.CDLL:
    """Load libedgpu.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with `python -m ed_code_gb300.build`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            if not hasattr(L, name):
                continue
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != EDG_OK:
        msg = lib().edg_last_error()
        raise EdgError(rc, msg.decode() if msg else "")
