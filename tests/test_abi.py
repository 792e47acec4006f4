"""The C-ABI library builds, loads and exports what include/edgpu.h declares (no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(edg_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def libedgpu():
    from ed_code_gb300 import build

    build.build()
    return ctypes.CDLL(build.LIB)


def test_header_declares_entry_points():
    names = declared_functions("edgpu.h")
    for required in ("edg_sector_create", "edg_hv", "edg_hv_host", "edg_sector_destroy", "edg_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol(libedgpu):
    missing = [n for n in declared_functions("edgpu.h") if not hasattr(libedgpu, n)]
    assert not missing, missing


def test_python_binding_covers_every_symbol():
    from ed_code_gb300 import _native

    missing = [n for n in declared_functions("edgpu.h") if n not in _native.SIGNATURES]
    assert not missing, missing


def test_abi_version_and_error_string(libedgpu):
    libedgpu.edg_abi_version.restype = ctypes.c_int
    assert libedgpu.edg_abi_version() == 8
    libedgpu.edg_last_error.restype = ctypes.c_char_p
    assert isinstance(libedgpu.edg_last_error(), bytes)


def test_invalid_arguments_fail_without_touching_the_gpu(libedgpu):
    """Argument checks run before any CUDA call: a NULL model is EDG_ERR_INVALID."""
    out = ctypes.c_void_p()
    libedgpu.edg_sector_create.restype = ctypes.c_int
    rc = libedgpu.edg_sector_create(None, 8, 0, 0, ctypes.byref(out))
    assert rc == 1
    assert out.value is None
