"""The Python bindings' ctypes structures match the C header's layout: size
and every field's offset, as a C compiler lays them out (gcc on
include/edgpu.h, no GPU needed)."""
import ctypes
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STRUCTS = ["edg_bond", "edg_triangle", "edg_bowtie", "edg_model", "edg_sector_info", "edg_solver_opts",
           "edg_solver_stats", "edg_mixed_opts", "edg_mixed_stats", "edg_batch_opts", "edg_batch_request",
           "edg_batch_result"]


def _c_name(field):
    """The C name of a ctypes field (a Python keyword gets a trailing underscore)."""
    import keyword

    return field[:-1] if field.endswith("_") and keyword.iskeyword(field[:-1]) else field


@pytest.fixture(scope="module")
def c_layout():
    """{struct: (sizeof, {field: offsetof})} from a C program built against the header."""
    from ed_code_gb300 import _native as N

    if shutil.which("gcc") is None:
        pytest.skip("gcc not found")
    out_dir = os.path.join(ROOT, "tests", "_build")
    os.makedirs(out_dir, exist_ok=True)
    src = os.path.join(out_dir, "abi_layout.c")
    exe = os.path.join(out_dir, "abi_layout")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "edgpu.h"', "int main(void) {"]
    for s in STRUCTS:
        lines.append(f'  printf("S {s} %zu\\n", sizeof({s}));')
        for f, _ in getattr(N, s)._fields_:
            lines.append(f'  printf("F {s} {f} %zu\\n", offsetof({s}, {_c_name(f)}));')
    lines += ["  return 0;", "}"]
    with open(src, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
    res = {}
    for ln in subprocess.run([exe], check=True, capture_output=True, text=True).stdout.splitlines():
        p = ln.split()
        if p[0] == "S":
            res.setdefault(p[1], [0, {}])[0] = int(p[2])
        else:
            res.setdefault(p[1], [0, {}])[1][p[2]] = int(p[3])
    return res


@pytest.mark.parametrize("name", STRUCTS)
def test_ctypes_struct_matches_header(c_layout, name):
    from ed_code_gb300 import _native as N

    cls = getattr(N, name)
    size, offsets = c_layout[name]
    assert ctypes.sizeof(cls) == size, (name, ctypes.sizeof(cls), size)
    for f, _ in cls._fields_:
        assert getattr(cls, f).offset == offsets[f], (name, f)
