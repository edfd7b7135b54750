"""The ctypes mirrors of the C ABI's structs (molds_gb300/__init__.py) have
the C layout: every field at the offset gcc gives it in include/nddo_gpu.h,
and the same total size (arrays of results are filled element by element by
the library, so a size mismatch would shift every element after the first)."""
import ctypes
import os
import subprocess

import pytest

import molds_gb300 as M

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

STRUCTS = {"nddo_scf_params": M.ScfParamsC, "nddo_scf_result": M.ScfResultC, "nddo_serve_result": M.ServeResultC}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    d = tmp_path_factory.mktemp("abi")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "nddo_gpu.h"', "int main(void) {"]
    for cname, py in STRUCTS.items():
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'  printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    src = d / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = str(d / "layout")
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", exe], check=True)
    out = {}
    for line in subprocess.run([exe], check=True, capture_output=True, text=True).stdout.splitlines():
        s, f, v = line.split()
        out[(s, f)] = int(v)
    return out


@pytest.mark.parametrize("cname", list(STRUCTS))
def test_ctypes_mirror_matches_c(c_layout, cname):
    py = STRUCTS[cname]
    assert ctypes.sizeof(py) == c_layout[(cname, "sizeof")]
    for f, _ in py._fields_:
        assert getattr(py, f).offset == c_layout[(cname, f)], f
