"""The ctypes mirrors of the C ABI's structures match the header (CPU, gcc): every field's offset and each struct's
size, as a C compiler lays them out from include/self_gpu.h.  Catches a field added to one side only."""
import ctypes
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _mirrors():
    from self_gb300 import _native as nat
    from self_gb300.cgsem import CG2DDesc, SolveOpts, SolveReport
    from self_gb300.serving import ServeInfo, ServeOpts, ServeStats
    return {"self_dg2d_desc": nat.DG2DDesc, "self_cg2d_desc": CG2DDesc, "self_solve_opts": SolveOpts,
            "self_solve_report": SolveReport, "self_serve_opts": ServeOpts, "self_serve_info": ServeInfo,
            "self_serve_statistics": ServeStats}


# Python names that differ from the C field names (Python keywords)
_ALIAS = {("self_cg2d_desc", "lam"): "lambda"}


def _c_layout(mirrors):
    """sizeof and offsetof of every mirrored field, from a C program compiled against the header."""
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "self_gpu.h"', "int main(void) {"]
    for cname, cls in mirrors.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            cf = _ALIAS.get((cname, fname), fname)
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {cf}));')
    lines += ["  return 0;", "}"]
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "layout.c"), os.path.join(d, "layout")
        with open(src, "w") as f:
            f.write("\n".join(lines) + "\n")
        subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True,
                       capture_output=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    layout = {}
    for line in out.splitlines():
        cname, key, val = line.split()
        layout[(cname, key)] = int(val)
    return layout


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs gcc")
def test_ctypes_mirrors_match_the_header():
    mirrors = _mirrors()
    layout = _c_layout(mirrors)
    for cname, cls in mirrors.items():
        assert layout[(cname, "size")] == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert layout[(cname, fname)] == getattr(cls, fname).offset, (cname, fname)
