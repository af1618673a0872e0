"""The ctypes mirrors of the C ABI match the header (CPU, gcc): every structure field's offset and each
structure's size as a C compiler lays them out from include/self_gpu.h, and the option and status constants.
Catches a field or a value changed on one side only."""
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


def _header_defines():
    import re
    vals = {}
    for line in open(os.path.join(ROOT, "include", "self_gpu.h")):
        m = re.match(r"#define\s+(SELF_\w+)\s+\(?(-?\d+)\)?", line)
        if m:
            vals[m.group(1)] = int(m.group(2))
    return vals


def test_python_constants_match_the_header():
    """The Python layer's option and status constants equal the header's #defines."""
    from self_gb300 import _native as nat
    from self_gb300 import cgsem, serving
    H = _header_defines()
    pairs = {
        "SELF_OK": nat.OK, "SELF_NO_NORMAL_FLOW": nat.NO_NORMAL_FLOW, "SELF_INFLOW_ONE": nat.INFLOW_ONE,
        "SELF_INFLOW_TWO": nat.INFLOW_TWO, "SELF_DIRICHLET": nat.DIRICHLET, "SELF_GAUSS": nat.GAUSS,
        "SELF_GAUSS_LOBATTO": nat.GAUSS_LOBATTO, "SELF_DG": nat.DG, "SELF_CG": nat.CG,
        "SELF_MODEL_SW_CONSERVATIVE": nat.MODEL_SW_CONSERVATIVE, "SELF_MODEL_ADVECTION": nat.MODEL_ADVECTION,
        "SELF_MODEL_SW_LINEAR": nat.MODEL_SW_LINEAR, "SELF_MODEL_SW_SKEW": nat.MODEL_SW_SKEW,
        "SELF_PREC_FP64": nat.PREC_FP64, "SELF_PREC_FP32": nat.PREC_FP32, "SELF_PREC_FP64_EXACT": nat.PREC_FP64_EXACT,
        "SELF_SOLVE_CG": cgsem.SOLVE_CG, "SELF_SOLVE_PCG_JACOBI": cgsem.SOLVE_PCG_JACOBI,
        "SELF_SOLVE_GMRES": cgsem.SOLVE_GMRES, "SELF_SOLVE_PGMRES_JACOBI": cgsem.SOLVE_PGMRES_JACOBI,
        "SELF_SOLVE_PCG_LINEAR": cgsem.SOLVE_PCG_LINEAR,
        "SELF_LAYOUT_COMPACT": cgsem.INNER_LAYOUTS["compact"], "SELF_LAYOUT_LOCAL": cgsem.INNER_LAYOUTS["local"],
        "SELF_PC_NODES_POSITION": cgsem.PC_NODES["position"],
        "SELF_PC_NODES_CONNECTIVITY": cgsem.PC_NODES["connectivity"],
        "SELF_F32_LOCAL": cgsem.F32_FORMS["local"], "SELF_F32_TENSOR_CORES": cgsem.F32_FORMS["tensor_cores"],
        "SELF_F32_COMPACT": cgsem.F32_FORMS["compact"],
        "SELF_SERVE_QUEUED": serving.QUEUED, "SELF_SERVE_RUNNING": serving.RUNNING, "SELF_SERVE_DONE": serving.DONE,
        "SELF_SERVE_CANCELLED": serving.CANCELLED, "SELF_SERVE_FAILED": serving.FAILED,
    }
    for name, value in pairs.items():
        assert H[name] == value, name
