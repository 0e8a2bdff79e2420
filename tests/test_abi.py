"""The C-ABI library without a GPU: it loads, exports every entry point the
headers in include/ declare, its structs have the layout ctypes mirrors, the
host copy of the factored line solve matches the oracle bit for bit, and
argument errors come back as status codes instead of aborts."""
import ctypes as C
import glob
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(INCLUDE, "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        txt = re.sub(r"//[^\n]*", "", txt)
        txt = re.sub(r"#[^\n]*", "", txt)
        for m in re.finditer(r"\b([A-Za-z_]\w*)\s*\(", txt):
            n = m.group(1)
            if n in ("sizeof", "extern", "if", "while", "for", "return"):
                continue
            # declarations only (a type precedes the name)
            pre = txt[:m.start()].rstrip()
            if pre.endswith(("*", "void", "int", "int64_t", "char", ")")) or re.search(r"\w$", pre):
                names.add(n)
    return names


def test_every_declared_symbol_is_exported(eglib):
    from einspline_gb300 import _lib
    decl = declared_functions()
    assert len(decl) >= 50
    missing = [n for n in decl if not hasattr(eglib, n)]
    assert not missing, missing
    # and the Python binding covers all of them
    assert decl <= set(_lib.SIGNATURES), sorted(decl - set(_lib.SIGNATURES))


LAYOUT_C = r"""
#include <stdio.h>
#include <stddef.h>
#include "einspline_gb300.h"
#define F(S, f) printf(#S " " #f " %zu\n", offsetof(S, f));
#define Z(S) printf(#S " sizeof %zu\n", sizeof(S));
int main(void) {
  Z(Ugrid) F(Ugrid, num) F(Ugrid, delta_inv)
  Z(BCtype_s) Z(BCtype_d) Z(BCtype_c) Z(BCtype_z)
  Z(multi_UBspline_3d_s) F(multi_UBspline_3d_s, coefs) F(multi_UBspline_3d_s, x_grid) F(multi_UBspline_3d_s, xBC)
  F(multi_UBspline_3d_s, num_splines) F(multi_UBspline_3d_s, gb300)
  Z(multi_UBspline_3d_d) F(multi_UBspline_3d_d, zBC) F(multi_UBspline_3d_d, num_splines) F(multi_UBspline_3d_d, gb300)
  Z(multi_UBspline_3d_c) F(multi_UBspline_3d_c, lapl3) F(multi_UBspline_3d_c, gb300)
  Z(multi_UBspline_3d_z) F(multi_UBspline_3d_z, zBC) F(multi_UBspline_3d_z, lapl3) F(multi_UBspline_3d_z, gb300)
  Z(multi_UBspline_3d_s_cuda) F(multi_UBspline_3d_s_cuda, stride) F(multi_UBspline_3d_s_cuda, gridInv)
  F(multi_UBspline_3d_s_cuda, dim) F(multi_UBspline_3d_s_cuda, num_splines) F(multi_UBspline_3d_s_cuda, gb300)
  Z(multi_UBspline_3d_d_cuda) F(multi_UBspline_3d_d_cuda, gridInv) F(multi_UBspline_3d_d_cuda, dim)
  F(multi_UBspline_3d_d_cuda, num_splines) F(multi_UBspline_3d_d_cuda, gb300)
  Z(multi_UBspline_3d_z_cuda) F(multi_UBspline_3d_z_cuda, gb300)
  Z(einspline_gb300_eval_opts) F(einspline_gb300_eval_opts, vstride) F(einspline_gb300_eval_opts, hstride)
  Z(einspline_gb300_table_info) F(einspline_gb300_table_info, x_stride) F(einspline_gb300_table_info, scale)
  return 0;
}
"""


def _cuda_include():
    for d in ("/usr/local/cuda/include", os.path.join(os.path.dirname(shutil.which("nvcc") or "/x/x"), "..", "include")):
        if os.path.exists(os.path.join(d, "vector_types.h")):
            return d
    return None


@pytest.mark.skipif(shutil.which("gcc") is None or _cuda_include() is None, reason="needs gcc and CUDA headers")
def test_struct_layouts_match_ctypes(tmp_path):
    from einspline_gb300 import _lib as L
    src = tmp_path / "layout.c"
    src.write_text(LAYOUT_C)
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=gnu99", "-I", INCLUDE, "-I", _cuda_include(), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    py = {"Ugrid": L.Ugrid, "BCtype_s": L.BCtype_s, "BCtype_d": L.BCtype_d, "BCtype_c": L.BCtype_c,
          "BCtype_z": L.BCtype_z, "einspline_gb300_eval_opts": L.EvalOpts,
          "einspline_gb300_table_info": L.TableInfo}
    for k in "sdcz":
        py[f"multi_UBspline_3d_{k}"] = L.HOST_STRUCTS[k]
        py[f"multi_UBspline_3d_{k}_cuda"] = L.CUDA_STRUCTS[k]
    n = 0
    for line in out:
        if not line:
            continue
        s, f, v = line.split()
        v = int(v)
        S = py[s]
        got = C.sizeof(S) if f == "sizeof" else getattr(S, f).offset
        assert got == v, (s, f, got, v)
        n += 1
    assert n > 30


def test_host_line_solve_matches_oracle(eglib, orc):
    rng = np.random.default_rng(0)
    for M in (4, 5, 8, 17, 64, 129):
        for lc, rc in [(0, 0), (5, 5), (1, 1), (2, 2), (3, 4), (4, 3), (1, 2), (2, 1)]:
            dinv, lv, rv = 1.3 + M * 0.01, 0.3, -0.8
            data = rng.uniform(-1, 1, M)
            N = M + 3 if lc in (0, 5) else M + 2
            lv_e = 0.0 if lc in (3, 4) else lv
            rv_e = 0.0 if rc in (3, 4) else rv
            out = np.zeros(N)
            eglib.einspline_gb300_solve_line_host(M, lc, rc, dinv, lv_e, rv_e, data.ctypes.data, out.ctypes.data)
            ax = orc.OrcAxis()
            orc.lib().orc_axis_init(C.byref(ax), 0.0, 1.0, M, lc, rc, lv, 0.0, rv, 0.0)
            ax.delta_inv = dinv
            ref = np.zeros(N)
            orc.lib().orc_find_coefs_1d_d(C.byref(ax), 0, data.ctypes.data, 1, ref.ctypes.data, 1)
            assert np.array_equal(out, ref), (M, lc, rc)


def test_argument_errors_are_status_codes(eglib):
    from einspline_gb300 import _lib as L
    g = L.Ugrid(0.0, 1.0, 8, 0.0, 0.0)
    bc = L.BCtype_s(0, 0, 0.0, 0.0)
    p = eglib.create_multi_UBspline_3d_s(g, g, g, bc, bc, bc, 0)
    assert not p
    assert eglib.einspline_gb300_last_error() == 1
    assert b"num_splines" in eglib.einspline_gb300_last_error_message()
    eglib.einspline_gb300_clear_error()
    tiny = L.Ugrid(0.0, 1.0, 2, 0.0, 0.0)
    assert not eglib.create_multi_UBspline_3d_s(tiny, g, g, bc, bc, bc, 4)
    assert eglib.einspline_gb300_last_error() == 1
    bad = L.BCtype_s(4, 0, 0.0, 0.0)  # NATURAL on the left with PERIODIC on the right
    assert not eglib.create_multi_UBspline_3d_s(g, g, g, bad, bc, bc, 4)
    assert eglib.einspline_gb300_last_error() == 1
    o = L.EvalOpts(1, 1, 5, 0, 0, 0, 0, 0)
    assert eglib.einspline_gb300_eval_3d(None, C.byref(o), 1, None, None, None, None, None) == 1
    eglib.einspline_gb300_clear_error()
    assert eglib.einspline_gb300_last_error() == 0
