"""Plain C programs using only the public headers (tests/c_api/*.c),
compiled with gcc against include/ and linked with the library.  drop_in.c:
create/set, the CPU entry and the batched CUDA entry agree (the reference's
test_multi_cuda pattern).  drop_in_more.c: the 1D/2D splines, the 1D GPU
entry, vghgh, double-float FP64 evaluation and the determinant ratio.  The
programs compile on any machine (CPU test); they run on the GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


PROGRAMS = ["drop_in", "drop_in_more"]


def _compile(tmp_path, name):
    from einspline_gb300 import build
    cuda = _cuda_home()
    exe = tmp_path / name
    libdir = os.path.dirname(build.LIB)
    cmd = ["gcc", "-std=gnu99", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda, "include"), os.path.join(ROOT, "tests", "c_api", name + ".c"), "-o", str(exe),
           "-L", libdir, "-leinspline_gb300", f"-Wl,-rpath,{libdir}", "-L", os.path.join(cuda, "lib64"),
           "-lcudart", "-lm"]
    subprocess.run(cmd, check=True)
    return exe


@pytest.mark.parametrize("name", PROGRAMS)
def test_c_programs_compile(tmp_path, eglib, name):
    """The headers are valid C and every entry the programs call links."""
    assert _compile(tmp_path, name).exists()


@pytest.mark.gpu
@pytest.mark.parametrize("name", PROGRAMS)
def test_c_drop_in(tmp_path, eglib, name):
    exe = _compile(tmp_path, name)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stdout + r.stderr
