"""A plain C program using only the einspline API (tests/c_api/drop_in.c),
compiled with gcc against include/ and linked with the library, runs on the
GPU: create/set, the CPU entry and the batched CUDA entry agree."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_home():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


@pytest.mark.gpu
def test_c_drop_in(tmp_path, eglib):
    from einspline_gb300 import build
    cuda = _cuda_home()
    exe = tmp_path / "drop_in"
    libdir = os.path.dirname(build.LIB)
    cmd = ["gcc", "-std=gnu99", "-O2", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(cuda, "include"),
           os.path.join(ROOT, "tests", "c_api", "drop_in.c"), "-o", str(exe), "-L", libdir, "-leinspline_gb300",
           f"-Wl,-rpath,{libdir}", "-L", os.path.join(cuda, "lib64"), "-lcudart", "-lm"]
    subprocess.run(cmd, check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    print(r.stdout, r.stderr)
    assert r.returncode == 0, r.stdout + r.stderr
