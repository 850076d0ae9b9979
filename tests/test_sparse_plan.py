"""The block integrator's sparse bordered Newton matrix plan, checked on the
host: structure (level order, closed fill, every Jacobian entry located) and
numbers (the device's elimination order and pivoting, in FP64, against a dense
solve of the chain-rule system) on all three networks.  The program includes
the library's own pdr_net.cpp and is built with g++ here."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def cuda_home():
    for d in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return d
    return None


def test_sparse_plan(tmp_path):
    cuda = cuda_home()
    if shutil.which("g++") is None or cuda is None:
        pytest.skip("g++ or the CUDA headers are missing")
    exe = str(tmp_path / "sparse_plan_check")
    src = os.path.join(ROOT, "tests", "sparse_plan", "sparse_plan_check.cpp")
    libdir = os.path.join(cuda, "lib64") if os.path.exists(os.path.join(cuda, "lib64")) else os.path.join(cuda, "lib")
    r = subprocess.run(["g++", "-O2", "-std=c++17", f"-I{cuda}/include", f"-I{ROOT}/include", "-o", exe, src,
                        f"-L{libdir}", "-lcudart", f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe, os.path.join(ROOT, "data"), "reduced", "mynetwork", "full"], capture_output=True,
                       text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "full: N 215" in r.stdout
