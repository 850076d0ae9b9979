"""The chemistry tables of both integrators, checked on the host: pdr_net.cpp
builds them with its device allocations redirected to host memory, and the
table-driven RHS (pair operands, merged rate constants, balanced chunks and
their partial sums) and term-parallel Jacobian assembly, replayed as the
kernels run them, agree with a direct evaluation from the stoichiometry to
1e-14 of each species' term scale on seeded states, for all three networks."""
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


def test_network_tables_replay_the_stoichiometry(tmp_path):
    cuda = cuda_home()
    if shutil.which("g++") is None or cuda is None:
        pytest.skip("g++ or the CUDA headers are missing")
    exe = str(tmp_path / "table_check")
    src = os.path.join(ROOT, "tests", "table_check", "table_check.cpp")
    libdir = os.path.join(cuda, "lib64") if os.path.exists(os.path.join(cuda, "lib64")) else os.path.join(cuda, "lib")
    r = subprocess.run(["g++", "-O2", "-std=c++17", f"-I{cuda}/include", f"-I{ROOT}/include", "-o", exe, src,
                        f"-L{libdir}", "-lcudart", f"-Wl,-rpath,{libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe, os.path.join(ROOT, "data"), "reduced", "mynetwork", "full"], capture_output=True,
                       text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count(": ok") == 3
