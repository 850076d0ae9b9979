"""Build lib3dpdr_gb300.so (sm_103a) and its test companions.

    python 3d-pdr_gb300/build.py            # library + oracle (+ reference objects when present)

The library is compiled in-tree with nvcc, one translation unit per process,
for exactly one target: -gencode arch=compute_103a,code=sm_103a.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "lib3dpdr_gb300.so")
SOURCES = ["pdr_net.cpp", "coolant.cpp", "capi.cu", "chem_warp.cu", "chem_cta.cu", "chem_noalloc.cu", "rates.cu", "levpop.cu", "heating.cu", "probe.cu", "serve.cpp", "rays.cu", "thermal.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "-Xcompiler", "-ffp-contract=off", f"-I{os.path.join(ROOT, 'include')}"]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(src):
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build_library(verbose=False):
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", LIB)
    return LIB


def build_test_driver():
    """C program that plays the Fortran caller of calculate_abundances_."""
    src = os.path.join(ROOT, "tests", "fortran_caller", "fortran_caller.c")
    exe = os.path.join(ROOT, "tests", "fortran_caller", "fortran_caller")
    cmd = ["gcc", "-O2", "-o", exe, src, f"-L{PKG}", "-l3dpdr_gb300", f"-Wl,-rpath,{PKG}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"test driver build failed:\n{r.stderr}")
    return exe


def reference_dir():
    """The 3D-PDR source tree, for the reference's own network code: the
    PDR_REFERENCE environment variable, else the tree mounted beside this
    build (absent on machines that only run the prebuilt library)."""
    d = os.environ.get("PDR_REFERENCE") or "/root/reference"
    return d if os.path.exists(os.path.join(d, "odes_reduced.c")) else None


def build_oracle(ref_dir=None):
    """liboracle.so (-O2) and liboracle_O0.so (-O0, the optimisation level the
    reference compiles its C with, makefile:139-145), plus the reference's
    generated network code (oracle/_ref) when its sources are present."""
    oracle = os.path.join(ROOT, "oracle")
    r = subprocess.run(["make", "-s", "-C", oracle, "all"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    ref_dir = ref_dir or reference_dir()
    if ref_dir:
        r = subprocess.run(["make", "-s", "-C", oracle, "ref", f"REF={ref_dir}"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference objects build failed:\n{r.stderr}")


if __name__ == "__main__":
    build_library(verbose=True)
    build_oracle()
    if os.path.exists(os.path.join(ROOT, "tests", "fortran_caller", "fortran_caller.c")):
        build_test_driver()
    sys.exit(0)
