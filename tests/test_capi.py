"""C-ABI checks that need no GPU: the library loads, exports exactly what
include/pdrgpu.h declares, and refuses to compute without a device."""
import ctypes as C
import os
import re
import subprocess

import pytest

import pdrgpu as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "pdrgpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b([a-z_][a-z0-9_]*)\s*\(", txt)) -
                  {"if", "for", "while", "sizeof", "return"})


def exported_symbols():
    out = subprocess.run(["nm", "-D", "--defined-only", G.LIB_PATH], capture_output=True, text=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if " T " in ln}


def test_library_exports_every_declared_symbol():
    decl = declared_symbols()
    assert "calculate_abundances_" in decl and "pdr_chem_solve_batched" in decl
    exp = exported_symbols()
    missing = [s for s in decl if s not in exp]
    assert not missing, missing


def test_library_loads_and_binds_fortran_globals_weakly():
    lib = G.lib()
    for s in declared_symbols():
        assert hasattr(lib, s)
    out = subprocess.run(["nm", "-D", G.LIB_PATH], capture_output=True, text=True).stdout
    for g in ("chemistry_module_mp_relative_abundance_tolerance_", "maincode_module_mp_end_time_",
              "global_module_mp_nelect_"):
        assert re.search(r"\s[wVv]\s+" + g, out), g


def test_legacy_symbol_without_fortran_globals_fails_loudly():
    lib = G.lib()
    d = (C.c_double * 4)()
    n = C.c_int(1)
    rc = lib.calculate_abundances_(d, d, d, d, C.byref(n), C.byref(C.c_int(33)), C.byref(C.c_int(329)))
    assert rc != 0
    assert b"Fortran module variables" in lib.pdr_last_error()


def test_compute_without_gpu_fails_instead_of_falling_back():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError):
        G.Network("reduced")
    v = C.c_double()
    assert G.lib().pdr_probe_fma_tflops(64, C.byref(v), None) != 0
