"""The allocation-free chemistry entry point, for callers that cannot call
cudaMalloc (a device-memory pool owned by another framework, or a serving loop
that must not allocate once running).  It is called through the C ABI twice in
a row -- the second call finds the previous call's contents in the shared
static scratch -- and each result must equal pdr_chem_solve_batched's on the
same inputs within the chemistry tolerance (1e-4 relative, abundances above
1e-12).  This file is collected last so that a failure here stops a -x run
only after every other test has run."""
import ctypes as C
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("oracle", "3d-pdr_gb300"):
    sys.path.insert(0, os.path.join(ROOT, sub))

import oracle as O  # noqa: E402
import pdrgpu as G  # noqa: E402
import workloads as W  # noqa: E402

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _vp(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_noalloc_entry_point_matches_batched(precision):
    import torch
    assert torch.cuda.is_available()
    dev = torch.device("cuda:0")
    w = W.chemistry("C1")
    onet = O.Network("reduced")
    rates, st = onet.rates(O.phys(w.zeta, w.omega, w.grain_radius, w.metallicity, w.g2d, w.v_turb_kms),
                           w.T, w.Td, w.rad_surface, w.AV, w.column5)
    assert st == 0
    ab0 = np.tile(W.initial_abundances(onet.species, s_plus=False), (w.ncell, 1))
    net = G.Network("reduced")
    rate = torch.as_tensor(rates, device=dev)
    dens = torch.as_tensor(w.n_H, device=dev)
    opts = G.chem_opts(precision)
    stream = torch.cuda.current_stream()
    ref = torch.as_tensor(ab0, device=dev).clone()
    st_ref = torch.empty(w.ncell, dtype=torch.int32, device=dev)
    G.check(G.lib().pdr_chem_solve_batched(net.handle, w.ncell, _vp(ref), _vp(rate), _vp(dens), None,
                                           C.byref(opts), _vp(st_ref), None, C.c_void_p(stream.cuda_stream)),
            "pdr_chem_solve_batched")
    torch.cuda.synchronize()
    ref = ref.cpu().numpy()
    lib = G.lib()
    lib.pdr_chem_solve_batched_noalloc.argtypes = [C.c_void_p, C.c_int] + [C.c_void_p] * 4 + \
        [C.POINTER(G.ChemOpts), C.c_void_p, C.c_void_p, C.c_void_p]
    for call in range(2):
        ab = torch.as_tensor(ab0, device=dev).clone()
        status = torch.full((w.ncell,), 99, dtype=torch.int32, device=dev)
        rc = lib.pdr_chem_solve_batched_noalloc(net.handle, w.ncell, _vp(ab), _vp(rate), _vp(dens), None,
                                                C.byref(opts), _vp(status), None, C.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.pdr_last_error()
        torch.cuda.synchronize()
        got = ab.cpu().numpy()
        assert (status.cpu().numpy() == 0).all(), call
        mask = np.abs(ref[:, :-1]) > 1e-12
        err = (np.abs(got[:, :-1] - ref[:, :-1])[mask] / np.abs(ref[:, :-1])[mask]).max()
        assert err < TOL, (call, err)
        assert np.abs(got[:, -1] - ref[:, -1]).max() <= TOL * np.abs(ref[:, -1]).max()


def test_noalloc_rejects_more_cells_than_its_scratch():
    import torch
    net = G.Network("reduced")
    lib = G.lib()
    lib.pdr_chem_solve_batched_noalloc.argtypes = [C.c_void_p, C.c_int] + [C.c_void_p] * 4 + \
        [C.POINTER(G.ChemOpts), C.c_void_p, C.c_void_p, C.c_void_p]
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda:0")
    st = torch.zeros(8, dtype=torch.int32, device="cuda:0")
    rc = lib.pdr_chem_solve_batched_noalloc(net.handle, 262145, _vp(dummy), _vp(dummy), _vp(dummy), None,
                                            C.byref(G.chem_opts("mixed")), _vp(st), None, None)
    assert rc == -1001
    assert b"262144" in lib.pdr_last_error()


def test_noalloc_takes_the_batched_entry_points_options():
    """The same option checks as pdr_chem_solve_batched (an integrator outside
    0..2 is refused by both), and the same SM limit: with max_sms set, both
    give the same result bit for bit."""
    import torch
    dev = torch.device("cuda:0")
    net = G.Network("reduced")
    lib = G.lib()
    lib.pdr_chem_solve_batched_noalloc.argtypes = [C.c_void_p, C.c_int] + [C.c_void_p] * 4 + \
        [C.POINTER(G.ChemOpts), C.c_void_p, C.c_void_p, C.c_void_p]
    w = W.chemistry("C1", ncell=16)
    onet = O.Network("reduced")
    rates, _ = onet.rates(O.phys(w.zeta, w.omega, w.grain_radius, w.metallicity, w.g2d, w.v_turb_kms),
                          w.T, w.Td, w.rad_surface, w.AV, w.column5)
    ab0 = np.tile(W.initial_abundances(onet.species, s_plus=False), (w.ncell, 1))
    rate = torch.as_tensor(rates, device=dev)
    dens = torch.as_tensor(w.n_H, device=dev)
    st = torch.zeros(w.ncell, dtype=torch.int32, device=dev)
    bad = G.chem_opts("mixed")
    bad.integrator = 7
    ab = torch.as_tensor(ab0, device=dev).clone()
    for fn in (lib.pdr_chem_solve_batched, lib.pdr_chem_solve_batched_noalloc):
        assert fn(net.handle, w.ncell, _vp(ab), _vp(rate), _vp(dens), None, C.byref(bad), _vp(st), None,
                  None) == -1001
    opts = G.chem_opts("mixed")
    opts.max_sms = 8
    out = []
    for fn in (lib.pdr_chem_solve_batched, lib.pdr_chem_solve_batched_noalloc):
        ab = torch.as_tensor(ab0, device=dev).clone()
        rc = fn(net.handle, w.ncell, _vp(ab), _vp(rate), _vp(dens), None, C.byref(opts), _vp(st), None,
                C.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert rc == 0, lib.pdr_last_error()
        torch.cuda.synchronize()
        assert (st.cpu().numpy() == 0).all()
        out.append(ab.cpu().numpy())
    assert np.array_equal(out[0], out[1])
