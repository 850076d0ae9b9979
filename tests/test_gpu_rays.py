"""Column densities and the UV field on the GPU (csrc/rays.cu) against the
oracle: columns, A_V and the surface field bit for bit (same operation order,
unfused), the attenuated field within 1e-14 (exp of a different libm)."""
import numpy as np
import pytest

import oracle as O
import pdrgpu as G
import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("field", [0, 1])
def test_uvfield_matches_oracle(cuda, field):
    import torch
    r = W.rays(8, 12)
    gvec = (10.0, 0.0, 0.0) if field == 0 else (3.0, -2.0, -7.0)
    col, av, rad, uv = O.uvfield(r, field=field, G=gvec, metallicity=0.7)
    rays, keep = G.device_rays(r, cuda)
    rho = torch.as_tensor(r["rho"], device=cuda)
    gcol, gav, grad, guv = G.uvfield(rays, rho, field, gvec, r["vectors"], metallicity=0.7)
    torch.cuda.synchronize()
    assert np.array_equal(gcol.cpu().numpy(), col)
    assert np.array_equal(gav.cpu().numpy(), av)
    assert np.array_equal(grad.cpu().numpy(), rad)
    m = uv > 0
    assert np.allclose(guv.cpu().numpy()[m], uv[m], rtol=1e-14, atol=0)


@pytest.mark.parametrize("species", [None, [5, 0, 17, 3, 9]])
def test_columns_match_oracle(cuda, species):
    import torch
    r = W.rays(8, 12, nspec=21)
    ref = O.columns(r, species)
    rays, keep = G.device_rays(r, cuda)
    out = G.column_densities(rays, torch.as_tensor(r["rho"], device=cuda),
                             torch.as_tensor(r["abundance"], device=cuda), species)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), ref)


def test_bad_grid_index_gives_nan_not_a_fault(cuda):
    import torch
    r = W.rays(4, 5, nspec=3)
    r["gridpoint"] = r["gridpoint"].copy()
    ray = 7
    p0 = int(r["offset"][ray])
    if r["epray"][ray] == 0:
        r["epray"] = r["epray"].copy()
        r["epray"][ray] = 1
    r["gridpoint"][p0 + 1] = r["ngrid"] + 5          # outside the grid
    rays, keep = G.device_rays(r, cuda)
    out = G.column_densities(rays, torch.as_tensor(r["rho"], device=cuda),
                             torch.as_tensor(r["abundance"], device=cuda))
    torch.cuda.synchronize()
    o = out.cpu().numpy().reshape(-1, 3)
    assert np.isnan(o[ray]).all()
    assert np.isfinite(np.delete(o, ray, axis=0)).all()


@pytest.mark.parametrize("key", ["CII", "CO"])
def test_optical_depths_match_oracle(cuda, key):
    """Line optical depths along the rays (escape_probability.F90:86-106), bit for bit."""
    import torch
    r = W.rays(6, 10)
    oc = O.Coolant(key)
    rng = np.random.Generator(np.random.PCG64(77))
    dens = r["rho"] * W.COOLANT_X[key]
    T = rng.uniform(10.0, 300.0, r["ngrid"])
    pop = np.array([oc.lte(t, d) for t, d in zip(T, dens)]) * rng.uniform(0.5, 1.5, (r["ngrid"], oc.nlev))
    ref = oc.optical_depths(r, pop, T[:r["ncell"]], 1.0e5)
    rays, keep = G.device_rays(r, cuda)
    out = G.optical_depths(G.Coolant(key), rays, torch.as_tensor(pop, device=cuda),
                           torch.as_tensor(T[:r["ncell"]], device=cuda), 1.0e5)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), ref)


def test_lvg_step_on_device_matches_oracle(cuda):
    """tau from the neighbours' populations, then the level populations, all
    on the device, against the same chain in the oracle (CO, pseudo-1D off)."""
    import torch
    key = "CO"
    r = W.rays(5, 8)
    oc = O.Coolant(key)
    lp = W.levpop(ncell=r["ngrid"], seed=91)
    dens = lp["n_H"] * W.COOLANT_X[key]
    spop = np.array([oc.lte(t, d) for t, d in zip(lp["T"], dens)])
    tau = oc.optical_depths(r, spop, lp["T"], 1.0e5)
    pop_r, cool_r, _, _ = oc.levpop(lp["n_H"], lp["T"], lp["Td"], lp["partner5"], dens, spop, tau)
    rays, keep = G.device_rays(r, cuda)
    d = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=cuda, dtype=torch.float64)
    gc = G.Coolant(key)
    gtau = G.optical_depths(gc, rays, d(spop), d(lp["T"]), 1.0e5)
    pop, cool, _, status = G.level_populations(gc, d(lp["n_H"]), d(lp["T"]), d(lp["Td"]), d(lp["partner5"]),
                                               d(dens), d(spop), gtau)
    pop, cool = pop.cpu().numpy(), cool.cpu().numpy()
    assert (status.cpu().numpy() == 0).all()
    m = pop_r > 1e-6 * dens[:, None]
    assert (np.abs(pop - pop_r)[m] / pop_r[m]).max() < 1e-6
    mc = np.abs(cool_r) > 1e-40
    assert (np.abs(cool - cool_r)[mc] / np.abs(cool_r[mc])).max() < 1e-6
