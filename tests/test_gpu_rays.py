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
