"""The oracle's CALC_UVFIELD and calc_columndens (oracle/orc_rays.c) against
values that follow from the definitions: a uniform density gives a column of
n_H x path length x pc; unit abundances give the total-H column; A_V and the
attenuated field follow from the column; the uni-directional field lands on
the ray most anti-parallel to G."""
import numpy as np

import oracle as O
import workloads as W

PC = 3.08568025e+18


def test_uniform_density_column_is_density_times_path():
    r = W.rays(5, 6)
    r["rho"] = np.full(r["ngrid"], 1.0e3)
    col, av, rad, uv = O.uvfield(r, field=0, G=(10.0, 0.0, 0.0))
    path = r["epray"].reshape(-1, 12) * 0.05
    assert np.allclose(col, 1.0e3 * path * PC, rtol=1e-14)
    assert np.allclose(av, col * float(np.float32(6.289e-22)), rtol=1e-15)
    assert np.all(rad == 10.0 / 12)
    expect = (10.0 / 12) * np.exp(-av * float(np.float32(3.02))).sum(axis=1)
    assert np.allclose(uv, expect, rtol=1e-13)


def test_unit_abundances_give_the_total_column():
    r = W.rays(4, 5, nspec=3)
    r["abundance"] = np.ones_like(r["abundance"])
    col, _, _, _ = O.uvfield(r)
    c = O.columns(r)
    for k in range(3):
        assert np.allclose(c[..., k], col, rtol=1e-14)


def test_uni_directional_field_on_the_antiparallel_ray():
    r = W.rays(3, 3)
    G = (0.0, 0.0, -5.0)            # light travelling towards -z: the rays pointing to +z see it
    _, _, rad, _ = O.uvfield(r, field=1, G=G)
    dots = -(r["vectors"] @ np.array(G))
    j = np.flatnonzero(dots == dots.max())[-1]
    assert np.all(rad[:, j] == dots[j]) and np.count_nonzero(rad[0]) == 1


def test_species_selection_matches_full_columns():
    r = W.rays(4, 5, nspec=9)
    full = O.columns(r)
    sel = O.columns(r, [7, 2, 5])
    assert np.array_equal(sel, full[..., [7, 2, 5]])
