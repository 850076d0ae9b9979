"""Oracle pins for the integrator, rates, shielding tables and level populations."""
import json
import os

import numpy as np
import pytest

import oracle as O
import workloads as W

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_bdf_matches_high_accuracy_radau():
    """The CVODE-method restatement (rtol 1e-8) against SciPy Radau at rtol
    1e-12 on cells of the 64-cell grid: species above 1e-12 agree to 1e-5."""
    scipy = pytest.importorskip("scipy.integrate")
    w = W.chemistry("C1", ncell=3)
    net = O.Network("reduced")
    ph = O.phys(w.zeta, w.omega, w.grain_radius, w.metallicity, w.g2d, w.v_turb_kms)
    rates, _ = net.rates(ph, w.T, w.Td, w.rad_surface, w.AV, w.column5)
    x0 = W.initial_abundances(net.species, s_plus=False)
    ab, st = net.calculate_abundances(np.tile(x0, (3, 1)), rates, w.n_H, w.T)
    assert st == 0
    for c in range(3):
        sol = scipy.solve_ivp(lambda t, y: net.rhs(rates[c], w.n_H[c], y)[0], (0.0, 1e7 * W.YEAR), x0[:-1],
                              method="Radau", jac=lambda t, y: net.jac(rates[c], w.n_H[c], y),
                              rtol=1e-12, atol=1e-40)
        y = sol.y[:, -1]
        m = np.abs(y) > 1e-12
        assert (np.abs(ab[c, :-1][m] - y[m]) / np.abs(y[m])).max() < 1e-5


def test_bdf_counters_are_cvode_like():
    w = W.chemistry("C1", ncell=8)
    net = O.Network("reduced")
    ph = O.phys()
    rates, _ = net.rates(ph, w.T, w.Td, w.rad_surface, w.AV, w.column5)
    x0 = W.initial_abundances(net.species, s_plus=False)
    _, st, stats = net.calculate_abundances(np.tile(x0, (8, 1)), rates, w.n_H, w.T, want_stats=True)
    nst, nfe, nje, nsu, nni = (stats[:, i] for i in range(5))
    assert st == 0
    assert (nsu >= nst / 20.0 - 1).all()            # matrix refreshed at least every 20 steps
    assert (nni >= nst).all() and (nni <= 3 * nst + 3 * nsu).all()
    assert (nfe >= nni).all()


def _natural_y2(x, y):
    from scipy.interpolate import CubicSpline
    return CubicSpline(x, y, bc_type="natural")(x, 2)


def test_shield_tables_match_reference_sources():
    """Spline second derivatives of the library's shielding tables equal those
    of the grids as written in the reference sources (tests/golden)."""
    pytest.importorskip("scipy.interpolate")
    import pdrgpu as G
    g = json.load(open(os.path.join(GOLDEN, "shield_tables.json")))
    xd, sd = G.shield_tables()
    assert np.allclose(xd, _natural_y2(np.array(g["L_GRID"]), np.array(g["X_GRID"])), rtol=1e-9, atol=1e-15)
    sco = np.array(g["SCO_GRID_cols"]).T          # [iNCO][iNH2]
    for i in range(8):
        y2 = _natural_y2(np.array(g["NH2_GRID"]), sco[i])
        assert np.allclose(np.array(sd[i * 6:(i + 1) * 6]), y2, rtol=1e-9, atol=1e-13)
    # the oracle's tables reproduce the grid values at the knots
    lib = O.lib()
    for lam, xv in zip(g["L_GRID"][:-1], g["X_GRID"][:-1]):
        assert abs(lib.orc_xlambda(lam, 0) - xv) < 1e-12
    for i, nco in enumerate(g["NCO_GRID"]):
        for j, nh2 in enumerate(g["NH2_GRID"]):
            v = lib.orc_coshield(10.0 ** nco - 1.0, 10.0 ** nh2 - 1.0)
            assert abs(np.log10(v) - sco[i][j]) < 1e-9


def test_duplicate_groups_select_one_member():
    net = O.Network("full")
    ph = O.phys()
    groups = []
    for r in range(net.nreac):
        if net.duplicate[r] == 1:
            g = [r]
            while g[-1] + 1 < net.nreac and net.duplicate[g[-1] + 1] == net.duplicate[g[-1]] + 1:
                g.append(g[-1] + 1)
            groups.append(g)
    assert groups
    for T in (10.0, 150.0, 800.0, 5000.0, 40000.0):
        rate, nr, st = net.rates_cell(ph, T, 15.0, np.full(12, 10.0 / 12), np.full(12, 1.0),
                                      np.tile([1e18, 0, 1e14, 1e14, 1e12], (12, 1)).ravel())
        for g in groups:
            assert (rate[g] > 0).sum() <= 1


def test_rate_clamps_and_special_reactions():
    net = O.Network("reduced")
    rate, nr, st = net.rates_cell(O.phys(), 100.0, 15.0, np.full(12, 10.0 / 12), np.full(12, 0.5),
                                  np.tile([1e18, 0, 1e14, 1e14, 0], (12, 1)).ravel())
    assert st == 0
    assert list(nr) == [328, 329, 0, 290, 269, 0]   # NRGR, NRH2, NRHD, NRCO, NRCI, NRSI
    assert (rate <= 1.0).all() and ((rate == 0) | (rate >= 1e-99)).all()


def test_gauss_jordan_matches_numpy():
    rng = np.random.Generator(np.random.PCG64(4))
    lib = O.lib()
    for n in (5, 41):
        a = rng.standard_normal((n, n)) + n * np.eye(n)
        b = rng.standard_normal(n)
        a2, b2 = a.copy(), b.copy()
        assert lib.orc_gauss_jordan(O._ptr(a2), n, O._ptr(b2)) == 0
        assert np.allclose(b2, np.linalg.solve(a, b), rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("key", ["CII", "CI", "OI", "CO"])
def test_coolant_tables_and_lte(key):
    c = O.Coolant(key)
    kb = 1.38065040e-16
    # detailed balance of the filled reverse rates at the table temperatures
    for p in range(7):
        for k in range(c.ntemp):
            T = c.temps[p, k]
            if T == 0:
                continue
            for i, j in zip(c.line_up[:3], c.line_lo[:3]):
                if c.col[p, i, j, k] > 0:
                    expect = c.col[p, i, j, k] * c.weights[i] / c.weights[j] * np.exp(
                        -(c.energies[i] - c.energies[j]) / (kb * T))
                    assert np.isclose(c.col[p, j, i, k], expect, rtol=1e-12)
    pop = c.lte(100.0, 1e3)
    assert abs(pop.sum() - 1e3) < 1e-9


@pytest.mark.parametrize("key", ["CII", "CO"])
def test_levpop_conservation(key):
    c = O.Coolant(key)
    lp = W.levpop(ncell=8)
    tau = W.levpop_tau(8, c.nlin, seed=9)
    dens = lp["n_H"] * W.COOLANT_X[key]
    spop = np.array([c.lte(T, d) for T, d in zip(lp["T"], dens)])
    pop, cool, line, st = c.levpop(lp["n_H"], lp["T"], lp["Td"], lp["partner5"], dens, spop, tau)
    assert st == 0
    assert np.allclose(pop.sum(axis=1), dens, rtol=1e-5)
    assert np.isfinite(cool).all()


def test_levpop_conditioning():
    """Perturbing the solvlevpop matrix of the oracle by one ulp (random
    relative 2.2e-16 per entry) moves populations of 1e-12..1e-6 of the
    coolant density by up to ~1e-6..1e-5 relative, while populations above
    1e-6 of it move by < 1e-9: the bound behind the GPU level-population
    tolerances."""
    import ctypes as C
    lib = O.lib()
    lib.orc_find_ccoeff.argtypes = [C.POINTER(O.OrcCoolant), C.c_double, O._dp, O._dp]
    lib.orc_escape_probability.argtypes = [C.POINTER(O.OrcCoolant), O._dp, O._dp, O._dp, C.c_int, C.c_int,
                                           C.c_double, C.c_double, C.c_double, C.c_double, O._dp, O._dp, O._dp]
    oc = O.Coolant("CO")
    lp = W.levpop(ncell=16, seed=21)
    tau = W.levpop_tau(16, oc.nlin, seed=22)
    dens = lp["n_H"] * W.COOLANT_X["CO"]
    spop = np.array([oc.lte(T, d) for T, d in zip(lp["T"], dens)])
    n = oc.nlev
    worst_small = worst_big = 0.0
    for c in range(16):
        Cm, R, L, cool = np.zeros(n * n), np.zeros(n * n), np.zeros(n * n), C.c_double()
        lib.orc_find_ccoeff(oc.p, lp["T"][c], O._ptr(np.ascontiguousarray(lp["partner5"][c])), O._ptr(Cm))
        lib.orc_escape_probability(oc.p, O._ptr(Cm), O._ptr(np.ascontiguousarray(spop[c])),
                                   O._ptr(np.ascontiguousarray(tau[c])), 12, 0, lp["Td"][c], lp["n_H"][c], 1.0,
                                   100.0, O._ptr(R), O._ptr(L), C.byref(cool))
        R = R.reshape(n, n)
        A = R.T.copy()
        np.fill_diagonal(A, -R.sum(axis=1))
        A[-1, :] = 1e-8
        b = np.zeros(n)
        b[-1] = dens[c] * 1e-8
        x = np.linalg.solve(A, b)
        rng = np.random.Generator(np.random.PCG64(c))
        xp = np.linalg.solve(A * (1 + 2.2e-16 * rng.standard_normal(A.shape)), b)
        rel = np.abs(xp - x) / np.maximum(np.abs(x), 1e-300)
        small = (np.abs(x) > 1e-12 * dens[c]) & (np.abs(x) <= 1e-6 * dens[c])
        big = np.abs(x) > 1e-6 * dens[c]
        if small.any():
            worst_small = max(worst_small, rel[small].max())
        worst_big = max(worst_big, rel[big].max())
    assert worst_big < 1e-9
    assert worst_small > 1e-7
