"""Oracle pins: the CPU restatement against the reference's own network code.

The reference's generated f() (odes_<net>.c) is the only part of its chemistry
path that compiles here; tests/golden/rhs_<net>.npz holds its outputs on seeded
states (tests/golden/make_golden.py), and oracle/_ref has it compiled when the
reference sources are present.
"""
import os

import numpy as np
import pytest

import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
NETS = ["reduced", "full", "mynetwork"]


def term_scale(net, rate, n_H, x, ode):
    J = net.jac(rate, n_H, x)
    return np.abs(J) @ np.abs(x) + np.abs(ode) + 1e-300


@pytest.mark.parametrize("name", NETS)
def test_oracle_rhs_matches_reference_golden(name):
    g = np.load(os.path.join(GOLDEN, f"rhs_{name}.npz"))
    net = O.Network(name)
    for x, rate, n_H, ode_ref, xe_ref in zip(g["x"], g["rate"], g["n_H"], g["ode"], g["x_e"]):
        ode, xe = net.rhs(rate, n_H, x)
        assert abs(xe - xe_ref) <= 1e-14 * abs(xe_ref)
        err = np.abs(ode - ode_ref) / term_scale(net, rate, n_H, x, ode_ref)
        assert err.max() < 1e-13, (name, err.max())


@pytest.mark.parametrize("name", NETS)
def test_oracle_rhs_matches_compiled_reference(name):
    try:
        ref = O.RefNetwork(name)
    except FileNotFoundError:
        pytest.skip("oracle/_ref not built (reference sources absent)")
    net = O.Network(name)
    rng = np.random.Generator(np.random.PCG64(11))
    for _ in range(6):
        x = 10.0 ** rng.uniform(-25, 0, net.neq)
        rate = 10.0 ** rng.uniform(-22, -6, net.nreac)
        rate[net.ode_kind == 3] = 0.0
        n_H = 10.0 ** rng.uniform(1, 6)
        ode_ref, xe_ref = ref.rhs(net.neq, rate, n_H, x)
        ode, xe = net.rhs(rate, n_H, x)
        assert abs(xe - xe_ref) <= 1e-14 * abs(xe_ref)
        assert (np.abs(ode - ode_ref) / term_scale(net, rate, n_H, x, ode_ref)).max() < 1e-13


def test_reduced_layout_is_the_generated_code_order():
    """odes_reduced.c treats slots 4-6 as CH5+, O2, H2+ (species file: H2+, CH5+, O2)."""
    rows = [ln.strip().split(",") for ln in open(os.path.join(O.DATA, "layout_reduced.d"))]
    moved = [(r[1], r[2]) for r in rows if r[1] != r[2]]
    assert moved == [("H2+", "CH5+"), ("CH5+", "O2"), ("O2", "H2+")]
    # the generated electron sum counts the charged slots of that order
    xe = {r[2]: int(r[3]) for r in rows}
    assert xe["CH5+"] == 1 and xe["H2+"] == 1 and xe["O2"] == 0
    for name in ("full", "mynetwork"):
        rows = [ln.strip().split(",") for ln in open(os.path.join(O.DATA, f"layout_{name}.d"))]
        assert all(r[1] == r[2] for r in rows)


@pytest.mark.parametrize("name", NETS)
def test_analytic_jacobian_matches_finite_differences(name):
    net = O.Network(name)
    rng = np.random.Generator(np.random.PCG64(5))
    x = 10.0 ** rng.uniform(-12, 0, net.neq)
    rate = 10.0 ** rng.uniform(-16, -8, net.nreac)
    rate[net.ode_kind == 3] = 0.0
    n_H = 1e3
    J = net.jac(rate, n_H, x)
    f0, _ = net.rhs(rate, n_H, x)
    scale = np.abs(J) @ np.abs(x) + np.abs(f0)
    for j in range(net.neq):
        h = 1e-6 * x[j]
        xp, xm = x.copy(), x.copy()
        xp[j] += h
        xm[j] -= h
        col = (net.rhs(rate, n_H, xp)[0] - net.rhs(rate, n_H, xm)[0]) / (2 * h)
        err = np.abs((J[:, j] - col) * x[j]) / scale
        assert err.max() < 1e-7, (j, err.max())


def test_reference_generated_jac_omits_xe_chain_and_factor_two():
    """The reference's own Jac() (unused by it) holds x_e constant and drops
    the factor 2 of A+A terms; the oracle's x_e-constant Jacobian differs from
    it exactly on homonuclear two-body columns."""
    try:
        ref = O.RefNetwork("reduced")
    except FileNotFoundError:
        pytest.skip("oracle/_ref not built")
    net = O.Network("reduced")
    rng = np.random.Generator(np.random.PCG64(3))
    x = 10.0 ** rng.uniform(-3, 0, net.neq)
    rate = 10.0 ** rng.uniform(-12, -8, net.nreac)
    _, xe = ref.rhs(net.neq, rate, 100.0, x)
    Jr = ref.jac(net.neq, rate, 100.0, x, xe)
    Jx = net.jac_xe_const(rate, 100.0, x, xe)
    bad = np.argwhere(np.abs(Jr - Jx) > 1e-12 * (np.abs(Jr) + np.abs(Jx)))
    assert 0 < len(bad) < 20
