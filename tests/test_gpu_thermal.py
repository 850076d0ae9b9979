"""The device thermal-balance update and level-population convergence check
against the oracle (oracle/orc_thermal.c), bit for bit: every state array,
the flags and the counts.  Also a closed heating/cooling loop run to
convergence with the state resident on the device, and the chain from the
device heating and level-population kernels into the update."""
import numpy as np
import pytest

import oracle as O
import pdrgpu as G
import workloads as W
from test_oracle_thermal import random_rates, random_state

pytestmark = pytest.mark.gpu
KEYS = ("T", "Tprev", "Tlow", "Thigh", "Fmean", "Fratio")


def dev(a, d, dtype=None):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), device=d, dtype=dtype or torch.float64)


def device_state(st, d):
    import torch
    tb = G.ThermalBalance(dev(st["T"], d))
    for k in KEYS:
        getattr(tb, k).copy_(dev(st[k], d))
    tb.flags.copy_(dev(st["flags"], d, torch.uint8))
    return tb


def assert_same(tb, st):
    for k in KEYS:
        assert np.array_equal(getattr(tb, k).cpu().numpy(), st[k]), k
    assert np.array_equal(tb.flags.cpu().numpy(), st["flags"])


@pytest.mark.parametrize("level_conv,first_time,temp_fix", [(1, 1, 1), (1, 0, 1), (1, 0, 0), (0, 0, 1)])
def test_thermal_update_matches_oracle(cuda, level_conv, first_time, temp_fix):
    rng = np.random.default_rng(100 + 4 * level_conv + 2 * first_time + temp_fix)
    n = 200003
    st = random_state(rng, n)
    st["T"][:500] = rng.uniform(1.0, 2.69, 500)
    st["T"][500:1000] = rng.uniform(30001.0, 50000.0, 500)
    heat, cool = random_rates(rng, n)
    tb = device_state(st, cuda)
    tb.params.temp_fix = temp_fix
    nconv = tb.update(dev(heat, cuda), [dev(c, cuda) for c in cool], level_conv, first_time)
    tot, nconv_r = O.thermal_balance(st, heat, cool, level_conv, first_time, temp_fix=bool(temp_fix))
    assert_same(tb, st)
    assert np.array_equal(tb.total_cooling.cpu().numpy(), tot)
    assert int(nconv.item()) == nconv_r


def test_heating_stride_and_single_coolant(cuda):
    rng = np.random.default_rng(5)
    n = 1000
    st = random_state(rng, n)
    heat, cool = random_rates(rng, n)
    h12 = rng.uniform(0.0, 1.0, (n, 12))
    h12[:, 11] = heat
    tb = device_state(st, cuda)
    tb.update(dev(h12, cuda), [dev(cool[0], cuda)], 1, 0)
    O.thermal_balance(st, heat, [cool[0]], 1, 0)
    assert_same(tb, st)


def test_closed_loop_converges_on_device(cuda):
    """heating 1e-20, cooling 1e-20 (T/T0)^2 per cell: the device loop follows
    the oracle's trajectory exactly and settles on T0."""
    import torch
    rng = np.random.default_rng(9)
    n = 4096
    T0 = np.exp(rng.uniform(np.log(5.0), np.log(20000.0), n))
    st = dict(T=np.full(n, 10.0), Tprev=np.full(n, 10.0), Tlow=np.full(n, 10.0), Thigh=np.full(n, 8000.0),
              Fmean=np.zeros(n), Fratio=np.zeros(n), flags=np.zeros(n, dtype=np.uint8))
    tb = G.ThermalBalance(dev(st["T"], cuda))
    T0d = dev(T0, cuda)
    heat = torch.full((n,), 1.0e-20, dtype=torch.float64, device=cuda)
    it_d, it_o = G.OuterIteration(n), G.OuterIteration(n)
    it_d.level_conv = it_o.level_conv = True
    for step in range(300):
        cool_d = 1.0e-20 * (tb.T * tb.T) / (T0d * T0d)
        nconv = tb.update(heat, [cool_d], it_d.level_conv, it_d.first_time)
        cool_o = 1.0e-20 * (st["T"] * st["T"]) / (T0 * T0)
        _, nconv_o = O.thermal_balance(st, np.full(n, 1.0e-20), [cool_o], it_o.level_conv, it_o.first_time)
        assert int(nconv.item()) == nconv_o, step
        it_d.after_thermal(int(nconv.item()))
        it_o.after_thermal(nconv_o)
        it_d.level_conv = it_o.level_conv = True
        if it_d.done:
            break
    assert it_d.done and it_o.done
    assert_same(tb, st)
    # roots inside the initial bracket [Tlow0, Thigh0] = [10, 8000] are found;
    # below Tlow0 the reference's first cooling step leaves Tlow at Tlow0, so the
    # chop returns to 10 K and TEMP_FIX stops it there (3DPDR.F90:946-950, 976)
    Tfin = tb.Tprev.cpu().numpy()
    inside = (T0 > 10.0 * 1.01) & (T0 < 8000.0)
    assert np.all(np.abs(Tfin[inside] - T0[inside]) / T0[inside] < 5e-3)


def dev_offset(a, d, offset):
    """a contiguous device copy of a whose data starts `offset` doubles into a
    larger buffer (offset 1: not 16-byte aligned, the kernel's scalar path)"""
    import torch
    buf = torch.zeros(a.size + offset, dtype=torch.float64, device=d)
    buf[offset:] = torch.as_tensor(a.ravel(), device=d)
    return buf[offset:].view(a.shape)


@pytest.mark.parametrize("thermal_balance,offset", [(True, 0), (False, 0), (True, 1)])
def test_level_convergence_matches_oracle(cuda, thermal_balance, offset):
    import torch
    rng = np.random.default_rng(17 + thermal_balance + 2 * offset)
    n = 50001
    nlev = (5, 5, 5, 41)
    species = (3, 5, 7, 11)
    ab = 10.0 ** rng.uniform(-12, -3, (n, 20))
    sols, pops = [], []
    for k, m in enumerate(nlev):
        s = 10.0 ** rng.uniform(-20, 2, (n, m))
        s[rng.random((n, m)) < 0.05] = 0.0
        kind = rng.integers(0, 5, (n, 1))
        # unchanged, small changes, large changes, changes around the 1e-2
        # threshold (both sides, within the band the integer filter leaves to FP64)
        near = 1 + rng.choice([-1.0, 1.0], (n, m)) * rng.uniform(4.9e-3, 1.02e-2, (n, m))
        p = np.where(kind == 0, s, np.where(kind == 1, s * (1 + rng.uniform(-4e-3, 4e-3, (n, m))),
                                            np.where(kind == 2, s * rng.uniform(0.5, 2.0, (n, m)), s * near)))
        p[(kind[:, 0] == 3)] = s[(kind[:, 0] == 3)]
        z = rng.random((n, m)) < 0.02
        p[z] = 0.0
        # values outside the positive normal range: negatives, subnormals, inf, NaN
        for arr in (s, p):
            odd = rng.random((n, m)) < 0.003
            arr[odd] = rng.choice([-1e-5, -3.0, 5e-320, 1e-310, np.inf, -np.inf, np.nan], odd.sum())
        sols.append(s)
        pops.append(p)
    flags = rng.integers(0, 64, n).astype(np.uint8)
    tb = G.ThermalBalance(torch.zeros(n, dtype=torch.float64, device=cuda))
    tb.flags.copy_(dev(flags, cuda, torch.uint8))
    dpops = [dev_offset(p, cuda, offset) for p in pops]
    counts = tb.level_convergence([dev_offset(s, cuda, offset) for s in sols], dpops, dev(ab, cuda), species,
                                  thermal_balance=thermal_balance)
    cconv, counts_r = O.level_convergence(sols, pops, ab, species, flags, thermal_balance)
    assert np.array_equal(counts.cpu().numpy(), counts_r)
    assert np.array_equal(tb.flags.cpu().numpy(), flags)
    assert np.array_equal(tb.coolant_conv.cpu().numpy(), cconv)
    for a, b in zip(dpops, pops):
        assert np.array_equal(a.cpu().numpy(), b, equal_nan=True)


def test_all_converged_resets_level_flags_on_device(cuda):
    import torch
    n = 777
    s = np.abs(np.random.default_rng(2).normal(size=(n, 5))) + 0.1
    tb = G.ThermalBalance(torch.zeros(n, dtype=torch.float64, device=cuda))
    counts = tb.level_convergence([dev(s, cuda)], [dev(s, cuda)], dev(np.ones((n, 2)), cuda), [0])
    assert counts.cpu().tolist() == [n, n]
    assert int(tb.flags.sum().item()) == 0
    counts = tb.level_convergence([dev(s, cuda)], [dev(s, cuda)], dev(np.ones((n, 2)), cuda), [0],
                                  thermal_balance=False)
    assert np.all(tb.flags.cpu().numpy() == G.TB_LEVEL_CONVERGED)


@pytest.mark.parametrize("offset", [0, 1])
def test_all_converged_without_thermal_balance_keeps_the_populations(cuda, offset):
    """3DPDR.F90:1161-1172: without thermal balance, once every cell converged
    the populations are not replaced by SOLUTION (levels below the 1e-10 floor
    may differ by any amount); with one cell unconverged all are replaced."""
    import torch
    rng = np.random.default_rng(31)
    n = 1001
    s = np.abs(rng.normal(size=(n, 41))) + 0.1
    s[:, 40] = 1e-13                      # below the floor 1e-10 * abundance
    p = s.copy()
    p[:, 40] = 7e-12                      # differs, but is never checked
    ab = np.ones((n, 3))
    for thermal_balance, unconverged in ((False, False), (True, False), (False, True)):
        pp = p.copy()
        if unconverged:
            pp[n // 2, 3] *= 1.5
        tb = G.ThermalBalance(torch.zeros(n, dtype=torch.float64, device=cuda))
        dp = dev_offset(pp, cuda, offset)
        counts = tb.level_convergence([dev_offset(s, cuda, offset)], [dp], dev(ab, cuda), [1],
                                      thermal_balance=thermal_balance)
        want = pp.copy()
        flags = np.zeros(n, dtype=np.uint8)
        _, counts_r = O.level_convergence([s], [want], ab, [1], flags, thermal_balance)
        assert np.array_equal(counts.cpu().numpy(), counts_r)
        assert np.array_equal(dp.cpu().numpy(), want)
        assert np.array_equal(want, pp if not (thermal_balance or unconverged) else s)


def test_device_heating_and_cooling_feed_the_update(cuda):
    """The rates -> heating -> (levpop cooling) -> thermal update chain with
    every array on the device; the oracle update on the same heating and
    cooling values agrees bit for bit."""
    w = W.chemistry("C1", ncell=32)
    onet = O.Network("reduced")
    ph = O.phys(w.zeta, w.omega, w.grain_radius, w.metallicity, w.g2d, w.v_turb_kms)
    rates, _ = onet.rates(ph, w.T, w.Td, w.rad_surface, w.AV, w.column5)
    rng = np.random.default_rng(8)
    ab = 10.0 ** rng.uniform(-12, -1, (32, onet.nspec))
    uv = 10.0 ** rng.uniform(-2, 2, 32)
    gnet = G.Network("reduced")
    h = G.heating(gnet, 0, G.phys(w.zeta, w.omega, w.grain_radius, w.metallicity, w.g2d, w.v_turb_kms),
                  dev(w.n_H, cuda), dev(w.T, cuda), dev(w.Td, cuda), dev(uv, cuda), dev(ab, cuda), dev(rates, cuda))
    lp = W.levpop(ncell=32, seed=3)
    cools = []
    for key in ("CII", "CI", "OI", "CO"):
        oc = O.Coolant(key)
        dens = lp["n_H"] * W.COOLANT_X[key]
        spop = np.array([oc.lte(T, d) for T, d in zip(lp["T"], dens)])
        tau = W.levpop_tau(32, oc.nlin, seed=4)
        _, cool, _, _ = G.level_populations(G.Coolant(key), dev(lp["n_H"], cuda), dev(lp["T"], cuda),
                                            dev(lp["Td"], cuda), dev(lp["partner5"], cuda), dev(dens, cuda),
                                            dev(spop, cuda), dev(tau, cuda))
        cools.append(cool)
    st = dict(T=w.T.astype(np.float64).copy(), Tprev=w.T.astype(np.float64).copy(), Tlow=np.full(32, 10.0),
              Thigh=np.full(32, 8000.0), Fmean=np.zeros(32), Fratio=np.zeros(32), flags=np.zeros(32, np.uint8))
    tb = device_state(st, cuda)
    tb.update(h, cools, 1, 1)
    O.thermal_balance(st, h[:, 11].cpu().numpy(), [c.cpu().numpy() for c in cools], 1, 1)
    assert_same(tb, st)
    assert np.all(np.isfinite(st["Fratio"]))
