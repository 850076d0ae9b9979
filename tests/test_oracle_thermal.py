"""The oracle's thermal-balance update and level-population convergence check
(oracle/orc_thermal.c) against a line-by-line Python transcription of
3DPDR.F90:928-1050 and 1084-1229 with the reference's own variables
(previouschange as a character, one logical per flag), and against cases whose
answers follow from the text: the first 30% bracket, the Tmin/Tmax ends, the
doleveltmin retry, a closed heating/cooling loop that must settle on its root.
Also the host-side bookkeeping of 3DPDR.F90:1064-1174 (OuterIteration)."""
import numpy as np
import pytest

import oracle as O
import pdrgpu as P

CONV, CHOP, LTMIN, LCONV, HEAT, COOL = 1, 2, 4, 8, 16, 32


def fortran_cell(c, heat, cool, level_conv, first_time, Tmin=2.7, Tmax=30000.0, Fcrit=0.005, Tdiff=0.01,
                 temp_fix=True):
    """3DPDR.F90:928-1050 for one cell; c is a dict of the reference's per-cell variables."""
    if c["converged"]:
        return
    c["Fmean"] = heat - cool
    c["Fratio"] = 2.0 * abs(c["Fmean"]) / abs(heat + cool)
    Fmean, Fratio = c["Fmean"], c["Fratio"]
    if level_conv and first_time:
        dummy = c["T"]
        if Fmean == 0:
            c["Tlow"] = c["T"]
            c["Thigh"] = c["T"]
        elif Fmean > 0:
            c["Tlow"] = c["T"]
            c["T"] = 1.3 * c["T"]
            c["prev"] = "H"
        elif Fmean < 0:
            c["Thigh"] = c["T"]
            c["T"] = 0.7 * c["T"]
            if c["T"] < Tmin:
                c["T"] = Tmin
            c["prev"] = "C"
        c["Tprev"] = dummy
        if c["Tprev"] < Tmin:
            c["Tprev"] = Tmin
    elif level_conv and not first_time:
        dummy = c["T"]
        if Fratio <= Fcrit:
            c["converged"] = True
        if not c["chop"]:
            if Fmean > 0 and c["prev"] == "H":
                c["Tlow"] = c["T"]
                c["T"] = 1.3 * c["T"]
                c["Thigh"] = c["T"]
                c["prev"] = "H"
            if Fmean < 0 and c["prev"] == "C":
                c["Thigh"] = c["T"]
                c["T"] = 0.7 * c["T"]
                c["Tlow"] = c["T"]
                c["prev"] = "C"
                if c["T"] < Tmin:
                    c["T"] = Tmin
                    c["Tlow"] = Tmin
                    c["Thigh"] = Tmin
            if Fmean > 0 and c["prev"] == "C":
                c["T"] = (c["Thigh"] + c["Tlow"]) / 2.0
                c["chop"] = True
            if Fmean < 0 and c["prev"] == "H":
                c["T"] = (c["Thigh"] + c["Tlow"]) / 2.0
                c["chop"] = True
        else:
            if Fmean > 0:
                c["Tlow"] = c["T"]
                c["T"] = (c["T"] + c["Thigh"]) / 2.0
            if Fmean < 0:
                c["Thigh"] = c["T"]
                c["T"] = (c["T"] + c["Tlow"]) / 2.0
        if temp_fix and abs(c["T"] - c["Tprev"]) <= Tdiff and Fratio > Fcrit:
            c["converged"] = True
        c["Tprev"] = dummy
        if dummy < Tmin and Fmean < 0:
            c["converged"] = True
        if dummy > Tmax and Fmean > 0:
            c["converged"] = True
        if c["converged"]:
            if dummy < Tmin:
                c["Tprev"] = Tmin
                c["T"] = Tmin
                if c["tmin"]:
                    c["converged"] = True
                else:
                    c["converged"] = False
                    c["lconv"] = False
                    dummy = Tmin
                c["tmin"] = True
            if dummy > Tmax:
                c["Tprev"] = Tmax
                c["T"] = Tmax


def to_cells(st):
    out = []
    for i in range(st["T"].shape[0]):
        f = int(st["flags"][i])
        out.append(dict(T=st["T"][i], Tprev=st["Tprev"][i], Tlow=st["Tlow"][i], Thigh=st["Thigh"][i],
                        Fmean=st["Fmean"][i], Fratio=st["Fratio"][i], converged=bool(f & CONV),
                        chop=bool(f & CHOP), tmin=bool(f & LTMIN), lconv=bool(f & LCONV),
                        prev="H" if f & HEAT else ("C" if f & COOL else " ")))
    return out


def from_cells(cells):
    st = {k: np.array([c[k] for c in cells], dtype=np.float64) for k in ("T", "Tprev", "Tlow", "Thigh", "Fmean",
                                                                         "Fratio")}
    st["flags"] = np.array([(CONV if c["converged"] else 0) | (CHOP if c["chop"] else 0) |
                            (LTMIN if c["tmin"] else 0) | (LCONV if c["lconv"] else 0) |
                            (HEAT if c["prev"] == "H" else 0) | (COOL if c["prev"] == "C" else 0)
                            for c in cells], dtype=np.uint8)
    return st


def random_state(rng, n):
    T = np.exp(rng.uniform(np.log(1.0), np.log(40000.0), n))
    lo = T * rng.uniform(0.3, 1.0, n)
    hi = T * rng.uniform(1.0, 3.0, n)
    flags = rng.integers(0, 64, n).astype(np.uint8)
    flags[(flags & (HEAT | COOL)) == (HEAT | COOL)] &= np.uint8(~COOL & 0xFF)
    flags[rng.random(n) < 0.5] &= np.uint8(~CONV & 0xFF)
    Tprev = np.where(rng.random(n) < 0.2, T + rng.uniform(-0.01, 0.01, n), T * rng.uniform(0.5, 1.5, n))
    return dict(T=T, Tprev=Tprev, Tlow=lo, Thigh=hi, Fmean=np.zeros(n), Fratio=np.zeros(n), flags=flags)


def random_rates(rng, n):
    heat = np.exp(rng.uniform(np.log(1e-26), np.log(1e-18), n))
    cool = heat * np.exp(rng.uniform(-0.05, 0.05, n) * rng.choice([1.0, 100.0], n))
    eq = rng.random(n) < 0.03
    cool[eq] = heat[eq]     # Fmean == 0
    parts = rng.dirichlet(np.ones(4), n).T * cool
    return heat, [parts[k].copy() for k in range(4)]


@pytest.mark.parametrize("level_conv,first_time,temp_fix", [(1, 1, 1), (1, 0, 1), (1, 0, 0), (0, 1, 1), (0, 0, 1)])
def test_oracle_matches_the_fortran_transcription(level_conv, first_time, temp_fix):
    rng = np.random.default_rng(7 + 3 * level_conv + first_time + 5 * temp_fix)
    n = 3000
    st = random_state(rng, n)
    st["T"][:40] = rng.uniform(1.0, 2.69, 40)          # below Tmin: the doleveltmin path
    st["T"][40:80] = rng.uniform(30001.0, 50000.0, 40)  # above Tmax
    heat, cool = random_rates(rng, n)
    cells = to_cells(st)
    total = ((cool[0] + cool[1]) + cool[2]) + cool[3]
    for i, c in enumerate(cells):
        fortran_cell(c, heat[i], total[i], level_conv, first_time, temp_fix=temp_fix)
    want = from_cells(cells)
    tot, nconv = O.thermal_balance(st, heat, cool, level_conv, first_time, temp_fix=temp_fix)
    assert np.array_equal(tot, total)
    for k in ("T", "Tprev", "Tlow", "Thigh", "Fmean", "Fratio"):
        assert np.array_equal(st[k], want[k]), k
    assert np.array_equal(st["flags"], want["flags"])
    assert nconv == int(np.count_nonzero(want["flags"] & CONV))


def one_cell(T, **kw):
    st = dict(T=np.array([T]), Tprev=np.array([kw.get("Tprev", T)]), Tlow=np.array([kw.get("Tlow", 10.0)]),
              Thigh=np.array([kw.get("Thigh", 8000.0)]), Fmean=np.zeros(1), Fratio=np.zeros(1),
              flags=np.array([kw.get("flags", 0)], dtype=np.uint8))
    return st


def test_first_bracket_heats_or_cools_by_thirty_percent():
    st = one_cell(10.0)
    O.thermal_balance(st, [2.0e-20], [[1.0e-20]], 1, 1)
    assert st["T"][0] == 1.3 * 10.0 and st["Tlow"][0] == 10.0 and st["Tprev"][0] == 10.0
    assert st["flags"][0] == HEAT and st["Fmean"][0] == 1.0e-20
    assert st["Fratio"][0] == 2.0 * 1.0e-20 / (2.0e-20 + 1.0e-20)
    st = one_cell(3.0)
    O.thermal_balance(st, [1.0e-20], [[2.0e-20]], 1, 1)
    assert st["T"][0] == 2.7 and st["Thigh"][0] == 3.0 and st["flags"][0] == COOL   # 0.7*3 < Tmin
    st = one_cell(50.0)
    O.thermal_balance(st, [1.0e-20], [[1.0e-20]], 1, 1)
    assert st["T"][0] == 50.0 and st["Tlow"][0] == 50.0 and st["Thigh"][0] == 50.0 and st["flags"][0] == 0


def test_level_conv_off_updates_only_the_imbalance():
    st = one_cell(100.0, flags=HEAT)
    before = {k: v.copy() for k, v in st.items()}
    O.thermal_balance(st, [3.0], [[1.0]], 0, 0)
    assert st["Fmean"][0] == 2.0 and st["Fratio"][0] == 1.0
    for k in ("T", "Tprev", "Tlow", "Thigh", "flags"):
        assert np.array_equal(st[k], before[k])


def test_closed_loop_settles_on_the_root():
    # heating 1e-20, cooling 1e-20 (T/T0)^2: balance at T0 for every cell
    T0 = np.array([40.0, 100.0, 333.0, 2500.0, 17000.0])
    n = T0.size
    st = dict(T=np.full(n, 10.0), Tprev=np.full(n, 10.0), Tlow=np.full(n, 10.0), Thigh=np.full(n, 8000.0),
              Fmean=np.zeros(n), Fratio=np.zeros(n), flags=np.zeros(n, dtype=np.uint8))
    it = P.OuterIteration(n)
    it.level_conv = True
    for _ in range(200):
        heat = np.full(n, 1.0e-20)
        cool = 1.0e-20 * (st["T"] * st["T"]) / (T0 * T0)
        _, nconv = O.thermal_balance(st, heat, [cool], it.level_conv, it.first_time)
        it.after_thermal(nconv)
        it.level_conv = True
        if it.done:
            break
    assert it.done and it.reason == "thermal balance"
    # converged either on Fratio <= Fcrit or on |dT| <= Tdiff (TEMP_FIX) after the chop
    assert np.all(np.abs(st["Tprev"] - T0) / T0 < 5e-3)
    assert np.all(st["flags"] & CHOP)


def test_tmax_end_clamps_and_converges():
    st = one_cell(29000.0, flags=HEAT, Tlow=25000.0, Thigh=29000.0)
    O.thermal_balance(st, [2.0], [[1.0]], 1, 0)      # 1.3 * 29000 > Tmax, not yet past it
    assert st["T"][0] == 1.3 * 29000.0 and not st["flags"][0] & CONV
    O.thermal_balance(st, [2.0], [[1.0]], 1, 0)      # the temperature used was above Tmax
    assert st["flags"][0] & CONV and st["T"][0] == 30000.0 and st["Tprev"][0] == 30000.0


def test_below_tmin_retries_once_then_converges():
    st = one_cell(2.0, flags=COOL, Tlow=2.0, Thigh=3.0, Tprev=5.0)
    O.thermal_balance(st, [1.0], [[2.0]], 1, 0)
    f = int(st["flags"][0])
    assert not f & CONV and f & LTMIN and not f & LCONV
    assert st["T"][0] == 2.7 and st["Tprev"][0] == 2.7
    st["T"][0] = 2.0
    st["Tprev"][0] = 5.0
    O.thermal_balance(st, [1.0], [[2.0]], 1, 0)
    assert st["flags"][0] & CONV and st["T"][0] == 2.7


def test_converged_cells_are_left_alone():
    st = one_cell(100.0, flags=CONV | HEAT, Tlow=1.0, Thigh=2.0)
    st["Fmean"][0] = 7.0
    before = {k: v.copy() for k, v in st.items()}
    tot, nconv = O.thermal_balance(st, [3.0], [[1.0]], 1, 0)
    assert nconv == 1 and tot[0] == 1.0
    for k in before:
        assert np.array_equal(st[k], before[k])


def test_level_convergence_rules():
    # one coolant, 4 levels; abundance 1 so the floor is 1e-10
    sol = np.array([[1.0, 0.0, 1e-11, 2.0],       # converged: level 3 below the floor, level 2 zero/zero
                    [1.0, 0.5, 0.0, 1.0],         # level 1 changes by 2*0.5/1.5 > 1e-2
                    [1.0, 1.0, 1.0, 1.0],         # relch exactly 2*0.005/1.995 < 1e-2
                    [np.nan, 1.0, 1.0, 1.0]])     # NaN solution is not checked
    pop = np.array([[1.0, 0.0, 5.0, 2.0],
                    [1.0, 1.0, 0.0, 1.0],
                    [1.0, 1.0, 1.0, 1.005],
                    [1.0, 1.0, 1.0, 1.0]])
    ab = np.ones((4, 2))
    flags = np.array([0, LCONV, 0, CONV], dtype=np.uint8)
    p = pop.copy()
    cconv, counts = O.level_convergence([sol], [p], ab, [1], flags, thermal_balance=True)
    assert list(cconv) == [1, 0, 1, 1]
    assert list(counts) == [3, 3]
    assert list(flags) == [LCONV, 0, LCONV, CONV | LCONV]
    assert np.array_equal(p, sol, equal_nan=True)
    # all converged: with thermal balance every level_converged is reset
    flags = np.zeros(2, dtype=np.uint8)
    cconv, counts = O.level_convergence([sol[[0, 2]]], [pop[[0, 2]].copy()], ab[:2], [0], flags, True)
    assert list(counts) == [2, 2] and list(flags) == [0, 0]
    flags = np.zeros(2, dtype=np.uint8)
    O.level_convergence([sol[[0, 2]]], [pop[[0, 2]].copy()], ab[:2], [0], flags, False)
    assert list(flags) == [LCONV, LCONV]


def test_all_converged_without_thermal_balance_keeps_the_populations():
    """Without THERMALBALANCE the reference leaves the loop once every cell
    converged (3DPDR.F90:1161-1172, goto 2) and skips the update of
    :1212-1229: the previous populations are kept, also on levels below the
    floor whose SOLUTION differs from them by any amount.  While one cell has
    not converged every cell's populations are replaced."""
    sol = np.array([[1.0, 0.0, 1e-11, 2.0], [1.0, 1.0, 1.0, 1.0]])
    pop = np.array([[1.0, 0.0, 5.0, 2.0], [1.0, 1.0, 1.0, 1.005]])
    ab = np.ones((2, 2))
    p = pop.copy()
    flags = np.zeros(2, dtype=np.uint8)
    cconv, counts = O.level_convergence([sol], [p], ab, [0], flags, False)
    assert list(counts) == [2, 2] and list(flags) == [LCONV, LCONV]
    assert np.array_equal(p, pop)
    # with thermal balance the reference still updates (goto 1)
    p = pop.copy()
    O.level_convergence([sol], [p], ab, [0], np.zeros(2, dtype=np.uint8), True)
    assert np.array_equal(p, sol)
    # one cell not converged: every cell is updated
    sol2 = np.vstack([sol, [[1.0, 2.0, 1.0, 1.0]]])
    pop2 = np.vstack([pop, [[1.0, 1.0, 1.0, 1.0]]])
    p = pop2.copy()
    cconv, counts = O.level_convergence([sol2], [p], np.ones((3, 2)), [0], np.zeros(3, dtype=np.uint8), False)
    assert list(counts) == [2, 2]
    assert np.array_equal(p, sol2)


def test_level_convergence_needs_every_coolant():
    rng = np.random.default_rng(3)
    n = 50
    sols = [rng.uniform(0.5, 1.0, (n, 5)), rng.uniform(0.5, 1.0, (n, 41))]
    pops = [s * (1.0 + rng.choice([0.0, 0.1], (n, 1))) for s in sols]
    flags = np.zeros(n, dtype=np.uint8)
    want0 = np.all(pops[0] == sols[0], axis=1)
    want1 = np.all(pops[1] == sols[1], axis=1)
    cconv, counts = O.level_convergence(sols, [p.copy() for p in pops], np.ones((n, 3)), [0, 2], flags, False)
    assert np.array_equal(cconv & 1, want0.astype(np.uint8))
    assert np.array_equal((cconv >> 1) & 1, want1.astype(np.uint8))
    assert counts[0] == np.count_nonzero(want0 & want1) and counts[1] == want0.sum() and counts[2] == want1.sum()
    assert np.array_equal((flags & LCONV) != 0, want0 & want1)


def test_outer_iteration_bookkeeping():
    it = P.OuterIteration(10)
    assert not it.after_thermal(3) and it.first_time and not it.level_conv
    assert not it.after_levels(9) and not it.level_conv
    assert not it.after_levels(10) and it.level_conv          # levels converged: thermal balance enabled
    assert not it.after_thermal(4) and not it.first_time and not it.level_conv
    it.after_levels(10)
    assert it.after_thermal(10) and it.reason == "thermal balance"
    it = P.OuterIteration(4, thermal_balance=False)
    assert it.after_levels(4) and it.reason == "level populations"
