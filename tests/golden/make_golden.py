"""Generate the golden fixtures of tests/golden from the reference itself.

Run here, where the reference sources exist (oracle/_ref built by
`make -C oracle ref`):  python tests/golden/make_golden.py

  rhs_<net>.npz       the reference's own generated f() (odes_<net>.c, compiled
                      from its sources) evaluated on seeded states: x, rate,
                      n_H -> ode, x_e.  X-ray rates are zero, as the reference's
                      rate evaluator makes them (calc_reac_rates.F90:265-268).
  shield_tables.json  the shielding grids as written in the reference sources
                      (modules.F90:346-366, 3DPDR.F90:1532-1537), parsed from text.
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PDR_REFERENCE", "")
if not os.path.exists(os.path.join(REF, "modules.F90")):
    raise SystemExit("usage: python tests/golden/make_golden.py <3D-PDR source tree> (or set PDR_REFERENCE)")


def fortran_numbers(text):
    return [float(v.replace("D", "e").replace("d", "e")) for v in
            re.findall(r"[-+]?\d+\.\d*(?:[DdEe][-+]?\d+)?", text)]


def shield_tables():
    mod = open(os.path.join(REF, "modules.F90")).read()
    main = open(os.path.join(REF, "3DPDR.F90")).read()

    def block(name):
        m = re.search(r"\b" + name + r"=\(/(.*?)/\)", mod, re.S)
        return fortran_numbers(m.group(1).replace("&", " "))

    sco = []
    for j in range(1, 7):
        m = re.search(r"SCO_GRID\(1:8,%d\) = \(/(.*?)/\)" % j, main)
        sco.append(fortran_numbers(m.group(1)))
    return {"L_GRID": block("L_GRID"), "X_GRID": block("X_GRID"), "NCO_GRID": block("NCO_GRID"),
            "NH2_GRID": block("NH2_GRID"), "SCO_GRID_cols": sco}


def rhs_fixture(name, nstate=8, seed=7):
    net = O.Network(name)
    ref = O.RefNetwork(name)
    rng = np.random.Generator(np.random.PCG64(seed))
    xs, rates, nhs, odes, xes = [], [], [], [], []
    for _ in range(nstate):
        x = 10.0 ** rng.uniform(-20, 0, net.neq)
        rate = 10.0 ** rng.uniform(-20, -8, net.nreac)
        rate[net.ode_kind == 3] = 0.0
        n_H = 10.0 ** rng.uniform(2, 5)
        ode, xe = ref.rhs(net.neq, rate, n_H, x)
        xs.append(x); rates.append(rate); nhs.append(n_H); odes.append(ode); xes.append(xe)
    np.savez_compressed(os.path.join(HERE, f"rhs_{name}.npz"), x=np.array(xs), rate=np.array(rates),
                        n_H=np.array(nhs), ode=np.array(odes), x_e=np.array(xes))


if __name__ == "__main__":
    for n in ("reduced", "full", "mynetwork"):
        rhs_fixture(n)
    with open(os.path.join(HERE, "shield_tables.json"), "w") as f:
        json.dump(shield_tables(), f, indent=1)
