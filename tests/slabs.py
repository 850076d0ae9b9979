"""The B01-B04 benchmark slabs of the reference (tests/golden/benchmark_slabs.npz,
made by tests/golden/make_benchmark_slabs.py) and the run parameters that
reproduce them: reduced network, PSEUDO_1D, uni-directional field G0 along
+x onto the x = 0 face (HEALPix ray 6 points back at it), params.dat's
physics (omega 0.42, grain radius 1e-7 cm, gas-to-dust 100, metallicity 1,
v_turb 1 km/s), cosmic-ray rate 1.3e-17 s^-1 (1.3e-15 for B03, which the
cosmic-ray heating column shows).  G0 is the UV field of the surface cell."""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ("B01", "B02", "B03", "B04")
ZETA = {"B01": 1.3e-17, "B02": 1.3e-17, "B03": 1.3e-15, "B04": 1.3e-17}
NLEV = {"CII": 5, "CI": 5, "OI": 5, "CO": 41}
# reduced-network species (species_reduced.d order, 0-based)
SP = {"C+": 10, "H+": 18, "C": 24, "He": 25, "CO": 27, "O": 29, "H2": 30, "H": 31, "e-": 32}
COOLANT_SPECIES = {"CII": "C+", "CI": "C", "OI": "O", "CO": "CO"}
_CACHE = {}


def _decode(m, e):
    out = np.zeros(m.shape)
    for idx, v in np.ndenumerate(m):
        if v:
            out[idx] = float(f"{int(v)}e{int(e[idx]) - 3}")
    return out


def load(case):
    """dict: x, AV6, Tg, Td, n, uv, ab (294, 33), heat (294, 12), cool (294, 5),
    spop {coolant: (294, nlev)}, opdp (294, 17), G0, zeta"""
    if case in _CACHE:
        return _CACHE[case]
    z = np.load(os.path.join(HERE, "golden", "benchmark_slabs.npz"))
    get = lambda k: _decode(z[f"{case}_{k}_m"], z[f"{case}_{k}_e"])
    pdr = get("pdr")
    d = dict(x=pdr[:, 0], AV6=pdr[:, 1], Tg=pdr[:, 2], Td=pdr[:, 3], n=pdr[:, 5], uv=pdr[:, 6],
             ab=pdr[:, 7:].copy(), heat=get("heat"), cool=get("cool"), opdp=get("opdp"), zeta=ZETA[case])
    sp, k = get("spop"), 0
    d["spop"] = {}
    for key in ("CII", "CI", "OI", "CO"):
        d["spop"][key] = sp[:, k:k + NLEV[key]].copy()
        k += NLEV[key]
    d["G0"] = d["uv"][np.argmin(d["x"])]
    _CACHE[case] = d
    return d


def partners(d):
    """number densities of H, H+, e-, He, H2 (the level-population partners)"""
    ab, n = d["ab"], d["n"]
    return np.stack([ab[:, SP[s]] * n for s in ("H", "H+", "e-", "He", "H2")], axis=1)


def coolant_density(d, key):
    return d["ab"][:, SP[COOLANT_SPECIES[key]]] * d["n"]
