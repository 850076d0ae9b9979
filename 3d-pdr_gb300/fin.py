"""The `.fin` output files of 3D-PDR (3DPDR.F90:1270-1507), byte for byte.

Each writer takes the per-cell results in PDR-cell order (pp = 1..ptot, the
order of IDlist_pdr) and reproduces the reference's records:

* `<out>.pdr.fin`  I7,4ES11.3,I5,300ES11.3: id, x, A_V(ray 6), T_gas, T_dust,
  etype, n_H, UV field, abundances (PSEUDO_1D; the 3D form writes x, y, z,
  T_gas, T_dust, etype, n_H, UV, abundances, then A_V of every ray);
* `<out>.ion.fin`, `<out>.mol.fin`  the ionised and dark cells, without T_dust;
* `<out>.cool.fin`  I7,200ES11.3: id, x, A_V, CII, CI, OI, CO and total cooling;
* `<out>.heat.fin`  I7,200ES11.3: id, x, A_V, the 12 heating terms;
* `<out>.line.fin`  I9,200ES11.3: pp, x, A_V, the emissivities of CII 2-1,
  CI 2-1 3-1 3-2, OI 2-1 3-1 3-2, CO 2-1 ... 11-10;
* `<out>.spop.fin`  I9,200ES11.3: pp, A_V, the populations of CII, CI, OI, CO;
* `<out>.opdp.fin`  I9,200ES11.3 (PSEUDO_1D only): pp, x, the ray-6 optical
  depths of the same lines as `.line.fin`.

The `.pdr.fin` and `.line.fin` records of the last two cells come in the
order ptot, ptot-1, as the reference writes them (3DPDR.F90:1276-1302,
1401-1457).  Fortran's ES11.3 prints a 3-digit exponent without the E
(5.712-130), which `es` and `read_fin` follow.
"""
import math

import numpy as np

# (upper, lower) 1-based level pairs of the lines written to .line.fin / .opdp.fin
LINES = {"CII": [(2, 1)], "CI": [(2, 1), (3, 1), (3, 2)], "OI": [(2, 1), (3, 1), (3, 2)],
         "CO": [(k + 1, k) for k in range(1, 11)]}
COOLANTS = ("CII", "CI", "OI", "CO")


def es(x, w=11, d=3):
    """Fortran ESw.d of one value."""
    x = float(x)
    if math.isnan(x):
        return "NaN".rjust(w)
    if math.isinf(x):
        return ("-Infinity" if x < 0 else "Infinity").rjust(w)
    m, e = ("%.*E" % (d, x)).split("E")
    e = int(e)
    s = f"{m}E{e:+03d}" if abs(e) <= 99 else f"{m}{e:+04d}"
    return s.rjust(w)


def _row(lead, width, *cols):
    out = [f"{int(lead):{width}d}"]
    for c in cols:
        if isinstance(c, tuple):          # ("I", width, value)
            out.append(f"{int(c[2]):{c[1]}d}")
        else:
            for v in np.atleast_1d(c).ravel():
                out.append(es(v))
    return "".join(out) + "\n"


def _order(n, swap_last):
    idx = list(range(n))
    if swap_last and n >= 2:
        idx = idx[:n - 2] + [n - 1, n - 2]
    return idx


def _ids(ids, n):
    return np.arange(1, n + 1) if ids is None else np.asarray(ids)


def pdr_fin(path, x, av6, Tgas, Tdust, etype, rho, uv, abundance, ids=None, pseudo1d=True, y=None, z=None,
            AV=None):
    """`.pdr.fin` (3DPDR.F90:1270-1302); 3D form: pseudo1d=False with y, z and AV (ncell, nrays)."""
    n = len(x)
    ids = _ids(ids, n)
    with open(path, "w") as f:
        for i in _order(n, True):
            if pseudo1d:
                f.write(_row(ids[i], 7, [x[i], av6[i], Tgas[i], Tdust[i]], ("I", 5, etype[i]),
                             [rho[i], uv[i]], abundance[i]))
            else:
                f.write(_row(ids[i], 7, [x[i], y[i], z[i], Tgas[i], Tdust[i]], ("I", 5, etype[i]),
                             [rho[i], uv[i]], abundance[i], AV[i]))


def region_fin(path, x, av6, Tgas, etype, rho, uv, abundance, ids=None, pseudo1d=True, y=None, z=None, AV=None):
    """`.ion.fin` / `.mol.fin` (3DPDR.F90:1305-1340): cells in list order."""
    n = len(x)
    ids = _ids(ids, n)
    with open(path, "w") as f:
        for i in range(n):
            if pseudo1d:
                f.write(_row(ids[i], 7, [x[i], av6[i], Tgas[i]], ("I", 5, etype[i]), [rho[i], uv[i]], abundance[i]))
            else:
                f.write(_row(ids[i], 7, [x[i], y[i], z[i], Tgas[i]], ("I", 5, etype[i]), [rho[i], uv[i]],
                             abundance[i], AV[i]))


def cool_fin(path, x, av6, cooling, total, ids=None, pseudo1d=True, y=None, z=None, AV=None):
    """`.cool.fin` (3DPDR.F90:1350-1361); cooling = (CII, CI, OI, CO) arrays."""
    n = len(x)
    ids = _ids(ids, n)
    with open(path, "w") as f:
        for i in range(n):
            c = [cooling[k][i] for k in range(4)] + [total[i]]
            if pseudo1d:
                f.write(_row(ids[i], 7, [x[i], av6[i]], c))
            else:
                f.write(_row(ids[i], 7, [x[i], y[i], z[i]], c, AV[i]))


def heat_fin(path, x, av6, heating, ids=None, pseudo1d=True, y=None, z=None, AV=None):
    """`.heat.fin` (3DPDR.F90:1372-1385); heating (ncell, 12)."""
    n = len(x)
    ids = _ids(ids, n)
    with open(path, "w") as f:
        for i in range(n):
            if pseudo1d:
                f.write(_row(ids[i], 7, [x[i], av6[i]], heating[i]))
            else:
                f.write(_row(ids[i], 7, [x[i], y[i], z[i]], heating[i], AV[i]))


def _line_values(mats, i, ray=None):
    """The written lines of cell i from per-coolant (ncell, nlev, nlev[, nrays])
    arrays indexed [cell, upper-1, lower-1(, ray)]."""
    out = []
    for key in COOLANTS:
        for u, l in LINES[key]:
            m = mats[key]
            out.append(m[i, u - 1, l - 1] if ray is None else m[i, u - 1, l - 1, ray])
    return out


def line_fin(path, x, av6, lines, pseudo1d=True, y=None, z=None, AV=None):
    """`.line.fin` (3DPDR.F90:1390-1460); lines[key] (ncell, nlev, nlev) emissivities."""
    n = len(x)
    with open(path, "w") as f:
        for i in _order(n, True):
            v = _line_values(lines, i)
            if pseudo1d:
                f.write(_row(i + 1, 9, [x[i], av6[i]], v))
            else:
                f.write(_row(i + 1, 9, [x[i], y[i], z[i]], v, AV[i]))


def spop_fin(path, av6, pops):
    """`.spop.fin` (3DPDR.F90:1466-1476); pops[key] (ncell, nlev)."""
    n = len(av6)
    with open(path, "w") as f:
        for i in range(n):
            f.write(_row(i + 1, 9, [av6[i]], *[pops[k][i] for k in COOLANTS]))


def opdp_fin(path, second, optdepth, ray=6):
    """`.opdp.fin` (3DPDR.F90:1484-1500, PSEUDO_1D): pp, `second` (x in the
    reference's source), the ray's optical depths; optdepth[key] (ncell, nlev,
    nlev, nrays)."""
    n = len(second)
    with open(path, "w") as f:
        for i in range(n):
            f.write(_row(i + 1, 9, [second[i]], _line_values(optdepth, i, ray)))


def _float(tok):
    t = tok.strip()
    if "E" in t or "e" in t or t in ("NaN", "Infinity", "-Infinity"):
        return float(t.replace("Infinity", "inf"))
    # a 3-digit exponent: mantissa then a signed exponent without the E
    k = max(t.rfind("+"), t.rfind("-"))
    return float(t[:k] + "E" + t[k:])


def read_fin(path, lead=7, w=11):
    """Parse a `.fin` file of one leading integer (width `lead`: 7 for
    .cool/.heat, 9 for .line/.spop/.opdp) and ESw.d fields into a float array
    (the integer is column 0)."""
    rows = []
    with open(path) as f:
        for line in f:
            line = line.rstrip("\n")
            vals, pos = [float(line[:lead])], lead
            while pos < len(line):
                vals.append(_float(line[pos:pos + w]))
                pos += w
            rows.append(vals)
    return np.array(rows)


def read_pdr_fin(path, pseudo1d=True):
    """`.pdr.fin` into (ids, table) with the etype column in place: columns
    x, A_V, T_gas, T_dust, etype, n_H, UV, abundances... (PSEUDO_1D)."""
    nlead = 4 if pseudo1d else 5
    ids, rows = [], []
    with open(path) as f:
        for line in f:
            line = line.rstrip("\n")
            ids.append(int(line[:7]))
            pos = 7
            vals = []
            for _ in range(nlead):
                vals.append(_float(line[pos:pos + 11]))
                pos += 11
            vals.append(float(int(line[pos:pos + 5])))
            pos += 5
            while pos < len(line):
                vals.append(_float(line[pos:pos + 11]))
                pos += 11
            rows.append(vals)
    return np.array(ids), np.array(rows)
