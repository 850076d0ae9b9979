"""The `.fin` writers (3d-pdr_gb300/fin.py, 3DPDR.F90:1270-1507) against the
reference's golden outputs: every B0x file of Benchmarks.tgz is parsed and
written again from the parsed values, and must come out byte for byte (which
pins ES11.3 with its 3-digit exponents, the integer widths, the column
layout and the swapped order of the last two records of .pdr.fin and
.line.fin).  The committed excerpt tests/golden/fin_rows.txt covers the
formatter where the reference tree is absent."""
import os
import tarfile

import numpy as np
import pytest

import fin as F

HERE = os.path.dirname(os.path.abspath(__file__))
import build  # noqa: E402  (the build recipe knows where the reference tree is, if anywhere)

BENCH = os.path.join(build.reference_dir() or "", "Benchmarks.tgz")
NLEV = {"CII": 5, "CI": 5, "OI": 5, "CO": 41}


def test_es_format():
    assert F.es(0.0) == "  0.000E+00"
    assert F.es(78.46) == "  7.846E+01"
    assert F.es(-1.559e-10) == " -1.559E-10"
    assert F.es(5.712e-130) == "  5.712-130"
    assert F.es(-3.3e-200) == " -3.300-200"
    assert F.es(1.0e100) == "  1.000+100"
    assert F.es(9.9995e99) == "  1.000+100"   # rounding carries into the exponent
    assert F._float("5.712-130") == 5.712e-130 and F._float(" 1.000+100") == 1.0e100


def test_committed_rows_round_trip():
    """Each excerpt row re-formatted from its parsed values is identical."""
    with open(os.path.join(HERE, "golden", "fin_rows.txt")) as f:
        for line in f:
            kind, row = line.rstrip("\n").split("|", 1)
            lead = 9 if kind in ("line", "spop", "opdp") else 7
            if kind == "pdr":
                _, t = _parse_pdr_line(row)
                out = f"{int(row[:7]):7d}" + "".join(F.es(v) for v in t[:4]) + f"{int(t[4]):5d}" + \
                      "".join(F.es(v) for v in t[5:])
            else:
                vals = [F._float(row[p:p + 11]) for p in range(lead, len(row), 11)]
                out = f"{int(row[:lead]):{lead}d}" + "".join(F.es(v) for v in vals)
            assert out == row


def _parse_pdr_line(row):
    vals, pos = [], 7
    for _ in range(4):
        vals.append(F._float(row[pos:pos + 11]))
        pos += 11
    vals.append(float(int(row[pos:pos + 5])))
    pos += 5
    while pos < len(row):
        vals.append(F._float(row[pos:pos + 11]))
        pos += 11
    return int(row[:7]), vals


def _pp_order(a):
    """file order (1..n-2, n, n-1) back to pp order"""
    return np.concatenate([a[:-2], a[-1:], a[-2:-1]])


def _lines_from(cols, nrays=None):
    n = cols.shape[0]
    mats, k = {}, 0
    for key in F.COOLANTS:
        m = np.zeros((n, NLEV[key], NLEV[key]) + ((nrays,) if nrays else ()))
        for u, l in F.LINES[key]:
            if nrays:
                m[:, u - 1, l - 1, 6] = cols[:, k]
            else:
                m[:, u - 1, l - 1] = cols[:, k]
            k += 1
        mats[key] = m
    return mats


@pytest.fixture(scope="module")
def benchmarks(tmp_path_factory):
    if not os.path.exists(BENCH):
        pytest.skip("Benchmarks.tgz of the reference is not present")
    d = tmp_path_factory.mktemp("bench")
    with tarfile.open(BENCH) as t:
        t.extractall(d, filter="data")
    return os.path.join(d, "Benchmarks")


@pytest.mark.parametrize("case", ["B01", "B02", "B03", "B04"])
def test_benchmark_files_rewrite_byte_for_byte(benchmarks, tmp_path, case):
    src = lambda k: os.path.join(benchmarks, f"{case}.{k}.fin")
    out = lambda k: str(tmp_path / f"{case}.{k}.fin")
    same = lambda k: open(src(k), "rb").read() == open(out(k), "rb").read()

    ids, t = F.read_pdr_fin(src("pdr"))
    ids, t = _pp_order(ids), _pp_order(t)
    F.pdr_fin(out("pdr"), t[:, 0], t[:, 1], t[:, 2], t[:, 3], t[:, 4].astype(int), t[:, 5], t[:, 6], t[:, 7:],
              ids=ids)
    assert same("pdr")

    c = F.read_fin(src("cool"))
    F.cool_fin(out("cool"), c[:, 1], c[:, 2], [c[:, 3 + k] for k in range(4)], c[:, 7], ids=c[:, 0].astype(int))
    assert same("cool")

    h = F.read_fin(src("heat"))
    F.heat_fin(out("heat"), h[:, 1], h[:, 2], h[:, 3:15], ids=h[:, 0].astype(int))
    assert same("heat")

    ln = _pp_order(F.read_fin(src("line"), lead=9))
    assert np.array_equal(ln[:, 0], np.arange(1, ln.shape[0] + 1))
    F.line_fin(out("line"), ln[:, 1], ln[:, 2], _lines_from(ln[:, 3:]))
    assert same("line")

    sp = F.read_fin(src("spop"), lead=9)
    pops, k = {}, 2
    for key in F.COOLANTS:
        pops[key] = sp[:, k:k + NLEV[key]]
        k += NLEV[key]
    F.spop_fin(out("spop"), sp[:, 1], pops)
    assert same("spop")

    # the benchmarks' .opdp.fin carries A_V(6) where the source writes x
    op = F.read_fin(src("opdp"), lead=9)
    assert np.array_equal(op[:, 1], t[:, 1])
    F.opdp_fin(out("opdp"), op[:, 1], _lines_from(op[:, 2:], nrays=12))
    assert same("opdp")


def test_three_dimensional_layouts(tmp_path):
    """The non-PSEUDO_1D records (3DPDR.F90:1283-1285, 1411-1418): x, y, z instead
    of x, A_V(6), and the A_V of every ray at the end of the record."""
    n, nrays = 3, 12
    x, y, z = np.array([0.1, 0.2, 0.3]), np.array([1.0, 2.0, 3.0]), np.array([-1.0, -2.0, -3.0])
    ab = np.full((n, 33), 1.0e-5)
    AV = np.arange(n * nrays, dtype=float).reshape(n, nrays) + 0.5
    p = tmp_path / "x.pdr.fin"
    F.pdr_fin(str(p), x, None, [10.0, 20.0, 30.0], [5.0, 5.0, 5.0], [1, 1, 2], [1e3, 1e3, 1e3], [1.0, 2.0, 3.0],
              ab, pseudo1d=False, y=y, z=z, AV=AV)
    rows = p.read_text().splitlines()
    assert len(rows) == n and all(len(r) == 7 + 5 * 11 + 5 + (2 + 33 + nrays) * 11 for r in rows)
    # records of the last two cells come in the order n, n-1
    assert [int(r[:7]) for r in rows] == [1, 3, 2]
    r = rows[0]
    assert r[7:18] == F.es(0.1) and r[18:29] == F.es(1.0) and r[29:40] == F.es(-1.0)
    assert int(r[62:67]) == 1 and r[-11:] == F.es(AV[0, -1])
    lines = {k: np.zeros((n, 41 if k == "CO" else 5, 41 if k == "CO" else 5)) for k in F.COOLANTS}
    lines["CII"][:, 1, 0] = [7.0, 8.0, 9.0]
    q = tmp_path / "x.line.fin"
    F.line_fin(str(q), x, None, lines, pseudo1d=False, y=y, z=z, AV=AV)
    rows = q.read_text().splitlines()
    assert [int(r[:9]) for r in rows] == [1, 3, 2]
    assert all(len(r) == 9 + (3 + 17 + nrays) * 11 for r in rows)
    assert rows[1][9 + 3 * 11:9 + 4 * 11] == F.es(9.0)
