"""Extract tests/golden/benchmark_slabs.npz from the reference's
Benchmarks.tgz: for each of B01-B04 (reduced network, PSEUDO_1D slab of 294
points) the final state and outputs as the `.fin` files print them, in
PDR-cell order:
  pdr   (294, 40)  x [pc], A_V(ray 6), T_gas, T_dust, etype, n_H, UV, 33 abundances
  heat  (294, 12)  the heating terms of .heat.fin
  cool  (294, 5)   CII, CI, OI, CO and total cooling of .cool.fin
  spop  (294, 56)  the CII, CI, OI, CO level populations of .spop.fin
  opdp  (294, 17)  the ray-6 optical depths of .opdp.fin (lines as in .line.fin)
Each array is stored exactly as printed: 4-digit signed mantissas and
decimal exponents (int16 pairs <key>_m, <key>_e; value = m x 10^(e-3)),
read back with tests/slabs.py.  Run from the repository root:
    python tests/golden/make_benchmark_slabs.py /path/to/reference/Benchmarks.tgz"""
import os
import sys
import tarfile
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "3d-pdr_gb300"))
import fin as F  # noqa: E402

out = {}
with tempfile.TemporaryDirectory() as d:
    with tarfile.open(sys.argv[1]) as t:
        t.extractall(d, filter="data")
    b = os.path.join(d, "Benchmarks")
    for case in ("B01", "B02", "B03", "B04"):
        ids, pdr = F.read_pdr_fin(os.path.join(b, f"{case}.pdr.fin"))
        # .pdr.fin holds the last two cells in the order ptot, ptot-1
        ids = np.concatenate([ids[:-2], ids[-1:], ids[-2:-1]])
        pdr = np.concatenate([pdr[:-2], pdr[-1:], pdr[-2:-1]])
        heat = F.read_fin(os.path.join(b, f"{case}.heat.fin"))
        cool = F.read_fin(os.path.join(b, f"{case}.cool.fin"))
        spop = F.read_fin(os.path.join(b, f"{case}.spop.fin"), lead=9)
        opdp = F.read_fin(os.path.join(b, f"{case}.opdp.fin"), lead=9)
        assert np.array_equal(heat[:, 0], ids) and np.array_equal(cool[:, 0], ids)
        out[f"{case}_pdr"] = pdr
        out[f"{case}_heat"] = heat[:, 3:]
        out[f"{case}_cool"] = cool[:, 3:]
        out[f"{case}_spop"] = spop[:, 2:]
        out[f"{case}_opdp"] = opdp[:, 2:]


def encode(a):
    """4-significant-digit decimals -> (mantissa, exponent) int16 arrays"""
    m = np.zeros(a.shape, np.int16)
    e = np.zeros(a.shape, np.int16)
    for idx, v in np.ndenumerate(a):
        if v != 0.0:
            mant, ex = ("%.3E" % v).split("E")
            m[idx] = int(mant.replace(".", ""))
            e[idx] = int(ex)
    return m, e


enc = {}
for k, a in out.items():
    enc[k + "_m"], enc[k + "_e"] = encode(a)
path = os.path.join(HERE, "benchmark_slabs.npz")
np.savez_compressed(path, **enc)
print(path, os.path.getsize(path), "bytes")
