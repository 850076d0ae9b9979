"""Derive the species layout each reference network's generated code uses.

The reference's generated network code (odes_<net>.c) addresses species by
ODE slot x[0..neq-1] and sums the electron abundance over a fixed set of slots
(odes_<net>.c:44).  The Fortran driver fills those slots in species_<net>.d
order.  For the reduced network the two orders differ: the generated code
expects CH5+, O2, H2+ in slots 4-6 (1-based) while species_reduced.d lists
H2+, CH5+, O2 there, so the reference integrates the permuted system.  A
drop-in has to interpret the slots the same way, so this script recovers, for
every slot, the species the generated code treats it as, by matching each
ode[i] block's loss/formation reactions against the rate file, and records the
electron-sum coefficient of the slot.

Run here, where the reference sources exist:
    python data/make_layouts.py /path/to/reference
It writes data/layout_<net>.d with one record per ODE slot:
    slot(1-based),species_in_species_file,species_in_generated_code,xe_coefficient
"""
import os
import re
import sys


def species_of_slot(block, reac, prod, names):
    loss = [int(r) for r in re.findall(r"rate\[(\d+)\]", block["loss"])]
    form = [int(r) for r in re.findall(r"rate\[(\d+)\]", block["form"])]
    cands = []
    for nm in names:
        if all(nm in reac[r] for r in loss) and all(nm in prod[r] for r in form):
            cands.append(nm)
    return cands


def main(ref):
    here = os.path.dirname(os.path.abspath(__file__))
    for net in ("reduced", "full", "mynetwork"):
        species = [ln.split(",")[1].strip() for ln in open(os.path.join(here, f"species_{net}.d"))
                   if ln.strip()]
        reac, prod = [], []
        for ln in open(os.path.join(here, f"rates_{net}.d")):
            if not ln.strip():
                continue
            f = [x.strip() for x in ln.split(",")]
            reac.append(set(f[1:4]))
            prod.append(set(f[4:8]))
        src = open(os.path.join(ref, f"odes_{net}.c")).read()
        expr = re.search(r"x_e = (.*?);", src).group(1)
        coef = {}
        for sgn, mul, idx in re.findall(r"([+-]?)(\d+\*)?x\[(\d+)\]", expr):
            c = int(mul[:-1]) if mul else 1
            coef[int(idx)] = coef.get(int(idx), 0) + (-c if sgn == "-" else c)
        blocks = {}
        for m in re.finditer(r"loss = (.*?);\s*form = (.*?);\s*ode\[(\d+)\] = form\+x\[(\d+)\]\*loss;",
                             src, re.S):
            blocks[int(m.group(3))] = {"loss": m.group(1), "form": m.group(2)}
        neq = len(species) - 1
        names = species[:neq]
        layout = []
        for s in range(neq):
            c = species_of_slot(blocks[s], reac, prod, names)
            if len(c) != 1:
                # ambiguous: keep the species-file name if it is among the candidates
                c = [species[s]] if species[s] in c else c
            if len(c) != 1:
                raise SystemExit(f"{net}: slot {s + 1} ambiguous {c}")
            layout.append(c[0])
        if sorted(layout) != sorted(names):
            raise SystemExit(f"{net}: layout is not a permutation")
        with open(os.path.join(here, f"layout_{net}.d"), "w") as f:
            for s in range(neq):
                f.write(f"{s + 1},{species[s]},{layout[s]},{coef.get(s, 0)}\n")
        moved = [(s + 1, species[s], layout[s]) for s in range(neq) if species[s] != layout[s]]
        print(net, "slots that differ from the species file:", moved)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PDR_REFERENCE")
    if not ref:
        raise SystemExit("usage: python data/make_layouts.py <3D-PDR source tree> (or set PDR_REFERENCE)")
    main(ref)
