"""Extract tests/golden/fin_rows.txt from the reference's Benchmarks.tgz:
per benchmark and output kind, the first and last record and the first
records holding a 3-digit exponent and a negative value.  Each line is
"<kind>|<record>".  Run from the repository root:
    python tests/golden/make_fin_rows.py /path/to/reference/Benchmarks.tgz"""
import os
import re
import sys
import tarfile

src = sys.argv[1]
out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fin_rows.txt")
three = re.compile(r"\d\.\d{3}[+-]\d{3}")
picked = []
with tarfile.open(src) as t:
    for m in sorted(t.getmembers(), key=lambda m: m.name):
        name = os.path.basename(m.name)
        if not name.endswith(".fin"):
            continue
        kind = name.split(".")[1]
        rows = t.extractfile(m).read().decode().splitlines()
        sel = {0, len(rows) - 1}
        for pat in (three, re.compile(r" -\d")):
            for i, r in enumerate(rows):
                if pat.search(r[9:]):
                    sel.add(i)
                    break
        picked += [f"{kind}|{rows[i]}" for i in sorted(sel)]
with open(out, "w") as f:
    f.write("\n".join(picked) + "\n")
print(f"{len(picked)} records -> {out}")
