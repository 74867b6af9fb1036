"""Regenerate kirkland_fparams.inc, the table of Kirkland's electron
scattering-factor fit parameters (3 Lorentzians + 3 Gaussians per element,
Z = 1..103), from the reference's hard-coded copy in
TemsimLibrary/slicelib.cpp:958-2212 (ReadfeTable).

The numbers are physical fit constants that must stay identical to the
reference's for the projected potential to match; this script only changes
their layout into a C array initialiser.  Run it from a tree that has the
reference sources:

    python utr_public_gb300/csrc/gen_kirkland_fparams.py <reference tree>

(or with the tree in MSK_REFERENCE_TREE).
"""
import os
import re
import sys


def main(ref_root):
    src = os.path.join(ref_root, "TemsimLibrary", "slicelib.cpp")
    table = [[0.0] * 12 for _ in range(104)]
    seen = set()
    pat = re.compile(r"fparams\[(\d+)\]\[(\d+)\]\s*=\s*([-+0-9.eE]+)\s*;")
    with open(src, "r", errors="replace") as f:
        for line in f:
            m = pat.search(line)
            if m:
                z, i, v = int(m.group(1)), int(m.group(2)), m.group(3)
                table[z][i] = v
                seen.add((z, i))
    missing = [(z, i) for z in range(1, 104) for i in range(12) if (z, i) not in seen]
    if missing:
        raise SystemExit("missing entries: %r" % missing[:5])
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kirkland_fparams.inc")
    with open(out, "w") as f:
        f.write("/* Kirkland electron scattering-factor fit parameters, rows Z = 0..103\n"
                " * (row 0 unused).  Per row: a1 b1 a2 b2 a3 b3 (Lorentzians),\n"
                " * c1 d1 c2 d2 c3 d3 (Gaussians).  Same values as the reference's\n"
                " * TemsimLibrary/slicelib.cpp:958-2212; generated by\n"
                " * gen_kirkland_fparams.py -- do not edit by hand. */\n")
        for z in range(104):
            vals = ", ".join(str(v) for v in table[z])
            f.write("{ %s },\n" % vals)
    print("wrote", out)


if __name__ == "__main__":
    tree = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MSK_REFERENCE_TREE")
    if not tree:
        raise SystemExit("usage: gen_kirkland_fparams.py <reference tree>")
    main(tree)
