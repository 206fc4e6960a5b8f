"""Extract the triangle volume-cubature rules used by HopeFOAM's DG elements.

HopeFOAM integrates element volume terms with a symmetric triangle cubature of
strength 3(N+1) (HopeFOAM-0.1/src/DG/element/gaussIntegration/gaussIntegration/
gaussIntegration.C:66), taken from the table in
HopeFOAM-0.1/src/DG/element/gaussIntegration/gaussTriangleIntegration/
gaussTriangleIntegrationDataTable.C (``switch(order-1)`` at :35, one ``case`` per
strength, three arrays r / s / w).  Fields computed with any other rule differ
from the reference's at the 1e-6 level, so bit-level parity needs the very same
15-digit numbers.  This script reads that table as data and writes the rules
for the strengths this package uses (N = 1..7) to ``tri_cubature.txt``:

    strength <q> <npts>
    <r> <s> <w>        (npts lines, reference-triangle coordinates, weights sum to 2)

Usage: python make_tri_cubature.py <path to gaussTriangleIntegrationDataTable.C>
"""
import os
import re
import sys

STRENGTHS = [3 * (n + 1) for n in range(1, 8)]


def parse_table(text):
    rules = {}
    for m in re.finditer(r"case\s+(\d+)\s*:\s*\{(.*?)break;", text, re.S):
        case = int(m.group(1))
        body = m.group(2)
        arrays = {}
        for am in re.finditer(r"scalar\s+(data\d+[abc])\[\]\s*=\s*\{([^}]*)\}", body):
            arrays[am.group(1)] = [float(x) for x in am.group(2).split(",")]
        # cub2D[k].append(UList<scalar>(<name>, n))
        cols = [None, None, None]
        for ap in re.finditer(r"cub2D\[(\d)\]\.append\(UList<scalar>\((data\d+[abc]),\s*(\d+)\)\)", body):
            k, name, n = int(ap.group(1)), ap.group(2), int(ap.group(3))
            vals = arrays[name]
            assert len(vals) == n, (case, name, len(vals), n)
            cols[k] = vals
        rules[case + 1] = cols
    return rules


def main():
    src = sys.argv[1]
    with open(src) as f:
        rules = parse_table(f.read())
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tri_cubature.txt")
    with open(out, "w") as f:
        f.write("# triangle cubature rules (reference triangle (-1,-1),(1,-1),(-1,1)); "
                "extracted by make_tri_cubature.py\n")
        for q in STRENGTHS:
            r, s, w = rules[q]
            f.write("strength %d %d\n" % (q, len(w)))
            for a, b, c in zip(r, s, w):
                f.write("%.15f %.15f %.15f\n" % (a, b, c))
    print("wrote", out)


if __name__ == "__main__":
    main()
