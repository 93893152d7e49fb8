"""Generate tests/golden/master_tables.json from the reference's own source.

Reads the constant tables of src/cartesian/dg/master.h (Gauss-Lobatto nodes,
Lagrange denominators, 1-D mass / inverse mass / differentiation matrices,
Gauss-Legendre nodes and weights) as TEXT -- nothing of the reference is
compiled or run -- and stores them as decimal strings so the oracle's and the
product's recomputed tables can be pinned against them.  It also records the
reference's only literal known answer, the 2x2-block multiply_mv of
tests/cartesian/matrix_tests.cpp:13,31-35.

Usage:  python tests/golden/make_golden.py [/path/to/reference]
"""
import json
import os
import re
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "master_tables.json")


def parse_list(body):
    return [s.strip() for s in body.split(",") if s.strip()]


def main():
    src = open(os.path.join(REF, "src/cartesian/dg/master.h")).read()
    out = {"source": "src/cartesian/dg/master.h", "tables": {}}
    pat_mat = re.compile(
        r"template<> const KronMat<1,(\d)> (Master<1,\d>::mass|Master<1,\d>::invmass|GaussLobatto<\d>::diff)"
        r" = \(KronMat<1,\d>\(\) << (.*?)\)\.finished\(\);")
    for m in pat_mat.finditer(src):
        P = int(m.group(1))
        kind = m.group(2).split("::")[1]
        out["tables"].setdefault(str(P), {})[kind] = parse_list(m.group(3))
    pat_arr = re.compile(r"template<> const double (GaussLobatto|LagrangePoly|Quadrature)<(\d+)>::"
                         r"(nodes|denom|weights)\[\]\s*= \{(.*?)\};")
    quad = {}
    for m in pat_arr.finditer(src):
        cls, n, kind, body = m.group(1), int(m.group(2)), m.group(3), m.group(4)
        vals = parse_list(body)
        if cls == "Quadrature":
            quad.setdefault(str(n), {})[kind] = vals
        else:
            key = "nodes" if cls == "GaussLobatto" else "denom"
            out["tables"].setdefault(str(n), {})[key] = vals
    out["quadrature"] = quad
    # tests/cartesian/matrix_tests.cpp:13 (x = ones), :31-34 (blocks), :35 (y = T x)
    mt = open(os.path.join(REF, "tests/cartesian/matrix_tests.cpp")).read()
    blocks = []
    for m in re.finditer(r"T\.setBlock\((\d),(\d),\(Mat\(\) << ([\d,]+)\)\.finished\(\)\);", mt):
        blocks.append({"i": int(m.group(1)), "j": int(m.group(2)),
                       "vals": [float(v) for v in m.group(3).split(",")]})
    ysum = [0.0] * 4
    for b in blocks:
        v = b["vals"]
        for r in range(2):
            ysum[2 * b["i"] + r] += v[2 * r] + v[2 * r + 1]
    out["matrix_tests_2x2"] = {"source": "tests/cartesian/matrix_tests.cpp:13,31-35",
                               "blocks": blocks, "x": [1.0] * 4, "y": ysum}
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", OUT, "P tables:", sorted(out["tables"]), "Q:", sorted(quad, key=int), "2x2 y:", ysum)


if __name__ == "__main__":
    main()
