"""Generate csrc/master_tables.inc: reference-element constants for P = 1..6.

The constants are defined mathematically (Gauss-Lobatto nodes on [0,1], the
Lagrange basis on them, its exact 1-D mass matrix, the inverse and the
differentiation matrix, and the 10-point Gauss-Legendre rule used on faces);
they are evaluated here with mpmath at 60 significant digits, rounded to the
nearest double and printed so that they parse back to that double.  They play the
role of the tables in the reference's src/cartesian/dg/master.h:147-214 and
src/cartesian/util/common.h:15 (Q = 10).

Usage:  python multigrid-ldg_gb300/gen_master_tables.py
"""
import os

import mpmath as mp

mp.mp.dps = 60
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc", "master_tables.inc")
PMAX = 6
QF = 10


def legendre_coeffs(n):
    """Coefficients (highest degree first) of the Legendre polynomial P_n."""
    p0, p1 = [mp.mpf(1)], [mp.mpf(1), mp.mpf(0)]
    if n == 0:
        return p0
    for k in range(2, n + 1):
        # k P_k = (2k-1) t P_{k-1} - (k-1) P_{k-2}
        a = [(2 * k - 1) * c for c in p1] + [mp.mpf(0)]
        b = [mp.mpf(0), mp.mpf(0)] + [(k - 1) * c for c in p0]
        p0, p1 = p1, [(u - v) / k for u, v in zip(a, b)]
    return p1


def real_roots(coeffs):
    roots = mp.polyroots(coeffs, maxsteps=500, extraprec=400)
    return sorted(mp.re(r) for r in roots)


def gll_nodes(P):
    if P == 1:
        return [mp.mpf(1) / 2]
    n = P - 1
    c = legendre_coeffs(n)
    deg = len(c) - 1
    dc = [c[i] * (deg - i) for i in range(deg)]   # P_n'
    inner = real_roots(dc) if n >= 2 else []
    return [mp.mpf(0)] + [(t + 1) / 2 for t in inner] + [mp.mpf(1)]


def lagrange_denoms(x):
    P = len(x)
    out = []
    for i in range(P):
        d = mp.mpf(1)
        for k in range(P):
            if k != i:
                d *= x[i] - x[k]
        out.append(1 / d)
    return out


def gauss_legendre(Q):
    c = legendre_coeffs(Q)
    deg = len(c) - 1
    dc = [c[i] * (deg - i) for i in range(deg)]
    ts = real_roots(c)
    ws = []
    for t in ts:
        dp = mp.polyval(dc, t)
        ws.append(1 / ((1 - t * t) * dp * dp))
    return [(t + 1) / 2 for t in ts], ws


def tables(P):
    x = gll_nodes(P)
    den = lagrange_denoms(x)

    def lag(i, s):
        v = den[i]
        for k in range(P):
            if k != i:
                v *= s - x[k]
        return v

    qx, qw = gauss_legendre(P + 1)
    M = mp.matrix(P, P)
    for q in range(P + 1):
        ls = [lag(i, qx[q]) for i in range(P)]
        for i in range(P):
            for j in range(P):
                M[i, j] += qw[q] * ls[i] * ls[j]
    Minv = M ** -1
    D = mp.matrix(P, P)
    for i in range(P):
        for j in range(P):
            if i != j:
                D[i, j] = (den[j] / den[i]) / (x[i] - x[j])
            else:
                D[i, j] = mp.fsum(1 / (x[i] - x[k]) for k in range(P) if k != i)
    return x, den, M, Minv, D


def fmt(v):
    """Nearest double, printed so that it parses back to the same double."""
    d = float(mp.mpf(v))
    if abs(d) < 1e-40:
        return "0.0"
    return repr(d)


def main():
    lines = ["// Generated by gen_master_tables.py -- do not edit.",
             "// Reference-element constants on [0,1] for P = 1..6 nodes per dimension:",
             "// Gauss-Lobatto nodes, Lagrange denominators, exact 1-D mass matrix, its",
             "// inverse, the differentiation matrix D(i,j) = l_j'(x_i), and the 10-point",
             "// Gauss-Legendre face rule.  Row-major, padded to 6 (x 6).",
             f"#define MGLDG_PMAX {PMAX}",
             f"#define MGLDG_QF {QF}"]
    for name in ["nodes", "denom"]:
        lines.append(f"static const double k{name.capitalize()}[{PMAX}][{PMAX}] = {{")
        for P in range(1, PMAX + 1):
            x, den, M, Minv, D = tables(P)
            arr = x if name == "nodes" else den
            vals = [fmt(v) for v in arr] + ["0.0"] * (PMAX - P)
            lines.append("  {" + ", ".join(vals) + "},")
        lines.append("};")
    for name, idx in [("Mass1", 2), ("InvMass1", 3), ("Diff1", 4)]:
        lines.append(f"static const double k{name}[{PMAX}][{PMAX * PMAX}] = {{")
        for P in range(1, PMAX + 1):
            t = tables(P)[idx]
            vals = []
            for i in range(P):
                for j in range(P):
                    vals.append(fmt(t[i, j]))
            vals += ["0.0"] * (PMAX * PMAX - P * P)
            lines.append("  {" + ", ".join(vals) + "},")
        lines.append("};")
    qx, qw = gauss_legendre(QF)
    lines.append(f"static const double kQuadNodes[{QF}] = {{" + ", ".join(fmt(v) for v in qx) + "};")
    lines.append(f"static const double kQuadWeights[{QF}] = {{" + ", ".join(fmt(v) for v in qw) + "};")
    with open(OUT, "w") as f:
        f.write("\n".join(lines) + "\n")
    print("wrote", OUT)


if __name__ == "__main__":
    main()
