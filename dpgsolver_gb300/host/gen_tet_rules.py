"""Fully symmetric cubature rules on the tetrahedron, derived here, for the volumes of tetrahedra of orders 1..3.

Each rule is a union of symmetry orbits in barycentric coordinates -- (a, a, a, 1-3a) (S31, 4 points),
(a, a, 1/2-a, 1/2-a) (S22, 6 points), (a, a, b, 1-2a-b) (S211, 12 points) -- whose parameters and weights solve the
moment equations of every monomial up to the rule's strength, found by least squares from seeded starting points
and kept only with positive weights and interior points (the search of gen_tri_rules.py, one dimension up).
Strengths 2, 4, 6 with 4, 14, 24 points (the point counts of the classical positive interior rules); order 4 keeps
the collapsed Gauss-Jacobi rule.  The 14-point orbit structure solves the strength-4 equations along a one-parameter
family; the member solved for is the one that also integrates degree 5 exactly (the one member whose degree-5
truncation error vanishes, as in Keast's and Witherden and Vincent's 14-point rule).

    python dpgsolver_gb300/host/gen_tet_rules.py   # writes dpgsolver_gb300/host/tet_sym_rules.inc

Needs numpy and scipy (the generated file is committed; the library's build only compiles it).
"""
import itertools
import os
from math import factorial

import numpy as np
from scipy.optimize import least_squares

STRUCTURES = {2: ["S31"], 4: ["S31", "S31", "S22"], 6: ["S31", "S31", "S31", "S211"]}
SOLVE_DEGREE = {2: 2, 4: 5, 6: 6}   # degree of the moment equations solved for each rule
_NPRM = {"S31": 1, "S22": 1, "S211": 2}


def _moment(i, j, k):
    """Integral of l1^i l2^j l3^k over the unit tetrahedron (volume 1/6)."""
    return factorial(i) * factorial(j) * factorial(k) / factorial(i + j + k + 3)


def _orbit(kind, prm):
    if kind == "S31":
        a = prm[0]
        base = (a, a, a, 1 - 3 * a)
    elif kind == "S22":
        a = prm[0]
        base = (a, a, 0.5 - a, 0.5 - a)
    else:
        a, b = prm
        base = (a, a, b, 1 - 2 * a - b)
    return sorted(set(itertools.permutations(base)))


def _unpack(structure, x):
    pts, ws, o = [], [], 0
    for k in structure:
        n = _NPRM[k]
        P = _orbit(k, x[o:o + n])
        pts += P
        ws += [x[o + n]] * len(P)
        o += n + 1
    return np.array(pts), np.array(ws)


def derive(strength):
    structure = STRUCTURES[strength]
    n = SOLVE_DEGREE[strength]
    mons = [(i, j, k) for i in range(n + 1) for j in range(n + 1 - i) for k in range(n + 1 - i - j)]

    def res(x):
        P, W = _unpack(structure, x)
        return np.array([np.sum(W * P[:, 1] ** i * P[:, 2] ** j * P[:, 3] ** k) - _moment(i, j, k) for i, j, k in mons])

    for seed in range(5000):
        rng = np.random.default_rng(seed)
        x0 = []
        for k in structure:
            x0 += ([rng.uniform(0.01, 0.32), rng.uniform(0.005, 0.05)] if k == "S31" else
                   [rng.uniform(0.01, 0.24), rng.uniform(0.005, 0.05)] if k == "S22" else
                   [rng.uniform(0.01, 0.45), rng.uniform(0.01, 0.45), rng.uniform(0.002, 0.03)])
        r = least_squares(res, x0, xtol=1e-15, ftol=1e-15, gtol=1e-15, max_nfev=2000)
        P, W = _unpack(structure, r.x)
        if np.max(np.abs(res(r.x))) < 1e-15 and np.all(W > 0) and np.all(P > 1e-12):
            return P, W / W.sum()   # weights of a unit-volume tetrahedron
    raise RuntimeError(f"no rule of strength {strength}")


def main():
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tet_sym_rules.inc")
    lines = ["/* Fully symmetric tetrahedron cubature rules (barycentric l0..l3 and weights summing to 1), strengths",
             " * 2, 4, 6: generated by gen_tet_rules.py (least-squares solution of the moment equations over symmetry",
             " * orbits); do not edit. */"]
    for s in sorted(STRUCTURES):
        P, W = derive(s)
        lines.append(f"static const int tet_sym_n{s} = {len(W)};")
        lines.append(f"static const double tet_sym_rule{s}[{len(W)}][5] = {{")
        for p, w in zip(P, W):
            lines.append("\t{" + ", ".join(f"{v:.17e}" for v in (*p, w)) + "},")
        lines.append("};")
    open(out, "w").write("\n".join(lines) + "\n")
    print("wrote", out)


if __name__ == "__main__":
    main()
