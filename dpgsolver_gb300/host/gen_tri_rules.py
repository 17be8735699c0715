"""Fully symmetric cubature rules on the triangle, derived here, for the faces of tetrahedra.

The two sides of a triangular face parametrise it from their own vertex orders, so its cubature must be invariant
under the six permutations of the triangle's vertices (then the node correspondence across the face is a
permutation).  Each rule is a union of symmetry orbits in barycentric coordinates -- the centroid (S3), three points
(a, a, 1-2a) (S21), six points (a, b, 1-a-b) (S111) -- whose parameters and weights solve the moment equations of
every monomial up to the rule's strength (the approach of Lyness and Jespersen, and of Witherden and Vincent's
search), found here by least squares from seeded starting points and kept only with positive weights and interior
points.  Strengths 2, 4, 6, 8 (the 2p of orders 1..4).

    python dpgsolver_gb300/host/gen_tri_rules.py   # writes dpgsolver_gb300/host/tri_sym_rules.inc

Needs numpy and scipy (the generated file is committed; the library's build only compiles it).
"""
import itertools
import os
from math import factorial

import numpy as np
from scipy.optimize import least_squares

# strength -> orbit structure (the point counts of the classical minimal positive interior rules: 3, 6, 12, 16)
STRUCTURES = {2: ["S21"], 4: ["S21", "S21"], 6: ["S21", "S21", "S111"], 8: ["S3", "S21", "S21", "S21", "S111"]}


def _moment(i, j):
    """Integral of x^i y^j over the unit triangle (0,0), (1,0), (0,1)."""
    return factorial(i) * factorial(j) / factorial(i + j + 2)


def _orbit(kind, prm):
    if kind == "S3":
        return [(1 / 3, 1 / 3, 1 / 3)]
    if kind == "S21":
        a = prm[0]
        return [(a, a, 1 - 2 * a), (a, 1 - 2 * a, a), (1 - 2 * a, a, a)]
    a, b = prm
    return sorted(set(itertools.permutations((a, b, 1 - a - b))))


def _unpack(structure, x):
    pts, ws, o = [], [], 0
    for k in structure:
        if k == "S3":
            w, P = x[o], _orbit("S3", ()); o += 1
        elif k == "S21":
            w, P = x[o + 1], _orbit("S21", (x[o],)); o += 2
        else:
            w, P = x[o + 2], _orbit("S111", (x[o], x[o + 1])); o += 3
        pts += P
        ws += [w] * len(P)
    return np.array(pts), np.array(ws)


def derive(strength):
    structure = STRUCTURES[strength]
    mons = [(i, j) for i in range(strength + 1) for j in range(strength + 1 - i)]

    def res(x):
        P, W = _unpack(structure, x)
        return np.array([np.sum(W * P[:, 1] ** i * P[:, 2] ** j) - _moment(i, j) for i, j in mons])

    for seed in range(5000):
        rng = np.random.default_rng(seed)
        x0 = []
        for k in structure:
            x0 += ([rng.uniform(0.05, 0.5)] if k == "S3" else
                   [rng.uniform(0.01, 0.49), rng.uniform(0.01, 0.3)] if k == "S21" else
                   [rng.uniform(0.01, 0.6), rng.uniform(0.01, 0.3), rng.uniform(0.01, 0.3)])
        r = least_squares(res, x0, xtol=1e-15, ftol=1e-15, gtol=1e-15, max_nfev=3000)
        P, W = _unpack(structure, r.x)
        if np.max(np.abs(res(r.x))) < 1e-15 and np.all(W > 0) and np.all(P > 1e-12):
            return P, W / W.sum()   # weights of a unit-area triangle
    raise RuntimeError(f"no rule of strength {strength}")


def main():
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tri_sym_rules.inc")
    lines = ["/* Fully symmetric triangle cubature rules (barycentric l0, l1, l2 and weights summing to 1), strengths",
             " * 2, 4, 6, 8: generated by gen_tri_rules.py (least-squares solution of the moment equations over",
             " * symmetry orbits); do not edit. */"]
    for s in sorted(STRUCTURES):
        P, W = derive(s)
        lines.append(f"static const int tri_sym_n{s} = {len(W)};")
        lines.append(f"static const double tri_sym_rule{s}[{len(W)}][4] = {{")
        for p, w in zip(P, W):
            lines.append("\t{" + ", ".join(f"{v:.17e}" for v in (*p, w)) + "},")
        lines.append("};")
    open(out, "w").write("\n".join(lines) + "\n")
    print("wrote", out)


if __name__ == "__main__":
    main()
