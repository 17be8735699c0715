"""The symmetric triangle rules of the TET faces (dpgsolver_gb300/host/tri_sym_rules.inc) and tetrahedron rules of
the TET volumes (tet_sym_rules.inc) are what their generators derive (gen_tri_rules.py, gen_tet_rules.py: least
squares over symmetry orbits), and each integrates every monomial up to its strength exactly, with positive weights
and interior points, invariant under the permutations of the vertices."""
import os
import re
from math import factorial

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "dpgsolver_gb300", "host", "tri_sym_rules.inc")


def _committed():
    text = open(INC).read()
    rules = {}
    for m in re.finditer(r"tri_sym_rule(\d+)\[(\d+)\]\[4\] = \{(.*?)\};", text, flags=re.S):
        vals = np.array([float(v) for v in re.findall(r"[-+0-9.e]+", m.group(3))]).reshape(int(m.group(2)), 4)
        rules[int(m.group(1))] = vals
    return rules


def test_committed_rules_are_exact_and_symmetric():
    rules = _committed()
    assert sorted(rules) == [2, 4, 6, 8]
    assert [len(rules[s]) for s in (2, 4, 6, 8)] == [3, 6, 12, 16]
    for s, r in rules.items():
        b, w = r[:, :3], r[:, 3]
        assert np.all(w > 0) and np.all(b > 0) and abs(w.sum() - 1.0) <= 1e-15
        for i in range(s + 1):
            for j in range(s + 1 - i):
                exact = 2.0 * factorial(i) * factorial(j) / factorial(i + j + 2)   # unit-area triangle
                assert abs(np.sum(w * b[:, 1] ** i * b[:, 2] ** j) - exact) <= 2e-16 * (1 + s), (s, i, j)
        for perm in ((1, 0, 2), (0, 2, 1), (2, 1, 0)):
            bp = b[:, list(perm)]
            for q in range(len(w)):
                k = np.argmin(np.linalg.norm(b - bp[q], axis=1))
                assert np.linalg.norm(b[k] - bp[q]) <= 1e-15 and w[k] == w[q]


def test_generator_reproduces_the_committed_rules():
    pytest.importorskip("scipy")
    import importlib.util
    spec = importlib.util.spec_from_file_location("gen_tri_rules", os.path.join(ROOT, "dpgsolver_gb300", "host",
                                                                                "gen_tri_rules.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    rules = _committed()
    for s in (2, 4, 6):
        P, W = gen.derive(s)
        assert np.max(np.abs(np.column_stack([P, W]) - rules[s])) <= 1e-15, s


def _committed_tet():
    text = open(os.path.join(ROOT, "dpgsolver_gb300", "host", "tet_sym_rules.inc")).read()
    rules = {}
    for m in re.finditer(r"tet_sym_rule(\d+)\[(\d+)\]\[5\] = \{(.*?)\};", text, flags=re.S):
        vals = np.array([float(v) for v in re.findall(r"[-+0-9.e]+", m.group(3))]).reshape(int(m.group(2)), 5)
        rules[int(m.group(1))] = vals
    return rules


def test_committed_tet_rules_are_exact_and_symmetric():
    import itertools
    rules = _committed_tet()
    assert sorted(rules) == [2, 4, 6] and [len(rules[s]) for s in (2, 4, 6)] == [4, 14, 24]
    for s, r in rules.items():
        b, w = r[:, :4], r[:, 4]
        assert np.all(w > 0) and np.all(b > 0) and abs(w.sum() - 1.0) <= 1e-15
        for i, j, k in itertools.product(range(s + 1), repeat=3):
            if i + j + k <= s:
                exact = 6.0 * factorial(i) * factorial(j) * factorial(k) / factorial(i + j + k + 3)   # unit volume
                assert abs(np.sum(w * b[:, 1] ** i * b[:, 2] ** j * b[:, 3] ** k) - exact) <= 1e-14, (s, i, j, k)
        for perm in itertools.permutations(range(4)):
            bp = b[:, list(perm)]
            for q in range(len(w)):
                kk = np.argmin(np.linalg.norm(b - bp[q], axis=1))
                assert np.linalg.norm(b[kk] - bp[q]) <= 1e-15 and w[kk] == w[q]


def test_tet_generator_reproduces_the_committed_rules():
    pytest.importorskip("scipy")
    import importlib.util
    spec = importlib.util.spec_from_file_location("gen_tet_rules", os.path.join(ROOT, "dpgsolver_gb300", "host",
                                                                                "gen_tet_rules.py"))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    rules = _committed_tet()
    for s in (2, 4):
        P, W = gen.derive(s)
        assert np.max(np.abs(np.column_stack([P, W]) - rules[s])) <= 1e-15, s


def test_rules_equal_the_references_witherden_vincent_rules():
    """The derived triangle and tetrahedron rules are the reference's WV rules of the same strengths
    (input/nodes/{tri,tet}/WV<strength>.txt, extracted into the golden fixture; printed to 15 digits)."""
    import itertools
    import json
    gold = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_goldens.json")))["wv_rules"]
    ours = {"tri": _committed(), "tet": _committed_tet()}
    for kind, rules in ours.items():
        nb = 3 if kind == "tri" else 4
        for st, r in rules.items():
            g = gold[kind][str(st)]
            pts, wts = [], []
            for b, w in zip(g["bary"], g["w"]):
                for perm in sorted(set(itertools.permutations(b))):
                    pts.append(perm)
                    wts.append(w)
            pts, wts = np.array(pts), np.array(wts) / np.sum(wts)
            assert len(pts) == len(r), (kind, st)
            for k in range(len(r)):
                dist = np.linalg.norm(pts - r[k, :nb], axis=1)
                j = int(np.argmin(dist))
                assert dist[j] <= 2e-13 and abs(wts[j] - r[k, nb]) <= 1e-13, (kind, st, k)
