"""Extract known-answer vectors from the reference's own test fixtures into reference_goldens.json.

Reads, as text, from the reference checkout given as the first argument or in $DPG_REFERENCE:
  input/testing/unit/nodes/nodes_tp.data              GL / GLL nodes and weights, tensor-product ordering
  input/testing/unit/nodes/nodes_si.data              2D simplex nodes: equidistant and alpha-optimised p = 3,
                                                      the Witherden-Vincent cubature rule of strength 6
  input/testing/unit/operators/operators_tp.data      tensor-product operators (Kronecker ordering) and products
  input/testing/integration/geom/TEST_straight_2d_quad_periodic.geom.data   face normals of a 2x2 periodic QUAD mesh
  input/testing/integration/mesh/straight_2d_quad_periodic.msh              that mesh
  input/testing/unit/inverse_mapping/quad.data        vertices and points of the inverse-mapping unit test
  input/testing/integration/fe/TEST_straight_2d_quad_periodic.fe.data        volumes and face sides of that mesh
  input/nodes/tri/WV{2,4,6,8}.txt, input/nodes/tet/WV{2,4,6}.txt   Witherden-Vincent cubature rules (symmetry
                                                      orbits in barycentric coordinates and their weights)
and copies that mesh file itself (straight_2d_quad_periodic.msh, the input of the gmsh reader's tests), and, under
reference_input/ with the reference's relative layout, one of its control files with the test case's parameter files:
  input/testing/control_files/euler/periodic_vortex/TEST_Euler_PeriodicVortex_QUAD__ml2__p2.ctrl
  input/input_files/euler/periodic/periodic_vortex/test_case.data, solution.data
The outputs are committed; the tests read only them (the reference checkout is not needed to run them).
"""
from __future__ import annotations

import json
import os
import re
import shutil
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DPG_REFERENCE", "")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_goldens.json")


def _read_matrix(lines, i):
    """lines[i] is 'R|C rows cols' (Matrix_d) or 'R|C order ext...' (Multiarray_d); values are printed row-wise."""
    tok = lines[i].split()
    dims = [int(t) for t in tok[1:]]
    if len(dims) == 2:
        rows, cols = dims
    else:  # Multiarray: 'C order e0 e1 ...' -> treat as e0 x prod(rest)
        order = dims[0]
        ext = dims[1:1 + order]
        rows, cols = ext[0], 1
        for e in ext[1:]:
            cols *= e
    vals = []
    j = i + 1
    while len(vals) < rows * cols:
        vals.extend(float(x) for x in lines[j].split())
        j += 1
    return {"rows": rows, "cols": cols, "data": vals}, j


def parse_nodes(path):
    lines = open(path).read().splitlines()
    out = {}
    i = 0
    while i < len(lines):
        m = re.match(r"^Nodes_d(\d)_p(\d+)_(\w+)$", lines[i].strip())
        if not m:
            i += 1
            continue
        key = lines[i].strip()
        entry = {"d": int(m.group(1)), "p": int(m.group(2)), "kind": m.group(3)}
        i += 1
        while i < len(lines) and not lines[i].startswith("Nodes_") and not lines[i].startswith("---"):
            s = lines[i].strip()
            if s in ("rst:", "w:"):
                name = s[:-1]
                # next lines: 'container Matrix_d', then header
                mat, i = _read_matrix(lines, i + 2)
                entry[name] = mat
                continue
            i += 1
        out[key] = entry
    return out


def parse_operators(path):
    lines = open(path).read().splitlines()
    out = {}
    i = 0
    while i < len(lines):
        s = lines[i].strip()
        m = re.match(r"^(\w+)_(ops_tp|op_std|b|c):$", s)
        if not m:
            i += 1
            continue
        key = m.group(1) + "_" + m.group(2)
        if m.group(2) == "ops_tp":
            n = int(lines[i + 3].split()[1])
            mats = []
            j = i + 4
            for _ in range(n):
                # 'container Matrix_d' then header
                while not lines[j].startswith("container Matrix_d"):
                    j += 1
                if lines[j + 1].strip() == "NULL":
                    mats.append(None)
                    j += 2
                    continue
                mat, j = _read_matrix(lines, j + 1)
                mats.append(mat)
            out[key] = mats
            i = j
        else:
            mat, i = _read_matrix(lines, i + 2)
            out[key] = mat
    return out


def parse_geom_normals(path):
    lines = open(path).read().splitlines()
    faces = []
    i = 0
    while i < len(lines):
        if lines[i].startswith("Face "):
            mat, i = _read_matrix(lines, i + 3)
            faces.append(mat["data"])
            continue
        i += 1
    return faces


def parse_msh_nodes(path):
    lines = open(path).read().splitlines()
    i = lines.index("$Nodes")
    n = int(lines[i + 1])
    return [[float(x) for x in lines[i + 2 + k].split()[1:]] for k in range(n)]


def parse_inverse_mapping(path):
    """ve_random / ve_std / ve_symm (4 x 2 vertex coordinates) and rst_std (n x 2 points of the standard [0, 1]^2
    element; 'C' layout: the values are printed row by row all the same)."""
    lines = open(path).read().splitlines()
    out = {}
    i = 0
    while i < len(lines):
        s = lines[i].strip()
        if s.endswith(":") and i + 2 < len(lines) and lines[i + 1].strip().startswith("container"):
            tok = lines[i + 2].split()
            rows, cols = int(tok[1]), int(tok[2])
            vals = []
            j = i + 3
            while len(vals) < rows * cols:
                vals.extend(float(x) for x in lines[j].split())
                j += 1
            out[s[:-1]] = [vals[r * cols:(r + 1) * cols] for r in range(rows)]
            i = j
            continue
        i += 1
    return out


def parse_fe(path):
    """Volumes' vertex coordinates (tensor-product order) and faces' two sides (ind_v, ind_lf) of a .fe.data file."""
    lines = open(path).read().splitlines()
    vols, faces = [], []
    i = 0
    while i < len(lines):
        s = lines[i].strip()
        if s.startswith("Volume "):
            j = lines.index("xyz_ve:", i)
            tok = lines[j + 2].split()   # 'R order ext0 ext1'
            n = int(tok[2])
            vols.append([[float(x) for x in lines[j + 3 + k].split()] for k in range(n)])
            i = j + 3 + n
            continue
        if s.startswith("Face "):
            sides = []
            j = i + 1
            while j < len(lines) and len(sides) < 2:
                if lines[j].strip().startswith("Neigh_Info"):
                    kv = {}
                    for k in range(1, 6):
                        key, val = lines[j + k].split()
                        kv[key] = int(val)
                    sides.append([kv["ind_v"], kv["ind_lf"]])
                    j += 6
                    continue
                j += 1
            faces.append(sides)
            i = j
            continue
        i += 1
    return {"xyz_ve": vols, "faces": faces}


def parse_wv(path):
    """A symmetric rule file: header, 'Barycentric Coordinates ...' and one orbit representative per line, then
    'Weights' and one weight per orbit (weights of the reference simplex's own volume)."""
    lines = open(path).read().split("\n")
    i = next(k for k, l in enumerate(lines) if l.startswith("Barycentric"))
    j = next(k for k, l in enumerate(lines) if l.startswith("Weights"))
    bary = [[float(x) for x in l.split()] for l in lines[i + 1:j] if l.strip()]
    w = [float(l) for l in lines[j + 1:] if l.strip()]
    return {"bary": bary, "w": w}


def main():
    if not REF:
        raise SystemExit("usage: make_golden.py <reference checkout> (or set DPG_REFERENCE)")
    base = os.path.join(REF, "input", "testing")
    if not os.path.isdir(base):
        sys.exit(f"reference fixtures not found under {base}")
    gold = {
        "source": "DPGSolver input/testing fixtures (nodes_tp.data, nodes_si.data, operators_tp.data, "
                  "TEST_straight_2d_quad_periodic.geom.data, straight_2d_quad_periodic.msh, inverse_mapping/quad.data, "
                  "TEST_straight_2d_quad_periodic.fe.data) and input/nodes/{tri,tet}/WV*.txt",
        "nodes_tp": parse_nodes(os.path.join(base, "unit", "nodes", "nodes_tp.data")),
        "nodes_si": {k: v for k, v in parse_nodes(os.path.join(base, "unit", "nodes", "nodes_si.data")).items()
                     if v["d"] == 2 and v["kind"] in ("EQ", "AO", "WV")},
        "operators_tp": parse_operators(os.path.join(base, "unit", "operators", "operators_tp.data")),
        "geom_straight_2d_quad_periodic_normals": parse_geom_normals(
            os.path.join(base, "integration", "geom", "TEST_straight_2d_quad_periodic.geom.data")),
        "mesh_straight_2d_quad_periodic_nodes": parse_msh_nodes(
            os.path.join(base, "integration", "mesh", "straight_2d_quad_periodic.msh")),
        "inverse_mapping_quad": parse_inverse_mapping(os.path.join(base, "unit", "inverse_mapping", "quad.data")),
        "fe_straight_2d_quad_periodic": parse_fe(
            os.path.join(base, "integration", "fe", "TEST_straight_2d_quad_periodic.fe.data")),
        "wv_rules": {kind: {str(st): parse_wv(os.path.join(REF, "input", "nodes", kind, f"WV{st}.txt")) for st in sts}
                     for kind, sts in (("tri", (2, 4, 6, 8)), ("tet", (2, 4, 6)))},
    }
    with open(OUT, "w") as f:
        json.dump(gold, f, indent=1)
    print(OUT)
    msh = os.path.join(os.path.dirname(OUT), "straight_2d_quad_periodic.msh")
    shutil.copyfile(os.path.join(base, "integration", "mesh", "straight_2d_quad_periodic.msh"), msh)
    print(msh)
    for rel in ("testing/control_files/euler/periodic_vortex/TEST_Euler_PeriodicVortex_QUAD__ml2__p2.ctrl",
                "input_files/euler/periodic/periodic_vortex/test_case.data",
                "input_files/euler/periodic/periodic_vortex/solution.data"):
        dst = os.path.join(os.path.dirname(OUT), "reference_input", rel)
        os.makedirs(os.path.dirname(dst), exist_ok=True)
        shutil.copyfile(os.path.join(REF, "input", rel), dst)
        print(dst)


if __name__ == "__main__":
    main()
