"""Pins of the host set-up against the reference's own fixtures (tests/golden/reference_goldens.json, extracted
from input/testing/unit/{nodes,operators} and input/testing/integration/{geom,mesh} by make_golden.py)."""
import ctypes as C
import json
import os

import numpy as np
import pytest

import dpgsolver_gb300 as dg

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))


def _nodes(kind: str, n: int):
    lib = dg.load_library()
    x = (C.c_double * n)()
    w = (C.c_double * n)()
    fn = lib.dpg_nodes_gll if kind == "GLoL" else lib.dpg_nodes_gl
    fn.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    fn.restype = None
    fn(n, x, w)
    return np.array(x[:]), np.array(w[:])


def _tp(d, x1, w1):
    """Tensor-product nodes/weights with the first coordinate fastest (reference ordering)."""
    n = len(x1)
    pts, wts = [], []
    for k in range(n if d > 2 else 1):
        for j in range(n if d > 1 else 1):
            for i in range(n):
                idx = [i, j, k][:d]
                pts.append([x1[t] for t in idx])
                wts.append(np.prod([w1[t] for t in idx]))
    return np.array(pts), np.array(wts)


@pytest.mark.parametrize("key", [k for k, v in GOLD["nodes_tp"].items() if v["kind"] in ("GLoL", "GLe")])
def test_nodes_tp_match_reference(key):
    g = GOLD["nodes_tp"][key]
    d, p = g["d"], g["p"]
    x1, w1 = _nodes(g["kind"], p + 1)
    pts, wts = _tp(d, x1, w1)
    rst = np.array(g["rst"]["data"]).reshape(g["rst"]["rows"], g["rst"]["cols"])
    w = np.array(g["w"]["data"])
    # the fixture prints 16 significant digits
    assert np.allclose(pts, rst, atol=2e-16 * 10, rtol=0), key
    assert np.allclose(wts, w, atol=1e-15, rtol=1e-15), key


@pytest.mark.parametrize("elem", ["quad", "hex"])
def test_tensor_product_operator_ordering(elem):
    lib = dg.load_library()
    lib.dpg_kron_rowmajor.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double), C.c_int, C.c_int,
                                      C.POINTER(C.c_double), C.POINTER(C.c_double)]
    lib.dpg_kron_rowmajor.restype = None
    ops = [np.array(m["data"]).reshape(m["rows"], m["cols"]) for m in GOLD["operators_tp"][elem + "_ops_tp"]]
    acc = ops[0]
    for b in ops[1:]:
        out = np.zeros((acc.shape[0] * b.shape[0], acc.shape[1] * b.shape[1]))
        a_c = np.ascontiguousarray(acc)
        b_c = np.ascontiguousarray(b)
        lib.dpg_kron_rowmajor(a_c.shape[0], a_c.shape[1], a_c.ctypes.data_as(C.POINTER(C.c_double)),
                              b_c.shape[0], b_c.shape[1], b_c.ctypes.data_as(C.POINTER(C.c_double)),
                              out.ctypes.data_as(C.POINTER(C.c_double)))
        acc = out
    g = GOLD["operators_tp"][elem + "_op_std"]
    ref = np.array(g["data"]).reshape(g["rows"], g["cols"])
    # fixture printed with 4 significant digits
    assert np.allclose(acc, ref, rtol=5e-4, atol=5e-7)
    gb, gc = GOLD["operators_tp"][elem + "_b"], GOLD["operators_tp"][elem + "_c"]
    b = np.array(gb["data"]).reshape(gb["rows"], gb["cols"])
    c = np.array(gc["data"]).reshape(gc["rows"], gc["cols"])
    assert np.allclose(acc @ b, c, rtol=1e-9, atol=1e-12)


def test_straight_2d_quad_periodic_normals():
    """The 2x2 periodic QUAD mesh of the reference's geometry test: every face's unit normals are axis-aligned
    and of the same multiset as the reference's (-x, +x, -y, +y) per face node."""
    cfg = dg.Config(d=2, p=2, n_elem=(2, 2, 1), lo=(-1.0, -1.0, 0.0), hi=(1.0, 1.0, 1.0), test_case="free_stream")
    sim = dg.Simulation(cfg)
    view = dg.load_library().dpg_sim_view(sim.handle)
    assert view
    ref = np.array(GOLD["geom_straight_2d_quad_periodic_normals"]).reshape(-1, 2)
    ours = _face_normals(sim)
    # the reference lists both orientations of each face once per side; compare the sets of directions
    ref_set = sorted({tuple(np.round(r, 12)) for r in ref})
    our_set = sorted({tuple(np.round(o, 12)) for o in np.concatenate([ours, -ours])})
    assert ref_set == our_set
    # face nodes: p+1 per face, as in the reference fixture (3 rows for p = 2)
    assert len(GOLD["geom_straight_2d_quad_periodic_normals"][0]) // 2 == sim.n_fc


def _face_normals(sim):
    from tests_support import sim_arrays

    return sim_arrays(sim)["normals_fc"]
