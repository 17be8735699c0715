"""The oracle's own set-up against the reference's fixtures and against the library's set-up, entry by entry.

The oracle (oracle/oracle_setup.c) builds nodes, operators, geometry, face connectivity and the initial state from
the problem parameters with its own algorithms (Sturm-bisected Golub-Welsch nodes, a modal Vandermonde basis,
Gauss-Jordan metric inverses, centroid face matching), so these tests check the library's set-up
(dpgsolver_gb300/host/) independently of it: operators and geometry to 1e-14 of their magnitude, the face tables
through the outward normal of every (volume, local face), and the residual of the oracle's restatement run on
either data model to 1e-12.
"""
import json
import os

import numpy as np
import pytest

import dpgsolver_gb300 as dg
from oracle import Oracle, Problem, nodes
from oracle import oracle_layout as L

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))
TOL = 1e-14

CASES = [
    dict(d=2, p=1, n_elem=(3, 4, 1)),
    dict(d=2, p=2, n_elem=(4, 4, 1), jitter=0.2, seed=5),
    dict(d=2, p=3, n_elem=(3, 2, 1), pde="advection", num_flux="upwind", test_case="advection_sine",
         lo=(0, 0, 0), hi=(1, 1, 1)),
    dict(d=2, p=4, n_elem=(2, 3, 1), jitter=0.15, seed=2),
    dict(d=3, p=1, n_elem=(2, 3, 2)),
    dict(d=3, p=2, n_elem=(3, 2, 2), jitter=0.15, seed=7),
    dict(d=3, p=3, n_elem=(2, 2, 2)),
    dict(d=3, p=4, n_elem=(2, 2, 1), jitter=0.1, seed=1, num_flux="Lax-Friedrichs"),
    # walls and the curved annulus (boundary faces, non-affine volumes)
    dict(d=2, p=2, n_elem=(4, 3, 1), lo=(0, 0, 0), hi=(2, 1, 1), jitter=0.1, seed=3, test_case="free_stream",
         bc=("periodic", "periodic", "slipwall", "riemann")),
    dict(d=2, p=3, n_elem=(4, 3, 1), lo=(-5, -5, 0), hi=(5, 5, 1), jitter=0.1, seed=4,
         bc=("periodic", "periodic", "slipwall", "slipwall")),
    dict(d=3, p=2, n_elem=(2, 3, 2), lo=(0, 0, 0), hi=(1, 1, 1), bc=("slipwall", "slipwall") + ("periodic",) * 4,
         test_case="free_stream"),
    dict(d=2, p=3, n_elem=(3, 8, 1), mesh="annulus", lo=(1, 0, 0), hi=(2, 0, 0), pde="navier_stokes", mu=5e-3,
         omega=0.5, test_case="taylor_couette", bc=("noslip_all_rotating", "noslip_adiabatic")),
    dict(d=2, p=2, n_elem=(3, 3, 1), lo=(0, 0, 0), hi=(1, 1, 1), pde="navier_stokes", mu=1e-2,
         test_case="free_stream", bc=("periodic", "periodic", "noslip_adiabatic", "noslip_adiabatic")),
]


def _ids(c):
    return (f"d{c['d']}-p{c['p']}" + ("-jit" if c.get("jitter") else "") + ("-" + c["mesh"] if "mesh" in c else "")
            + ("-walls" if "bc" in c else ""))


@pytest.mark.parametrize("key", [k for k, v in GOLD["nodes_tp"].items() if v["kind"] in ("GLoL", "GLe")])
def test_oracle_nodes_match_reference(key):
    g = GOLD["nodes_tp"][key]
    d, p = g["d"], g["p"]
    x1, w1 = nodes("GLL" if g["kind"] == "GLoL" else "GL", p + 1)
    # tensor-product order, first coordinate fastest
    grid = np.array([[x1[(s // (p + 1) ** a) % (p + 1)] for a in range(d)] for s in range((p + 1) ** d)])
    wts = np.array([np.prod([w1[(s // (p + 1) ** a) % (p + 1)] for a in range(d)]) for s in range((p + 1) ** d)])
    rst = np.array(g["rst"]["data"]).reshape(g["rst"]["rows"], g["rst"]["cols"])
    assert grid.shape == rst.shape
    assert np.allclose(grid, rst, atol=2e-15, rtol=0), key
    assert np.allclose(wts, np.array(g["w"]["data"]), atol=1e-15, rtol=1e-15), key


def _pair(case):
    cfg = dg.Config(**case)
    sim = dg.Simulation(cfg)
    orc = Oracle(Problem.like(cfg))
    return sim, orc, L.arrays(dg.load_library().dpg_sim_view(sim.handle)), L.arrays(orc.model)


def _close(a, b, tol=TOL):
    scale = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b))) <= tol * scale


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_operators_entry_by_entry(case):
    sim, orc, A, B = _pair(case)
    for k in ("rst_vs", "rst_vc", "w_vc", "w_fc", "rst_fc", "cv0_vs_vc", "tw1_vt_vc", "cv0_vs_fc", "tw0_vt_fc"):
        assert A[k].shape == B[k].shape, k
        assert _close(A[k], B[k]), (k, float(np.max(np.abs(A[k] - B[k]))))


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_mesh_geometry_and_state_entry_by_entry(case):
    sim, orc, A, B = _pair(case)
    d = case["d"]
    assert np.array_equal(A["xyz_ve"][:, : 1 << d, :d], B["xyz_ve"][:, : 1 << d, :d])
    # curved volumes: metric terms from order-p derivative operators (the two set-ups differ at 1e-14 relative)
    tol = 1e-13 if case.get("mesh") == "annulus" else TOL
    for k in ("metrics_vc", "jacobian_det_vc", "xyz_vc", "sol_coef"):
        assert _close(A[k], B[k], tol), (k, float(np.max(np.abs(A[k] - B[k]))))


def _outward(F, n_vol, n_fl):
    """Per (volume, local face): outward unit normal and surface Jacobian at the face nodes in that volume's own face
    node order, from the face tables (normals are those of side 0; side 1 sees them negated at nc_fc[q])."""
    nfc = F["nc_fc"].shape[1]
    out_n = np.full((n_vol, n_fl, nfc, F["normals_fc"].shape[2]), np.nan)
    out_j = np.full((n_vol, n_fl, nfc), np.nan)
    for f in range(F["face_vol"].shape[0]):
        v0, v1 = F["face_vol"][f]
        l0, l1 = F["face_lf"][f]
        nc = F["nc_fc"][f]
        out_n[v0, l0] = F["normals_fc"][f]
        out_j[v0, l0] = F["jacobian_det_fc"][f]
        if v1 < 0:
            continue
        out_n[v1, l1, nc] = -F["normals_fc"][f]
        out_j[v1, l1, nc] = F["jacobian_det_fc"][f]
    return out_n, out_j


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_face_tables_through_outward_normals(case):
    sim, orc, A, B = _pair(case)
    n_fl = 2 * case["d"]
    na, ja = _outward(A, sim.n_vol, n_fl)
    nb, jb = _outward(B, sim.n_vol, n_fl)
    assert not np.isnan(na).any() and not np.isnan(nb).any(), "a local face without a face"
    tol = 1e-13 if case.get("mesh") == "annulus" else TOL
    assert np.max(np.abs(na - nb)) <= tol
    assert _close(ja, jb, tol)
    # the same pairs of (volume, local face) are neighbours
    pa = {tuple(sorted(((int(v0), int(l0)), (int(v1), int(l1)))))
          for (v0, v1), (l0, l1) in zip(A["face_vol"], A["face_lf"])}
    pb = {tuple(sorted(((int(v0), int(l0)), (int(v1), int(l1)))))
          for (v0, v1), (l0, l1) in zip(B["face_vol"], B["face_lf"])}
    assert pa == pb
    # boundary faces carry the same conditions
    ba = {(int(v), int(l), int(b)) for (v, _), (l, _), b in zip(A["face_vol"], A["face_lf"], A["face_bc"]) if b}
    bb = {(int(v), int(l), int(b)) for (v, _), (l, _), b in zip(B["face_vol"], B["face_lf"], B["face_bc"]) if b}
    assert ba == bb


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_residual_on_either_setup(case):
    """The oracle's residual restatement on the library's data model and on its own agree to 1e-12 (operator
    entries differ at 1e-14 of their magnitude; HEX p = 4 sums 125-term products with cancellation)."""
    sim, orc, A, B = _pair(case)
    on_lib = Oracle(data_model=dg.load_library().dpg_sim_view(sim.handle))
    rng = np.random.default_rng(3)
    u = orc.initial_solution() * (1.0 + 1e-2 * rng.standard_normal(orc.n_dof))
    ma, ra = on_lib.compute_rhs(u)
    mb, rb = orc.compute_rhs(u)
    assert _close(ra, rb, 1e-12), float(np.max(np.abs(ra - rb)) / np.max(np.abs(rb)))
    assert abs(ma - mb) <= 1e-12 * mb


def test_states_are_finite():
    for case in CASES:
        orc = Oracle(Problem.like(dg.Config(**case)))
        u = orc.initial_solution()
        assert np.all(np.isfinite(u)) and np.all(np.isfinite(orc.compute_rhs(u)[1])), case


def test_threads_give_the_serial_result_bit_for_bit():
    orc = Oracle(Problem(d=3, p=2, n_elem=(4, 3, 3), jitter=0.1, seed=4))
    u = orc.initial_solution()
    _, r1 = orc.compute_rhs(u)
    orc.set_threads(5)
    _, r5 = orc.compute_rhs(u)
    assert np.array_equal(r1, r5)
    a, b = u.copy(), u.copy()
    orc.set_threads(1)
    orc.rk_step(a, 1e-3, 2)
    orc.set_threads(3)
    orc.rk_step(b, 1e-3, 2)
    assert np.array_equal(a, b)


def test_l2_error_matches_library():
    cfg = dg.Config(d=2, p=2, n_elem=(6, 6, 1), jitter=0.1, seed=3)
    sim = dg.Simulation(cfg)
    orc = Oracle(sim)
    u = orc.initial_solution()
    ea = sim.l2_error(0.0)
    eb = orc.l2_error(u, 0.0)
    assert np.allclose(ea, eb, rtol=1e-12, atol=0)
    assert np.allclose(sim.l2_error(0.7), orc.l2_error(u, 0.7), rtol=1e-12, atol=0)


def test_gmsh_mesh_read_by_the_oracle():
    ref = os.path.join(os.path.dirname(__file__), "golden", "straight_2d_quad_periodic.msh")
    cfg = dg.Config(d=2, p=2)
    sim = dg.Simulation(cfg, msh=ref)
    orc = Oracle(sim)
    A = L.arrays(dg.load_library().dpg_sim_view(sim.handle))
    B = L.arrays(orc.model)
    assert np.array_equal(A["xyz_ve"][:, :4, :2], B["xyz_ve"][:, :4, :2])
    na, _ = _outward(A, sim.n_vol, 4)
    nb, _ = _outward(B, sim.n_vol, 4)
    assert np.max(np.abs(na - nb)) <= 1e-14
    # the oracle's faces, sides and face order are the reference's own (its connectivity fixture)
    fe = GOLD["fe_straight_2d_quad_periodic"]["faces"]
    got = [[[int(B["face_vol"][f][s]), int(B["face_lf"][f][s])] for s in range(2)] for f in range(len(fe))]
    assert got == fe


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_face_side_zero_is_the_smaller_volume_and_local_face(case):
    """constructor_Faces (computational_elements/face.c:108-148) makes the first volume that reaches a face its
    neigh_info[0]; the Roe-Pike flux is not antisymmetric in its two states, so the library must follow."""
    sim, orc, A, B = _pair(case)
    for F in (A, B):
        k0 = F["face_vol"][:, 0] * 8 + F["face_lf"][:, 0]
        k1 = F["face_vol"][:, 1] * 8 + F["face_lf"][:, 1]
        inner = F["face_vol"][:, 1] >= 0
        assert np.all(k0[inner] < k1[inner])
        # faces in the order of their side 0, as constructor_Faces creates them
        assert np.all(np.diff(k0) > 0)
