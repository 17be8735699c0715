"""TRI elements (2D linear advection on periodic boxes of cells split into two triangles, the element type of the
advection configuration), CPU checks.

Pins against the reference's fixtures (input/testing/unit/nodes/nodes_si.data, extracted into
golden/reference_goldens.json):
- the alpha-optimised nodes of order 3 equal the reference's (as a set of points; 1e-14);
- the volume cubature of p = 3 is the reference's Witherden-Vincent rule of strength 6 (points and weights, 5e-14)
  and integrates every monomial of degree <= 6 on the reference triangle as it does.
Independence: the oracle builds TRI operators with a monomial Vandermonde matrix and its own nodes, cubature (a
different rule) and geometry; the cubature-independent operators, the metrics, normals and face correspondences equal
the library's (1e-13) and the residual on either set-up agrees (1e-12).  Properties: constant states are preserved (free stream), and the oracle's L2 error
of the advected sine converges at order >= p + 1 - 0.165 (the reference's criterion,
test_integration_convergence_support.c:49) for p = 1, 2, 3 on jittered meshes."""
import ctypes as C
import json
import os

import numpy as np
import pytest

import dpgsolver_gb300 as dg
from oracle import Oracle, Problem
from oracle import oracle_layout as L
from tests_support import DpgSim, sim_arrays

GOLD = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_goldens.json")))


def _cfg(p, n=(4, 3), jitter=0.1, seed=3):
    return dict(d=2, p=p, n_elem=(n[0], n[1], 1), element="tri", pde="advection", num_flux="upwind",
                test_case="advection_sine", lo=(0, 0, 0), hi=(1, 1, 1), jitter=jitter, seed=seed, b_adv=(1.0, 0.5, 0.0))


def _matrix(e):
    return np.array(e["data"]).reshape(e["rows"], e["cols"])


def test_alpha_optimised_nodes_are_the_reference_nodes():
    ref = _matrix(GOLD["nodes_si"]["Nodes_d2_p3_AO"]["rst"])
    ours = sim_arrays(dg.Simulation(dg.Config(**_cfg(3))))["rst_vs"]
    assert ours.shape == ref.shape
    for x in ref:   # every reference node is one of ours, and the counts agree
        assert np.min(np.linalg.norm(ours - x, axis=1)) <= 1e-14
    for x in ours:
        assert np.min(np.linalg.norm(ref - x, axis=1)) <= 1e-14


def test_cubature_integrates_like_the_reference_rule():
    wv = GOLD["nodes_si"]["Nodes_d2_p6_WV"]
    xr, wr = _matrix(wv["rst"]), _matrix(wv["w"]).ravel()
    s = dg.Simulation(dg.Config(**_cfg(3)))
    ops = C.cast(s.handle, C.POINTER(DpgSim)).contents.ops[0]
    n_c = ops.n_c
    xc = np.ctypeslib.as_array(ops.rst_vc, shape=(n_c * 2,)).reshape(n_c, 2).copy()
    wc = np.ctypeslib.as_array(ops.w_vc, shape=(n_c,)).copy()
    assert abs(wc.sum() - np.sqrt(3.0)) <= 1e-14 and abs(wr.sum() - np.sqrt(3.0)) <= 1e-14
    for i in range(7):
        for j in range(7 - i):
            ours = np.sum(wc * xc[:, 0] ** i * xc[:, 1] ** j)
            theirs = np.sum(wr * xr[:, 0] ** i * xr[:, 1] ** j)
            assert abs(ours - theirs) <= 1e-14, (i, j, ours, theirs)
    assert n_c == len(wr) == 12
    for x, w in zip(xr, wr):   # the same points with the same weights
        k = int(np.argmin(np.linalg.norm(xc - x, axis=1)))
        assert np.linalg.norm(xc[k] - x) <= 5e-14 and abs(wc[k] - w) <= 5e-14


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_oracle_set_up_equals_the_library_set_up(p):
    """The two set-ups use different volume cubatures (the oracle Stroud's (p+2)^2-point rule, the library the
    symmetric rule of strength 2p), both exact for the integrands of affine triangles: the cubature-independent
    products -- mass matrix cv0^T W cv0, weak derivatives tw1_r cv0 -- the constant metrics and every face array
    agree entry by entry."""
    sim = dg.Simulation(dg.Config(**_cfg(p)))
    orc = Oracle(sim)
    A, B = L.arrays(orc.model), sim_arrays(sim)
    for k in ("cv0_vs_fc", "tw0_vt_fc", "normals_fc", "jacobian_det_fc"):
        a, b = np.asarray(A[k]).ravel(), np.asarray(B[k]).ravel()
        assert a.shape == b.shape and np.max(np.abs(a - b)) <= 1e-13 * max(1.0, np.max(np.abs(b))), k
    assert np.array_equal(np.asarray(A["nc_fc"]).ravel(), np.asarray(B["nc_fc"]).ravel())
    for X in (A, B):
        X["mass"] = X["cv0_vs_vc"].T @ (X["w_vc"][:, None] * X["cv0_vs_vc"])
        X["stiff"] = np.stack([X["tw1_vt_vc"][r] @ X["cv0_vs_vc"] for r in range(2)])
        X["met0"] = X["metrics_vc"][:, :, 0]
    for k in ("mass", "stiff", "met0"):
        assert np.max(np.abs(A[k] - B[k])) <= 1e-13 * max(1.0, np.max(np.abs(B[k]))), k
    assert B["w_vc"].size == {1: 3, 2: 6, 3: 12, 4: 16}[p] and A["w_vc"].size == (p + 2) ** 2
    u = orc.initial_solution()
    assert np.max(np.abs(u - sim.sol_coef())) <= 1e-13
    _, r1 = orc.compute_rhs(u)
    _, r2 = Oracle(data_model=dg.load_library().dpg_sim_view(sim.handle)).compute_rhs(u)
    assert np.max(np.abs(r1 - r2)) <= 1e-12 * np.max(np.abs(r1))


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_constant_state_is_preserved(p):
    """Zero to rounding: 1e-11 against a residual scale of ~10 (the oracle's monomial Vandermonde matrix has a
    condition number ~1e4 at p = 4, so its Lagrange basis sums to one only to ~1e-13)."""
    sim = dg.Simulation(dg.Config(**_cfg(p)))   # kept alive while the oracle reads its data model
    for orc in (Oracle(Problem(**_cfg(p))), Oracle(data_model=dg.load_library().dpg_sim_view(sim.handle))):
        m, _ = orc.compute_rhs(np.full(orc.n_dof, 1.7))
        assert m <= 1e-11


@pytest.mark.parametrize("p", [1, 2, 3])
def test_convergence_order(p):
    errs = []
    for n in (4, 8, 16):
        orc = Oracle(Problem(**_cfg(p, (n, n))), threads=8)
        u = orc.initial_solution()
        tf = 0.1
        dt = 0.1 * (1.0 / n) / (1.2 * (2 * p + 1))
        ns = int(np.ceil(tf / dt))
        orc.rk_step(u, tf / ns, ns)
        errs.append(orc.l2_error(u, tf)[0])
    e = np.array(errs)
    order = np.log2(e[-2] / e[-1])
    assert order >= p + 1 - 0.165, (e, order)


@pytest.mark.parametrize("p", [2, 3])
def test_gmsh_triangle_meshes(tmp_path, p):
    """A gmsh file of the same split mesh with rotated vertex lists, clockwise triangles and shuffled node numbers
    gives the residual of the structured TRI mesh (volumes matched by their solution nodes), and the oracle's own
    reader of the file gives the library's residual."""
    from gmsh_writer import write_tri_msh
    from tests_support import match_volumes, remap_state
    msh = str(tmp_path / "tri.msh")
    write_tri_msh(msh, (5, 4), (0.0, 0.0), (1.0, 1.0), rotate_seed=2, flip_every=3, shuffle_seed=5)
    cfg = dg.Config(**_cfg(p, (5, 4), jitter=0.0))
    sim = dg.Simulation(cfg, msh=msh)
    box = dg.Simulation(cfg)
    assert (sim.n_vol, sim.n_face) == (box.n_vol, box.n_face)
    vol, perm = match_volumes(box, sim, tol=1e-9)
    u = box.sol_coef()
    _, r_box = Oracle(data_model=dg.load_library().dpg_sim_view(box.handle)).compute_rhs(u)
    ub = u.reshape(box.n_vol, box.n_var, box.n_s)
    u_msh = np.empty_like(ub)
    u_msh[vol[:, None], :, perm] = ub.transpose(0, 2, 1)
    u_msh = u_msh.reshape(-1)
    _, r_msh = Oracle(data_model=dg.load_library().dpg_sim_view(sim.handle)).compute_rhs(u_msh)
    assert np.max(np.abs(remap_state(box, sim, r_msh, vol, perm) - r_box)) <= 1e-12 * np.max(np.abs(r_box))
    _, r_own = Oracle(cfg, msh=msh).compute_rhs(u_msh)
    assert np.max(np.abs(r_own - r_msh)) <= 1e-12 * np.max(np.abs(r_msh))


@pytest.mark.parametrize("n", [(2, 2), (3, 2), (2, 3)])
def test_periodic_meshes_two_cells_wide(n):
    """Two cells across a periodic direction: distinct edges share their end vertices there, and faces are matched
    by their periodic position; the library's mesh gives the oracle's residual."""
    cfg = _cfg(2, n)
    sim = dg.Simulation(dg.Config(**cfg))
    assert (sim.n_vol, sim.n_face) == (2 * n[0] * n[1], 3 * n[0] * n[1])
    u = sim.sol_coef()
    _, r1 = Oracle(Problem(**cfg)).compute_rhs(u)
    _, r2 = Oracle(data_model=dg.load_library().dpg_sim_view(sim.handle)).compute_rhs(u)
    assert np.max(np.abs(r1 - r2)) <= 1e-12 * np.max(np.abs(r1))
