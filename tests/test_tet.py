"""TET elements (3D linear advection on periodic boxes of cells split into six tetrahedra), CPU checks.

- the library's rules: the volume rules (gen_tet_rules.py's symmetric rules of strength 2p for p <= 3, the
  collapsed Gauss-Jacobi rule of strength 2p + 1 for p = 4) integrate every monomial up to their strength on the
  reference tetrahedron exactly; the face rules (gen_tri_rules.py) are invariant under the six vertex permutations
  of the face and integrate every monomial of degree <= 2p exactly;
- the oracle's own set-up (barycentric-monomial basis, Stroud's conical product rule, a symmetrised collapsed face
  rule, its own mesh and geometry) gives the library's residual (5e-12: the two bases' Vandermonde matrices at the
  equally spaced nodes of order 4 round differently) and the same initial state; mixed orders 1..4 as well;
- constant states are preserved; the L2 error of the advected sine converges at order >= p + 1 - 0.165 (the
  reference's criterion) for p = 1, 2, 3 on jittered meshes (6^3 and 12^3 cells)."""
import ctypes as C
import itertools
from math import factorial

import numpy as np
import pytest

import dpgsolver_gb300 as dg
from oracle import Oracle, Problem
from oracle import oracle_layout as L

S3, S6 = np.sqrt(3.0), np.sqrt(6.0)
TV = np.array([[-1.0, -1 / S3, -1 / S6], [1.0, -1 / S3, -1 / S6], [0.0, 2 / S3, -1 / S6], [0.0, 0.0, 3 / S6]])
FVE = [(2, 3, 1), (2, 3, 0), (0, 1, 3), (0, 1, 2)]


def _cfg(p, n=(3, 3, 2), jitter=0.1, seed=3, **kw):
    return dict(d=3, p=p, n_elem=n, element="tet", pde="advection", num_flux="upwind", test_case="advection_sine",
                lo=(0, 0, 0), hi=(1, 1, 1), jitter=jitter, seed=seed, b_adv=(1.0, 0.5, 0.25), **kw)


def _ops(sim, k=0):
    return C.cast(sim.handle, C.POINTER(L.DpgSim)).contents.ops[k]


def _arr(ptr, n):
    return np.ctypeslib.as_array(ptr, shape=(n,)).copy()


def _bary(x):
    """Barycentric coordinates of points x [n, 3] on the reference tetrahedron."""
    A = (TV[1:] - TV[0]).T
    l123 = np.linalg.solve(A, (x - TV[0]).T).T
    return np.column_stack([1 - l123.sum(axis=1), l123])


def _exact_tet(i, j, k):
    """Integral of l1^i l2^j l3^k over the reference tetrahedron (volume sqrt2 * 8 / 12 = 2 sqrt2 / 3)."""
    vol = abs(np.linalg.det(TV[1:] - TV[0])) / 6.0
    return 6.0 * vol * factorial(i) * factorial(j) * factorial(k) / factorial(i + j + k + 3)


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_volume_and_face_rules(p):
    sim = dg.Simulation(dg.Config(**_cfg(p)))   # kept alive while its operators are read
    o = _ops(sim)
    n_c, n_fc = o.n_c, o.n_fc
    assert n_c == {1: 4, 2: 14, 3: 24, 4: 125}[p] and n_fc == {1: 3, 2: 6, 3: 12, 4: 16}[p]
    l = _bary(_arr(o.rst_vc, 3 * n_c).reshape(n_c, 3))
    w = _arr(o.w_vc, n_c)
    strength = 2 * p if p <= 3 else 2 * p + 1
    for i, j, k in itertools.product(range(strength + 1), repeat=3):
        if i + j + k <= strength:
            assert abs(np.sum(w * l[:, 1] ** i * l[:, 2] ** j * l[:, 3] ** k) - _exact_tet(i, j, k)) <= 1e-14
    wf = _arr(o.w_fc, n_fc)
    xf = _arr(o.rst_fc, 4 * n_fc * 3).reshape(4, n_fc, 3)
    for f in range(4):
        lf = _bary(xf[f])[:, list(FVE[f])]                 # barycentric in the face's own vertex order
        assert np.max(np.abs(_bary(xf[f])[:, f])) <= 1e-15  # on the face opposite vertex f
        for perm in itertools.permutations(range(3)):       # the point set is invariant under the face's symmetries
            lp = lf[:, list(perm)]
            for q in range(n_fc):
                assert np.min(np.linalg.norm(lf - lp[q], axis=1)) <= 1e-14
        for i, j in itertools.product(range(2 * p + 1), repeat=2):   # area of the face: sqrt3
            if i + j <= 2 * p:
                exact = S3 * 2.0 * factorial(i) * factorial(j) / factorial(i + j + 2)
                assert abs(np.sum(wf * lf[:, 0] ** i * lf[:, 1] ** j) - exact) <= 1e-15


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_oracle_set_up_gives_the_library_residual(p):
    cfg = _cfg(p)
    sim = dg.Simulation(dg.Config(**cfg))
    own = Oracle(Problem(**cfg))
    u = sim.sol_coef()
    assert np.max(np.abs(own.initial_solution() - u)) <= 1e-14
    _, r1 = own.compute_rhs(u)
    _, r2 = Oracle(data_model=dg.load_library().dpg_sim_view(sim.handle)).compute_rhs(u)
    assert np.max(np.abs(r1 - r2)) <= 5e-12 * np.max(np.abs(r1))
    for orc in (own, Oracle(data_model=dg.load_library().dpg_sim_view(sim.handle))):
        m, _ = orc.compute_rhs(np.full(orc.n_dof, 1.3))
        assert m <= 1e-11


def test_mixed_orders():
    cfg = _cfg(1, p_max=4, p_seed=4)
    sim = dg.Simulation(dg.Config(**cfg))
    s = C.cast(sim.handle, C.POINTER(L.DpgSim)).contents
    assert len(set(_arr(s.vol_p, sim.n_vol).astype(int))) == 4
    own = Oracle(Problem(**cfg))
    u = sim.sol_coef()
    _, r1 = own.compute_rhs(u)
    _, r2 = Oracle(data_model=dg.load_library().dpg_sim_view(sim.handle)).compute_rhs(u)
    assert np.max(np.abs(r1 - r2)) <= 5e-12 * np.max(np.abs(r1))


@pytest.mark.parametrize("p", [1, 2, 3])
def test_convergence_order(p):
    errs = []
    for n in (6, 12):
        sim = dg.Simulation(dg.Config(**_cfg(p, (n, n, n))))
        orc = Oracle(data_model=dg.load_library().dpg_sim_view(sim.handle), threads=8)
        u = sim.sol_coef()
        tf = 0.05
        dt = 0.1 * (1.0 / n) / (1.2 * (2 * p + 1))
        ns = int(np.ceil(tf / dt))
        orc.rk_step(u, tf / ns, ns)
        sim.set_sol_coef(u)
        errs.append(sim.l2_error(tf)[0])
    order = np.log2(errs[0] / errs[1])
    assert order >= p + 1 - 0.165, (errs, order)


def test_refusals():
    with pytest.raises(dg.DpgError) as e:   # orders above 4: no face rule of that strength
        dg.Simulation(dg.Config(**_cfg(5)))
    assert e.value.status == dg.api.DPG_ERR_UNSUPPORTED
    with pytest.raises(dg.DpgError) as e:   # boundary faces: the TET meshes are periodic boxes
        dg.Simulation(dg.Config(**dict(_cfg(2), pde="euler", num_flux="Roe-Pike", test_case="isentropic_vortex",
                                       bc=("slipwall",) * 6)))
    assert e.value.status == dg.api.DPG_ERR_UNSUPPORTED


@pytest.mark.parametrize("p", [1, 3])
def test_gmsh_tetrahedral_meshes(tmp_path, p):
    """A gmsh file of the same split mesh with permuted vertex lists (some negatively oriented), shuffled node
    numbers and $Periodic pairs gives the residual of the structured TET mesh (volumes matched by their solution
    nodes), and the oracle's own reader of the file gives the library's residual."""
    from gmsh_writer import write_tet_msh
    from tests_support import match_volumes, remap_state
    msh = str(tmp_path / "tet.msh")
    write_tet_msh(msh, (3, 2, 2), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), rotate_seed=2, shuffle_seed=5)
    cfg = dg.Config(**_cfg(p, (3, 2, 2), jitter=0.0))
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
    assert np.max(np.abs(r_own - r_msh)) <= 5e-12 * np.max(np.abs(r_msh))
