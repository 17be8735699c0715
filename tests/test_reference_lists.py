"""dpg_sim_create_from_lists: the data model from the reference's own volume and face lists (struct Volume::xyz_ve,
struct Face::neigh_info[2].{volume, ind_lf}, Face::bc, Solver_Volume_T::sol_coef), as a binding reads them from the
reference's struct Simulation.

The lists are taken from simulations set up here (periodic boxes, jittered meshes, slip-wall and Riemann
boundaries), then renumbered -- volumes shuffled, faces shuffled, the sides of interior faces kept as the lists
give them -- as a reference mesh would number them.  The data model built from the lists must give the residual of
the original problem in the new numbering (the oracle's restatement on both; the face sums run in another order,
hence 1e-13), and bitwise the same data model when nothing is renumbered."""
import ctypes as C

import numpy as np
import pytest

import dpgsolver_gb300 as dg
from oracle import Oracle
from tests_support import DpgSim, sim_arrays

CASES = {
    "quad-p2-periodic": dict(d=2, p=2, n_elem=(4, 3, 1)),
    "quad-p3-jittered-walls": dict(d=2, p=3, n_elem=(4, 3, 1), lo=(0, 0, 0), hi=(2, 1, 1), jitter=0.1, seed=2,
                                   test_case="free_stream", vortex=(0, 0, 0, 1.0, 0.7, 0.3, 0, 1.0),
                                   bc=("riemann", "riemann", "slipwall", "riemann"), bc_state=(1.0, 0.7, 0.3, 0.0, 1.0)),
    "hex-p2-slip": dict(d=3, p=2, n_elem=(2, 3, 2), lo=(0, 0, 0), hi=(1, 1, 1), jitter=0.1, seed=3,
                        test_case="free_stream", vortex=(0, 0, 0, 1.0, 0.0, 0.3, 0.2, 1.0),
                        bc=("slipwall", "slipwall") + ("periodic",) * 4),
}


def _lists(sim):
    s = C.cast(sim.handle, C.POINTER(DpgSim)).contents
    d, n_vol, n_face = s.d, s.n_vol, s.n_face
    xyz = np.ctypeslib.as_array(s.xyz_ve, shape=(n_vol * 8 * 3,)).reshape(n_vol, 8, 3)[:, : 1 << d, :d].copy()
    fv = np.ctypeslib.as_array(s.face_vol, shape=(2 * n_face,)).reshape(n_face, 2).copy()
    fl = np.ctypeslib.as_array(s.face_lf, shape=(2 * n_face,)).reshape(n_face, 2).copy()
    fb = np.ctypeslib.as_array(s.face_bc, shape=(n_face,)).copy()
    return xyz, fv, fl, fb


@pytest.mark.parametrize("case", list(CASES.values()), ids=list(CASES))
def test_lists_give_the_same_data_model(case):
    cfg = dg.Config(**case)
    sim = dg.Simulation(cfg)
    xyz, fv, fl, fb = _lists(sim)
    u = sim.sol_coef() * (1.0 + 1e-3 * np.random.default_rng(1).standard_normal(sim.n_dof))
    got = dg.Simulation.from_reference_lists(cfg, xyz, fv, fl, fb, sol_coef=u)
    assert np.array_equal(got.sol_coef(), u)
    a, b = sim_arrays(sim), sim_arrays(got)
    for k in ("metrics_vc", "jacobian_det_vc", "normals_fc", "jacobian_det_fc", "nc_fc", "vol_face", "vol_face_side"):
        assert np.array_equal(a[k], b[k]), k
    _, r0 = Oracle(data_model=dg.load_library().dpg_sim_view(sim.handle)).compute_rhs(u)
    _, r1 = Oracle(data_model=dg.load_library().dpg_sim_view(got.handle)).compute_rhs(u)
    assert np.array_equal(r0, r1)


@pytest.mark.parametrize("case", list(CASES.values()), ids=list(CASES))
def test_renumbered_lists(case):
    cfg = dg.Config(**case)
    sim = dg.Simulation(cfg)
    xyz, fv, fl, fb = _lists(sim)
    rng = np.random.default_rng(5)
    new_of_old = rng.permutation(sim.n_vol)
    old_of_new = np.argsort(new_of_old)
    fperm = rng.permutation(sim.n_face)
    fv2 = np.where(fv >= 0, new_of_old[np.maximum(fv, 0)], -1)[fperm]
    u = sim.sol_coef() * (1.0 + 1e-3 * rng.standard_normal(sim.n_dof))
    ub = u.reshape(sim.n_vol, -1)
    got = dg.Simulation.from_reference_lists(cfg, xyz[old_of_new], fv2, fl[fperm], fb[fperm], sol_coef=ub[old_of_new])
    _, r0 = Oracle(data_model=dg.load_library().dpg_sim_view(sim.handle)).compute_rhs(u)
    _, r1 = Oracle(data_model=dg.load_library().dpg_sim_view(got.handle)).compute_rhs(got.sol_coef())
    r0b = r0.reshape(sim.n_vol, -1)[old_of_new].ravel()
    assert np.max(np.abs(r1 - r0b)) <= 1e-13 * np.max(np.abs(r0))


def test_inconsistent_lists_are_refused():
    cfg = dg.Config(**CASES["quad-p2-periodic"])
    sim = dg.Simulation(cfg)
    xyz, fv, fl, fb = _lists(sim)
    bad = fl.copy()
    bad[1] = bad[0]                       # two faces claim the same local faces
    bad_v = fv.copy()
    bad_v[1] = bad_v[0]
    with pytest.raises(dg.DpgError) as e:
        dg.Simulation.from_reference_lists(cfg, xyz, bad_v, bad, fb)
    assert e.value.status == dg.api.DPG_ERR_INVALID
    cfg_w = dg.Config(**CASES["quad-p3-jittered-walls"])
    sw = dg.Simulation(cfg_w)
    xyz, fv, fl, fb = _lists(sw)
    fb2 = fb.copy()
    fb2[fb2 != 0] = 10105                 # BC_SUPERSONIC_IN (straight): not on this path
    with pytest.raises(dg.DpgError) as e:
        dg.Simulation.from_reference_lists(cfg_w, xyz, fv, fl, fb2)
    assert e.value.status == dg.api.DPG_ERR_UNSUPPORTED
    fb3 = np.where(fb != 0, fb + 20000, 0)   # curved-boundary numbering (BC_CURVED_START): same conditions
    got = dg.Simulation.from_reference_lists(cfg_w, xyz, fv, fl, fb3)
    assert got.n_face == sw.n_face


def test_adapted_mesh_orders():
    """Solver_Volume_T::p_ref per volume (the orders of an adapted mesh) through the lists: a mixed-order advection
    mesh, renumbered, gives the residual of the original in the new numbering; orders out of range are refused, and
    mixed orders outside linear advection are refused."""
    cfg = dg.Config(d=2, p=1, p_max=4, p_seed=3, n_elem=(5, 4, 1), lo=(0, 0, 0), hi=(1, 1, 1), jitter=0.1, seed=2,
                    pde="advection", num_flux="upwind", test_case="advection_sine", b_adv=(1.0, 0.5, 0.0))
    sim = dg.Simulation(cfg)
    s = C.cast(sim.handle, C.POINTER(DpgSim)).contents
    vp = np.ctypeslib.as_array(s.vol_p, shape=(sim.n_vol,)).copy()
    off = np.ctypeslib.as_array(s.vol_dof_off, shape=(sim.n_vol + 1,)).copy()
    assert len(set(vp)) > 1
    xyz, fv, fl, fb = _lists(sim)
    rng = np.random.default_rng(7)
    new_of_old = rng.permutation(sim.n_vol)
    old_of_new = np.argsort(new_of_old)
    fperm = rng.permutation(sim.n_face)
    fv2 = np.where(fv >= 0, new_of_old[np.maximum(fv, 0)], -1)[fperm]
    u = sim.sol_coef() * (1.0 + 1e-3 * rng.standard_normal(sim.n_dof))
    blocks = [u[off[v]:off[v + 1]] for v in range(sim.n_vol)]
    base = dg.Config(**{**cfg.__dict__, "p_max": 0})
    got = dg.Simulation.from_reference_lists(base, xyz[old_of_new], fv2, fl[fperm], fb[fperm],
                                             sol_coef=[blocks[v] for v in old_of_new], p_ref=vp[old_of_new])
    assert got.n_dof == sim.n_dof
    _, r0 = Oracle(data_model=dg.load_library().dpg_sim_view(sim.handle)).compute_rhs(u)
    _, r1 = Oracle(data_model=dg.load_library().dpg_sim_view(got.handle)).compute_rhs(got.sol_coef())
    r0b = np.concatenate([r0[off[v]:off[v + 1]] for v in old_of_new])
    assert np.max(np.abs(r1 - r0b)) <= 1e-13 * np.max(np.abs(r0))
    bad = vp.copy()
    bad[0] = 9
    with pytest.raises(dg.DpgError) as e:
        dg.Simulation.from_reference_lists(base, xyz, fv, fl, fb, p_ref=bad)
    assert e.value.status == dg.api.DPG_ERR_INVALID
    euler = dg.Config(d=2, p=2, n_elem=(4, 3, 1))
    se = dg.Simulation(euler)
    xe, fve, fle, fbe = _lists(se)
    pe = np.full(se.n_vol, 2)
    pe[0] = 3
    mixed = dg.Simulation.from_reference_lists(euler, xe, fve, fle, fbe, p_ref=pe)   # Euler with adapted orders
    assert mixed.n_vol == se.n_vol and mixed.n_dof == se.n_dof + (16 - 9) * 4   # one QUAD of order 3
