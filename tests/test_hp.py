"""Mixed orders (hp meshes): each volume's order drawn uniformly from p .. p_max by a seed, a face of the larger
order of its two volumes (compute_face_reference_order, face_solver.c:123-132) with the cubature of that order and
the lower-order volume's basis interpolated to it (cv0_vs_fc[p_f][p], compute_face_rlhs_T.c:67-80).  CPU checks:

- the oracle's own mixed-order set-up (its own bases, cubature, geometry and draws) equals the library's: orders,
  face orders, operators, metrics, normals and node correspondences (1e-13), residuals (1e-12);
- a face operator of a higher face order interpolates every polynomial of the volume's order exactly;
- constant states are preserved; the residual conserves the advected quantity (the sum of the unscaled residual over
  all basis functions vanishes on a periodic mesh);
- the L2 error converges at order >= p_min + 1 - 0.165 (the reference's criterion,
  test_integration_convergence_support.c:49) with orders drawn from {p_min, p_min + 1} on jittered meshes.
"""
import ctypes as C

import numpy as np
import pytest

import dpgsolver_gb300 as dg
from oracle import Oracle, Problem
from oracle import oracle_layout as L
from tests_support import DpgSim


def _cfg(element, p, p_max, n, jitter=0.1, seed=3, p_seed=11):
    return dict(d=2, p=p, p_max=p_max, p_seed=p_seed, n_elem=(n[0], n[1], 1), element=element, pde="advection",
                num_flux="upwind", test_case="advection_sine", lo=(0, 0, 0), hi=(1, 1, 1), jitter=jitter, seed=seed,
                b_adv=(1.0, 0.5, 0.0))


def _model(addr):
    return L.model(addr)


def _ints(ptr, n):
    return np.ctypeslib.as_array(ptr, shape=(n,)).copy()


def _dbl(ptr, n):
    return np.ctypeslib.as_array(ptr, shape=(n,)).copy()


@pytest.mark.parametrize("element,n", [("tri", (6, 5)), ("tp", (5, 4))])
def test_oracle_set_up_equals_the_library_set_up(element, n):
    cfg = dg.Config(**_cfg(element, 1, 4, n))
    sim = dg.Simulation(cfg)
    orc = Oracle(Problem(**_cfg(element, 1, 4, n)))
    a, b = _model(orc.model), C.cast(sim.handle, C.POINTER(L.DpgSim)).contents
    nv, nf = b.n_vol, b.n_face
    assert (a.n_vol, a.n_face, a.n_ops) == (nv, nf, b.n_ops) == (nv, nf, 4)
    assert np.array_equal(_ints(a.vol_p, nv), _ints(b.vol_p, nv))
    assert len(set(_ints(b.vol_p, nv))) == 4   # every order present
    assert np.array_equal(_ints(a.face_p, nf), _ints(b.face_p, nf))
    assert np.array_equal(_ints(a.face_nfc, nf), _ints(b.face_nfc, nf))
    n_fnode = int(b.face_geo_off[nf])
    n_geo = int(b.vol_geo_off[nv])
    assert np.array_equal(_ints(a.nc_fc, n_fnode), _ints(b.nc_fc, n_fnode))
    fields = [("normals_fc", 2 * n_fnode), ("jacobian_det_fc", n_fnode)]
    if element == "tp":   # the same volume cubature (TRI: the two set-ups use different exact rules)
        fields += [("metrics_vc", 4 * n_geo), ("jacobian_det_vc", n_geo)]
    for name, size in fields:
        x, y = _dbl(getattr(a, name), size), _dbl(getattr(b, name), size)
        assert np.max(np.abs(x - y)) <= 1e-13 * max(1.0, np.max(np.abs(y))), name
    for k in range(4):
        oa, ob = a.ops[k], b.ops[k]
        for pf in range(ob.p + 1, 5):
            na = ob.n_fl * b.ops[pf - 1].n_fc * ob.n_s
            assert bool(oa.cv0_vs_fcp[pf]) == bool(ob.cv0_vs_fcp[pf]), (k, pf)
            if ob.cv0_vs_fcp[pf]:
                for fld in ("cv0_vs_fcp", "tw0_vt_fcp"):
                    x, y = _dbl(getattr(oa, fld)[pf], na), _dbl(getattr(ob, fld)[pf], na)
                    assert np.max(np.abs(x - y)) <= 1e-13 * max(1.0, np.max(np.abs(y))), (fld, k, pf)
    u = sim.sol_coef()
    assert np.max(np.abs(orc.initial_solution() - u)) <= 1e-13
    _, r1 = orc.compute_rhs(u)
    _, r2 = Oracle(data_model=dg.load_library().dpg_sim_view(sim.handle)).compute_rhs(u)
    assert np.max(np.abs(r1 - r2)) <= 1e-12 * np.max(np.abs(r1))


@pytest.mark.parametrize("element", ["tri", "tp"])
def test_higher_order_face_operators_interpolate_exactly(element):
    sim = dg.Simulation(dg.Config(**_cfg(element, 1, 4, (6, 5))))
    s = C.cast(sim.handle, C.POINTER(L.DpgSim)).contents
    rng = np.random.default_rng(5)
    for k in range(s.n_ops):
        ov = s.ops[k]
        n_s, p = ov.n_s, ov.p
        xs = _dbl(ov.rst_vs, 2 * n_s).reshape(n_s, 2)
        # a random polynomial of total degree <= p (TRI) or degree <= p per direction (tensor product)
        terms = [(i, j) for i in range(p + 1) for j in range(p + 1) if element == "tp" or i + j <= p]
        coef = rng.standard_normal(len(terms))
        poly = lambda x: sum(c * x[:, 0] ** i * x[:, 1] ** j for c, (i, j) in zip(coef, terms))
        for pf in range(p + 1, 5):
            if not ov.cv0_vs_fcp[pf]:
                continue
            of = s.ops[pf - s.ops[0].p]
            n_pt = of.n_fl * of.n_fc
            xf = _dbl(of.rst_fc, 2 * n_pt).reshape(n_pt, 2)
            cv = _dbl(ov.cv0_vs_fcp[pf], n_pt * n_s).reshape(n_pt, n_s)
            assert np.max(np.abs(cv @ poly(xs) - poly(xf))) <= 1e-12 * max(1.0, np.max(np.abs(poly(xf))))


@pytest.mark.parametrize("element", ["tri", "tp"])
def test_free_stream_and_conservation(element):
    cfg = _cfg(element, 1, 4, (6, 5))
    orc = Oracle(Problem(**cfg))
    m, _ = orc.compute_rhs(np.full(orc.n_dof, 1.7))
    assert m <= 1e-11
    u = orc.initial_solution() + 0.1 * np.random.default_rng(2).standard_normal(orc.n_dof)
    _, r = orc.compute_rhs_unscaled(u)
    _, rs = orc.compute_rhs(u)
    assert abs(np.sum(r)) <= 1e-13 * np.sum(np.abs(r)) * 10, (np.sum(r), np.sum(np.abs(r)))
    assert np.max(np.abs(rs)) > 1e-3


@pytest.mark.parametrize("element,p", [("tri", 1), ("tri", 2), ("tp", 1), ("tp", 2)])
def test_convergence_order_with_mixed_orders(element, p):
    errs = []
    for n in (8, 16):
        orc = Oracle(Problem(**_cfg(element, p, p + 1, (n, n))), threads=8)
        u = orc.initial_solution()
        tf = 0.1
        dt = 0.1 * (1.0 / n) / (1.2 * (2 * (p + 1) + 1))
        ns = int(np.ceil(tf / dt))
        orc.rk_step(u, tf / ns, ns)
        errs.append(orc.l2_error(u, tf)[0])
    order = np.log2(errs[0] / errs[1])
    assert order >= p + 1 - 0.165, (errs, order)


def test_mixed_orders_are_refused_outside_periodic_advection_and_euler():
    for kw in (dict(pde="euler", num_flux="Roe-Pike", test_case="isentropic_vortex", bc=("slipwall",) * 4),):
        cfg = dg.Config(**dict(_cfg("tp", 1, 3, (4, 4)), **kw))
        with pytest.raises(dg.DpgError) as e:
            dg.Simulation(cfg)
        assert e.value.status == dg.api.DPG_ERR_UNSUPPORTED
    with pytest.raises(dg.DpgError) as e:
        dg.Simulation(dg.Config(**_cfg("tp", 1, 9, (4, 4))))
    assert e.value.status == dg.api.DPG_ERR_INVALID


def test_hex_mixed_orders():
    """HEX meshes of orders 1..3: the oracle's own set-up gives the library's residual; free stream preserved."""
    kw = dict(d=3, p=1, p_max=3, p_seed=4, n_elem=(3, 3, 2), lo=(0, 0, 0), hi=(1, 1, 1), pde="advection",
              num_flux="upwind", test_case="advection_sine", jitter=0.1, seed=3, b_adv=(1.0, 0.5, 0.25))
    sim = dg.Simulation(dg.Config(**kw))
    orc = Oracle(Problem(**kw))
    u = sim.sol_coef()
    assert np.max(np.abs(orc.initial_solution() - u)) <= 1e-13
    _, r1 = orc.compute_rhs(u)
    _, r2 = Oracle(data_model=dg.load_library().dpg_sim_view(sim.handle)).compute_rhs(u)
    assert np.max(np.abs(r1 - r2)) <= 1e-12 * np.max(np.abs(r1))
    m, _ = orc.compute_rhs(np.full(orc.n_dof, 1.3))
    assert m <= 1e-11
