"""ctypes mirror of include/dpg_simulation.h so that tests can read the host data model."""
import ctypes as C

import numpy as np

import dpgsolver_gb300 as dg

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)
lp = C.POINTER(C.c_int64)


class ElementOps(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("e_type", "d", "p", "n_s", "n_c", "n_fl", "n_fc", "n_ve")] + [
        (n, dp) for n in ("rst_vs", "rst_vc", "w_vc", "rst_fc", "w_fc", "normals_ref", "cv0_vs_vc", "tw1_vt_vc",
                          "cv0_vs_fc", "tw0_vt_fc", "cv0_vv_vc", "cv1_vv_vc", "cv0_vv_fc", "cv1_vv_fc", "m_inv_ref",
                          "ccBS0_vs_vs", "ccSB0_vs_vs", "bez1", "bez1_inv")] + [
        ("cv0_vs_fcp", dp * 9), ("tw0_vt_fcp", dp * 9)]


class DpgSim(C.Structure):
    _fields_ = [
        ("d", C.c_int), ("pde_index", C.c_int), ("n_var", C.c_int), ("n_eq", C.c_int), ("ind_num_flux", C.c_int * 2),
        ("solver_proc", C.c_int), ("solver_type_e", C.c_int), ("solver_type_i", C.c_int), ("test_case", C.c_int),
        ("dt", C.c_double), ("time", C.c_double), ("time_final", C.c_double), ("b_adv", C.c_double * 3),
        ("vortex", C.c_double * 8), ("domain_lo", C.c_double * 3), ("domain_hi", C.c_double * 3),
        ("n_ops", C.c_int), ("ops", C.POINTER(ElementOps)),
        ("n_vol", C.c_int), ("vol_ops", ip), ("vol_p", ip), ("vol_affine", ip), ("vol_dof_off", lp),
        ("vol_geo_off", lp), ("vol_minv_off", lp), ("xyz_ve", dp), ("sol_coef", dp), ("sol_coef_p", dp), ("rhs", dp),
        ("metrics_vc", dp), ("jacobian_det_vc", dp), ("xyz_vc", dp), ("m_inv", dp), ("vol_face", ip),
        ("vol_face_side", ip),
        ("n_face", C.c_int), ("face_vol", ip), ("face_lf", ip), ("face_nfc", ip), ("face_bc", ip), ("face_geo_off", lp),
        ("nc_fc", ip), ("normals_fc", dp), ("jacobian_det_fc", dp), ("xyz_fc", dp),
        ("geom", C.c_int), ("mu", C.c_double), ("Pr", C.c_double), ("r_s", C.c_double), ("bc_omega", C.c_double),
        ("bc_rho", C.c_double), ("bc_E", C.c_double), ("bc_state", C.c_double * 5), ("tc_data", C.c_double * 4),
        ("face_p", ip),
    ]


def _arr(ptr, n, dtype=np.float64):
    if not ptr:   # operators an element type does not form (the TRI's Bezier operators)
        return None
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


def _mat(ptr, r, c):
    a = _arr(ptr, r * c)
    return None if a is None else a.reshape(r, c)


def sim_arrays(sim):
    s = C.cast(sim.handle, C.POINTER(DpgSim)).contents
    d, nf, nfc = s.d, s.n_face, sim.n_fc
    ops = s.ops[0]
    n_s, n_c, n_fl = ops.n_s, ops.n_c, ops.n_fl
    return {
        "n_fl": n_fl,
        "cv0_vs_fc": _arr(ops.cv0_vs_fc, n_fl * nfc * n_s).reshape(n_fl * nfc, n_s),
        "tw1_vt_vc": _arr(ops.tw1_vt_vc, d * n_s * n_c).reshape(d, n_s, n_c),
        "tw0_vt_fc": _arr(ops.tw0_vt_fc, n_fl * n_s * nfc).reshape(n_fl, n_s, nfc),
        "metrics_vc": _arr(s.metrics_vc, s.n_vol * n_c * d * d).reshape(s.n_vol, d * d, n_c),
        "vol_face": _arr(s.vol_face, s.n_vol * 6, np.int32).reshape(s.n_vol, 6),
        "vol_face_side": _arr(s.vol_face_side, s.n_vol * 6, np.int32).reshape(s.n_vol, 6),
        "d": d,
        "normals_fc": _arr(s.normals_fc, nf * nfc * d).reshape(nf * nfc, d),
        "jacobian_det_fc": _arr(s.jacobian_det_fc, nf * nfc),
        "jacobian_det_vc": _arr(s.jacobian_det_vc, s.n_vol * sim.n_c),
        "vol_affine": _arr(s.vol_affine, s.n_vol, np.int32),
        "nc_fc": _arr(s.nc_fc, nf * nfc, np.int32),
        "w_vc": _arr(ops.w_vc, ops.n_c),
        "cv0_vs_vc": _arr(ops.cv0_vs_vc, ops.n_c * ops.n_s).reshape(ops.n_c, ops.n_s),
        "m_inv_ref": _arr(ops.m_inv_ref, ops.n_s * ops.n_s).reshape(ops.n_s, ops.n_s),
        "rst_vs": _arr(ops.rst_vs, ops.n_s * d).reshape(ops.n_s, d),
        "ccBS0_vs_vs": _mat(ops.ccBS0_vs_vs, ops.n_s, ops.n_s),
        "ccSB0_vs_vs": _mat(ops.ccSB0_vs_vs, ops.n_s, ops.n_s),
        "bez1": _mat(ops.bez1, ops.p + 1, ops.p + 1),
        "bez1_inv": _mat(ops.bez1_inv, ops.p + 1, ops.p + 1),
        "p": ops.p,
    }


def solution_node_xyz(sim):
    """Physical coordinates [n_vol, n_s, d] of every volume's solution nodes (P1 map of the tensor-product vertices
    at the reference nodes rst_vs)."""
    s = C.cast(sim.handle, C.POINTER(DpgSim)).contents
    a = sim_arrays(sim)
    d, n_vol = s.d, s.n_vol
    r = a["rst_vs"]                                          # [n_s, d]
    if s.ops[0].n_ve == 3:   # TRI: barycentric coordinates on the reference triangle (-1,-1/sqrt3), (1,-1/sqrt3), (0,2/sqrt3)
        xyz_ve = _arr(s.xyz_ve, n_vol * 8 * 3).reshape(n_vol, 8, 3)[:, :3, :2]
        l2 = (np.sqrt(3.0) * r[:, 1] + 1.0) / 3.0
        l1 = (r[:, 0] + 1.0 - l2) / 2.0
        phi = np.stack([1.0 - l1 - l2, l1, l2], axis=1)
        return np.einsum("sk,vkd->vsd", phi, xyz_ve)
    if s.ops[0].n_ve == 4 and d == 3:   # TET: barycentric coordinates on the reference tetrahedron
        s3, s6 = np.sqrt(3.0), np.sqrt(6.0)
        tv = np.array([[-1.0, -1 / s3, -1 / s6], [1.0, -1 / s3, -1 / s6], [0.0, 2 / s3, -1 / s6], [0.0, 0.0, 3 / s6]])
        l123 = np.linalg.solve((tv[1:] - tv[0]).T, (r - tv[0]).T).T
        phi = np.column_stack([1.0 - l123.sum(axis=1), l123])
        xyz_ve = _arr(s.xyz_ve, n_vol * 8 * 3).reshape(n_vol, 8, 3)[:, :4, :]
        return np.einsum("sk,vkd->vsd", phi, xyz_ve)
    xyz_ve = _arr(s.xyz_ve, n_vol * 8 * 3).reshape(n_vol, 8, 3)[:, : 1 << d, :d]
    phi = np.ones((r.shape[0], 1 << d))
    for k in range(1 << d):
        for b in range(d):
            sgn = 1.0 if (k >> b) & 1 else -1.0
            phi[:, k] *= 0.5 * (1.0 + sgn * r[:, b])
    return np.einsum("sk,vkd->vsd", phi, xyz_ve)


def match_volumes(sim_a, sim_b, tol=1e-9):
    """For two meshes of the same domain: for each volume of a, the volume of b with the same solution nodes and the
    permutation of b's nodes onto a's (index arrays [n_vol], [n_vol, n_s])."""
    xa, xb = solution_node_xyz(sim_a), solution_node_xyz(sim_b)
    ca, cb = xa.mean(axis=1), xb.mean(axis=1)
    vol = np.empty(xa.shape[0], int)
    perm = np.empty(xa.shape[:2], int)
    for v in range(xa.shape[0]):
        w = int(np.argmin(np.linalg.norm(cb - ca[v], axis=1)))
        dist = np.linalg.norm(xa[v][:, None, :] - xb[w][None, :, :], axis=2)
        p = np.argmin(dist, axis=1)
        assert np.max(dist[np.arange(dist.shape[0]), p]) <= tol and len(set(p.tolist())) == dist.shape[0]
        vol[v], perm[v] = w, p
    return vol, perm


def remap_state(sim_a, sim_b, u_b, vol, perm):
    """A state of mesh b in mesh a's volume and node order."""
    ub = u_b.reshape(sim_b.n_vol, sim_b.n_var, sim_b.n_s)
    return ub[vol[:, None], :, perm].transpose(0, 2, 1).reshape(-1).copy()


def wv_rule(kind, strength):
    """The reference's Witherden-Vincent rule (input/nodes/<kind>/WV<strength>.txt, from the golden fixture) with its
    orbits expanded: [n][d + 2] barycentric points and weights summing to 1."""
    import itertools
    import json
    import os
    g = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                    "reference_goldens.json")))["wv_rules"][kind][str(strength)]
    rows = [list(perm) + [w] for b, w in zip(g["bary"], g["w"]) for perm in sorted(set(itertools.permutations(b)))]
    a = np.array(rows)
    a[:, -1] /= a[:, -1].sum()
    return a


def oracle_rules(element, p, sim=None):
    """Cubature of the oracle's own simplex set-up for the Euler equations (whose integrands are not polynomial, so
    the rule is part of the discretisation): the reference's WV rules of strength 2p -- volumes of TRI p <= 4 and
    TET p <= 3, TET faces p <= 4; TET p = 4 volumes take the library's collapsed rule (no WV rule derived for it)."""
    kw = {}
    if element == "tri" or p <= 3:
        kw["vol_rules"] = {p: wv_rule(element, 2 * p)}
    elif sim is not None:
        o = C.cast(sim.handle, C.POINTER(DpgSim)).contents.ops[0]
        x = _arr(o.rst_vc, 3 * o.n_c).reshape(o.n_c, 3)
        w = _arr(o.w_vc, o.n_c)
        s3, s6 = np.sqrt(3.0), np.sqrt(6.0)
        V = np.array([[-1.0, -1 / s3, -1 / s6], [1.0, -1 / s3, -1 / s6], [0.0, 2 / s3, -1 / s6], [0.0, 0.0, 3 / s6]])
        l123 = np.linalg.solve((V[1:] - V[0]).T, (x - V[0]).T).T
        kw["vol_rules"] = {p: np.column_stack([1 - l123.sum(axis=1), l123, w / w.sum()])}
    if element == "tet":
        kw["face_rules"] = {p: wv_rule("tri", 2 * p)}
    return kw
