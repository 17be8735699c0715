"""ctypes mirror of the host data model of include/dpg_simulation.h (test infrastructure only).

Reads the sizes and arrays of a data model at a given address -- the oracle's own set-up or the library's -- so
that tests can compare the two entry by entry.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

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
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


def model(addr: int) -> DpgSim:
    return C.cast(C.c_void_p(addr), C.POINTER(DpgSim)).contents


def read(addr: int) -> dict:
    s = model(addr)
    return {"d": s.d, "n_var": s.n_var, "n_vol": s.n_vol, "n_face": s.n_face,
            "n_dof": int(s.vol_dof_off[s.n_vol]), "n_s": s.ops[0].n_s, "n_c": s.ops[0].n_c,
            "n_fc": s.ops[0].n_fc, "n_fl": s.ops[0].n_fl, "p": s.ops[0].p}


def arrays(addr: int) -> dict:
    """Operators (single element group), per-volume geometry, faces and the initial state as numpy arrays."""
    s = model(addr)
    o = s.ops[0]
    d, nv, nf = s.d, s.n_vol, s.n_face
    n_s, n_c, n_fl, n_fc = o.n_s, o.n_c, o.n_fl, o.n_fc
    return {
        "rst_vs": _arr(o.rst_vs, n_s * d).reshape(n_s, d),
        "rst_vc": _arr(o.rst_vc, n_c * d).reshape(n_c, d),
        "w_vc": _arr(o.w_vc, n_c),
        "w_fc": _arr(o.w_fc, n_fc),
        "rst_fc": _arr(o.rst_fc, n_fl * n_fc * d).reshape(n_fl, n_fc, d),
        "cv0_vs_vc": _arr(o.cv0_vs_vc, n_c * n_s).reshape(n_c, n_s),
        "tw1_vt_vc": _arr(o.tw1_vt_vc, d * n_s * n_c).reshape(d, n_s, n_c),
        "cv0_vs_fc": _arr(o.cv0_vs_fc, n_fl * n_fc * n_s).reshape(n_fl, n_fc, n_s),
        "tw0_vt_fc": _arr(o.tw0_vt_fc, n_fl * n_s * n_fc).reshape(n_fl, n_s, n_fc),
        "xyz_ve": _arr(s.xyz_ve, nv * 8 * 3).reshape(nv, 8, 3),
        "metrics_vc": _arr(s.metrics_vc, nv * n_c * d * d).reshape(nv, d * d, n_c),
        "jacobian_det_vc": _arr(s.jacobian_det_vc, nv * n_c).reshape(nv, n_c),
        "xyz_vc": _arr(s.xyz_vc, nv * n_c * d).reshape(nv, d, n_c),
        "sol_coef": _arr(s.sol_coef, int(s.vol_dof_off[nv])),
        "face_vol": _arr(s.face_vol, 2 * nf, np.int32).reshape(nf, 2),
        "face_lf": _arr(s.face_lf, 2 * nf, np.int32).reshape(nf, 2),
        "face_bc": _arr(s.face_bc, nf, np.int32),
        "nc_fc": _arr(s.nc_fc, nf * n_fc, np.int32).reshape(nf, n_fc),
        "normals_fc": _arr(s.normals_fc, nf * n_fc * d).reshape(nf, n_fc, d),
        "jacobian_det_fc": _arr(s.jacobian_det_fc, nf * n_fc).reshape(nf, n_fc),
        "xyz_fc": _arr(s.xyz_fc, nf * n_fc * d).reshape(nf, d, n_fc),
        "domain_lo": np.array(s.domain_lo[:]), "domain_hi": np.array(s.domain_hi[:]),
    }
