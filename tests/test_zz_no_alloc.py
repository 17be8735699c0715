"""The allocation-free residual entry point, dpg_gpu_compute_rhs_noalloc, against dpg_gpu_compute_rhs.

Callers that may not allocate device memory while they run (a memory manager owns every device allocation, or a
real-time loop cannot afford cudaMalloc's implicit synchronisation) pass every input and output as device pointers;
the library keeps its face traces and face fluxes in a fixed, statically declared scratch array.  This file is
collected last so that a failure here does not hide the results of the other tests.  The device buffers below are
allocated by the test (through torch), never by the entry point.
"""
import ctypes as C

import numpy as np
import pytest

import dpgsolver_gb300 as dg
from tests_support import sim_arrays

pytestmark = pytest.mark.gpu

TOL = 1e-11   # same FP64 parity bound as the other FP64 tests (rounding-order differences only)
SCRATCH_DOUBLES = 1 << 21


class NoallocMesh(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("d", "n_var", "num_flux", "n_vol", "n_face", "n_s", "n_c", "n_fl", "n_fc")] + [
        (n, C.c_void_p) for n in ("cv0_vs_vc", "cv0_vs_fc", "lift", "metrics", "jinv", "minv", "vol_face", "nc_fc",
                                  "nc_fc_inv", "normals_fc", "jacobian_det_fc")] + [("b_adv", C.c_double * 3)]


def _entry():
    lib = dg.load_library()
    fn = lib.dpg_gpu_compute_rhs_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.POINTER(NoallocMesh), C.c_void_p, C.c_void_p, C.POINTER(C.c_double), C.c_void_p]
    return fn


def _device_mesh(sim, cfg, torch):
    """Device copies of the operators, geometry and connectivity in the layout the entry point documents."""
    a = sim_arrays(sim)
    d, n_s, n_c, n_fl, n_fc = sim.d, sim.n_s, sim.n_c, a["n_fl"], sim.n_fc
    K = d * n_c + n_fl * n_fc
    lift = np.zeros((n_s, K))
    for r in range(d):
        lift[:, r * n_c:(r + 1) * n_c] = a["tw1_vt_vc"][r]
    for lf in range(n_fl):
        lift[:, d * n_c + lf * n_fc: d * n_c + (lf + 1) * n_fc] = -a["tw0_vt_fc"][lf]
    affine = bool(a["vol_affine"].all())
    jdet = a["jacobian_det_vc"].reshape(sim.n_vol, n_c)
    if affine:   # one metric block and 1/detJ per volume, the lift pre-multiplied by the reference mass inverse
        lift = a["m_inv_ref"] @ lift
        met = np.ascontiguousarray(a["metrics_vc"][:, :, 0])
        jinv, minv = 1.0 / jdet[:, 0], None
    else:        # per-node metrics and per-volume mass inverses (cv0^T diag(w detJ) cv0)^-1
        met = np.ascontiguousarray(a["metrics_vc"])
        cv0, w = a["cv0_vs_vc"], a["w_vc"]
        minv = np.stack([np.linalg.inv(cv0.T @ (cv0 * (w * jdet[e])[:, None])) for e in range(sim.n_vol)])
        jinv = None
    vol_face = (a["vol_face"][:, :n_fl] << 1) | a["vol_face_side"][:, :n_fl]
    nc = a["nc_fc"].reshape(sim.n_face, n_fc)
    nc_inv = np.empty_like(nc)
    rows = np.arange(sim.n_face)[:, None]
    nc_inv[rows, nc] = np.arange(n_fc)[None, :]
    keep = []

    def dev(x, dtype):
        t = torch.from_numpy(np.ascontiguousarray(x, dtype=dtype)).cuda()
        keep.append(t)
        return t.data_ptr()

    m = NoallocMesh()
    m.d, m.n_var, m.num_flux = d, sim.n_var, {"Roe-Pike": 31, "Lax-Friedrichs": 32, "upwind": 11}[cfg.num_flux]
    m.n_vol, m.n_face, m.n_s, m.n_c, m.n_fl, m.n_fc = sim.n_vol, sim.n_face, n_s, n_c, n_fl, n_fc
    m.cv0_vs_vc = dev(a["cv0_vs_vc"], np.float64)
    m.cv0_vs_fc = dev(a["cv0_vs_fc"], np.float64)
    m.lift = dev(lift, np.float64)
    m.metrics = dev(met, np.float64)
    m.jinv = dev(jinv, np.float64) if jinv is not None else None
    m.minv = dev(minv, np.float64) if minv is not None else None
    m.vol_face = dev(vol_face, np.int32)
    m.nc_fc = dev(nc, np.int32)
    m.nc_fc_inv = dev(nc_inv, np.int32)
    m.normals_fc = dev(a["normals_fc"], np.float64)
    m.jacobian_det_fc = dev(a["jacobian_det_fc"], np.float64)
    for i in range(3):
        m.b_adv[i] = cfg.b_adv[i]
    return m, keep


@pytest.mark.parametrize("cfg", [dg.Config(d=2, p=2, n_elem=(8, 8, 1)),
                                 dg.Config(d=3, p=2, n_elem=(4, 4, 3), num_flux="Lax-Friedrichs"),
                                 dg.Config(d=2, p=3, n_elem=(6, 5, 1), jitter=0.15, seed=4)],
                         ids=["quad-p2-roe", "hex-p2-lf", "quad-p3-jittered-minv"])
def test_noalloc_matches_compute_rhs_twice(cfg):
    torch = pytest.importorskip("torch")
    sim = dg.Simulation(cfg)
    ctx = dg.GpuContext(sim)
    mesh, keep = _device_mesh(sim, cfg, torch)
    fn = _entry()
    rng = np.random.default_rng(3)
    u0 = sim.sol_coef()
    for call in range(2):   # two calls in a row: the shared scratch keeps the previous call's contents
        sol = u0 * (1.0 + 1e-2 * call * rng.standard_normal(u0.shape))
        ctx.upload(sol)
        m_ref = ctx.compute_rhs()
        rhs_ref = ctx.rhs()
        d_sol = torch.from_numpy(sol).cuda()
        d_rhs = torch.full_like(d_sol, float("nan"))
        torch.cuda.synchronize()
        mx = C.c_double(-1.0)
        rc = fn(C.byref(mesh), d_sol.data_ptr(), d_rhs.data_ptr(), C.byref(mx), None)
        assert rc == 0, dg.load_library().dpg_status_string(rc)
        rhs = d_rhs.cpu().numpy()
        err = np.max(np.abs(rhs - rhs_ref)) / np.max(np.abs(rhs_ref))
        assert err <= TOL, (call, err)
        assert abs(mx.value - m_ref) <= TOL * m_ref
    del keep


def test_noalloc_rejects_problems_beyond_the_scratch():
    fn = _entry()
    m = NoallocMesh()
    m.d, m.n_var, m.num_flux = 3, 5, 31
    m.n_vol, m.n_s, m.n_c, m.n_fl, m.n_fc = 1, 8, 8, 6, 4
    m.n_face = SCRATCH_DOUBLES // (3 * 5 * 4) + 1
    for name in ("cv0_vs_vc", "cv0_vs_fc", "lift", "metrics", "jinv", "vol_face", "nc_fc", "nc_fc_inv",
                 "normals_fc", "jacobian_det_fc"):
        setattr(m, name, 16)   # never dereferenced: the size check comes first
    rc = fn(C.byref(m), 16, 16, None, None)
    assert rc == 9  # DPG_ERR_TOO_LARGE
