"""ctypes binding of the C ABI in include/dpg_gb300.h.

This is the host-side mirror a Python caller uses; the work happens in ``lib/libdpg_gb300.so``.  Loading fails
loudly when the library has not been built: there is no Python or CPU fallback for the residual path.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libdpg_gb300.so")

# status codes (include/dpg_gb300.h)
DPG_OK = 0
DPG_ERR_INVALID = 1
DPG_ERR_UNSUPPORTED = 2
DPG_ERR_CUDA = 3
DPG_ERR_NONFINITE = 4
DPG_ERR_TIMEOUT = 5
DPG_ERR_NOT_CONVERGED = 6
DPG_ERR_NO_DEVICE = 7
DPG_ERR_IO = 8

# reference codes
TRI, QUAD, TET, HEX = 2, 3, 4, 5
PDE_ADVECTION, PDE_EULER, PDE_NAVIER_STOKES = 1, 3, 4
NUM_FLUX_UPWIND, NUM_FLUX_BR2_STABLE, NUM_FLUX_ROE_PIKE, NUM_FLUX_LAX_FRIEDRICHS = 11, 21, 31, 32
TC_ISENTROPIC_VORTEX, TC_ADVECTION_SINE, TC_FREE_STREAM, TC_TAYLOR_COUETTE, TC_PERIODIC_VORTEX = 1, 2, 3, 4, 5
BC_RIEMANN, BC_SLIPWALL, BC_NOSLIP_ADIABATIC, BC_NOSLIP_ALL_ROTATING = 101, 102, 111, 113
BC_CODES = {"periodic": 0, "riemann": BC_RIEMANN, "slipwall": BC_SLIPWALL, "noslip_adiabatic": BC_NOSLIP_ADIABATIC,
            "noslip_all_rotating": BC_NOSLIP_ALL_ROTATING}
MESH_BOX, MESH_ANNULUS = 0, 1

PREC_FP64, PREC_BF16X3, PREC_TF32X3, PREC_BF16_SLICED = 0, 1, 2, 3
PRECOND_NONE, PRECOND_BLOCK_JACOBI, PRECOND_MLP, PRECOND_BLOCK_ILU = 0, 1, 2, 3
ILU_ORDER_VOLUME, ILU_ORDER_COLOUR = 0, 1
JACOBIAN_TANGENT, JACOBIAN_FD = 0, 1

EXPORTED_SYMBOLS = [
    "dpg_status_string", "dpg_sim_params_default", "dpg_sim_create", "dpg_sim_create_from_ctrl",
    "dpg_sim_create_from_gmsh", "dpg_sim_create_from_lists", "dpg_sim_destroy", "dpg_sim_write_restart", "dpg_sim_read_restart",
    "dpg_sim_write_vtk",
    "dpg_sim_info", "dpg_sim_get_sol_coef", "dpg_sim_set_sol_coef", "dpg_sim_get_rhs", "dpg_sim_set_time",
    "dpg_sim_l2_error", "dpg_sim_max_wave_speed", "dpg_sim_view",
    "dpg_gpu_create", "dpg_gpu_destroy", "dpg_gpu_set_precision", "dpg_gpu_upload_sol_coef",
    "dpg_gpu_download_sol_coef", "dpg_gpu_download_rhs", "dpg_gpu_compute_rhs", "dpg_gpu_rk_step",
    "dpg_gpu_solve_explicit", "dpg_gpu_rk_step_host", "dpg_gpu_kernel_times", "dpg_gpu_launches_per_rhs",
    "dpg_gpu_time_rk_steps", "dpg_newton_params_default", "dpg_gpu_newton_solve", "dpg_gpu_mlp_enable",
    "dpg_gpu_mlp_train", "dpg_gpu_mlp_samples", "dpg_gpu_mlp_params", "dpg_gpu_mlp_loss_grad", "dpg_gpu_mlp_dims",
    "dpg_gpu_compute_rhs_noalloc", "dpg_gpu_jacobian_apply", "dpg_gpu_get_tiles", "dpg_gpu_set_tiles",
    "dpg_gpu_autotune", "dpg_gpu_set_positivity", "dpg_gpu_enforce_positivity", "dpg_gpu_positivity_update",
    "dpg_gpu_mlp_set_wait_limit",
]


class NewtonParams(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_newton", C.c_int), ("gmres_restart", C.c_int), ("max_gmres", C.c_int),
                ("gmres_rtol", C.c_double), ("dtau0", C.c_double), ("dtau_max", C.c_double), ("precond", C.c_int),
                ("collect_blocks", C.c_int), ("verbose", C.c_int), ("forcing", C.POINTER(C.c_double)),
                ("jacobian", C.c_int), ("ilu_order", C.c_int), ("ilu_parts", C.c_int), ("cfl_initial", C.c_double)]


class NewtonStats(C.Structure):
    _fields_ = [("newton_iterations", C.c_int), ("gmres_iterations", C.c_int), ("residual_initial", C.c_double),
                ("residual_final", C.c_double), ("seconds", C.c_double), ("assembly_seconds", C.c_double),
                ("rejected_steps", C.c_int), ("fallback_steps", C.c_int)]


class TileConfig(C.Structure):
    """Block configuration of the split-precision kernels (struct dpg_tile_config)."""
    _fields_ = [("elems_per_block", C.c_int), ("fp64_share_eighths", C.c_int), ("face_block_warps", C.c_int)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class RefVolume(C.Structure):
    """struct dpg_ref_volume: one entry of the reference's volume list."""
    _fields_ = [("xyz_ve", C.POINTER(C.c_double)), ("sol_coef", C.POINTER(C.c_double)), ("p_ref", C.c_int)]


class RefFace(C.Structure):
    """struct dpg_ref_face: one entry of the reference's face list."""
    _fields_ = [("volume", C.c_int * 2), ("ind_lf", C.c_int * 2), ("bc", C.c_int)]


class SimParams(C.Structure):
    _fields_ = [
        ("d", C.c_int), ("e_type", C.c_int), ("p", C.c_int), ("n_elem", C.c_int * 3),
        ("lo", C.c_double * 3), ("hi", C.c_double * 3), ("jitter", C.c_double), ("seed", C.c_uint64),
        ("pde_index", C.c_int), ("num_flux", C.c_int), ("test_case", C.c_int),
        ("vortex", C.c_double * 8), ("b_adv", C.c_double * 3),
        ("solver_proc", C.c_int), ("solver_type_e", C.c_int), ("dt", C.c_double), ("time_final", C.c_double),
        ("bc_side", C.c_int * 6), ("mesh_kind", C.c_int), ("num_flux_2nd", C.c_int), ("mu", C.c_double),
        ("Pr", C.c_double), ("omega", C.c_double), ("bc_state", C.c_double * 5), ("wall_p", C.c_double),
        ("wall_T", C.c_double), ("p_max", C.c_int), ("p_seed", C.c_uint64),
    ]


class DpgError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__(f"{what}: status {status}")
        self.status = status


_lib = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: run __graft_entry__.build() (python -m dpgsolver_gb300._build)")
    lib = C.CDLL(path)
    dp = C.POINTER(C.c_double)
    vp = C.c_void_p
    sig = {
        "dpg_status_string": (C.c_char_p, [C.c_int]),
        "dpg_sim_params_default": (None, [C.POINTER(SimParams)]),
        "dpg_sim_create": (C.c_int, [C.POINTER(SimParams), C.POINTER(vp)]),
        "dpg_sim_create_from_ctrl": (C.c_int, [C.c_char_p, C.POINTER(vp)]),
        "dpg_sim_create_from_gmsh": (C.c_int, [C.POINTER(SimParams), C.c_char_p, C.POINTER(vp)]),
        "dpg_sim_create_from_lists": (C.c_int, [C.POINTER(SimParams), C.c_int, C.POINTER(RefVolume), C.c_int,
                                                C.POINTER(RefFace), C.POINTER(vp)]),
        "dpg_sim_write_restart": (C.c_int, [vp, C.c_char_p]),
        "dpg_sim_write_vtk": (C.c_int, [vp, C.c_char_p]),
        "dpg_sim_read_restart": (C.c_int, [vp, C.c_char_p]),
        "dpg_sim_destroy": (None, [vp]),
        "dpg_sim_info": (C.c_int, [vp, C.POINTER(C.c_int64)]),
        "dpg_sim_get_sol_coef": (C.c_int, [vp, dp]),
        "dpg_sim_set_sol_coef": (C.c_int, [vp, dp]),
        "dpg_sim_get_rhs": (C.c_int, [vp, dp]),
        "dpg_sim_set_time": (C.c_int, [vp, C.c_double]),
        "dpg_sim_l2_error": (C.c_int, [vp, C.c_double, dp, C.c_int]),
        "dpg_sim_max_wave_speed": (C.c_double, [vp]),
        "dpg_sim_view": (vp, [vp]),
        "dpg_gpu_create": (C.c_int, [vp, C.POINTER(vp)]),
        "dpg_gpu_destroy": (None, [vp]),
        "dpg_gpu_set_precision": (C.c_int, [vp, C.c_int, C.c_int]),
        "dpg_gpu_set_positivity": (C.c_int, [vp, C.c_int]),
        "dpg_gpu_enforce_positivity": (C.c_int, [vp]),
        "dpg_gpu_positivity_update": (C.c_int, [vp, dp]),
        "dpg_gpu_upload_sol_coef": (C.c_int, [vp, dp]),
        "dpg_gpu_download_sol_coef": (C.c_int, [vp, dp]),
        "dpg_gpu_download_rhs": (C.c_int, [vp, dp]),
        "dpg_gpu_compute_rhs": (C.c_int, [vp, dp]),
        "dpg_gpu_rk_step": (C.c_int, [vp, C.c_double, C.c_int, dp]),
        "dpg_gpu_solve_explicit": (C.c_int, [vp, C.c_double, C.c_double, C.c_double, C.POINTER(C.c_int), dp]),
        "dpg_gpu_rk_step_host": (C.c_int, [vp, dp, C.c_double, C.c_int, dp]),
        "dpg_gpu_kernel_times": (C.c_int, [vp, C.c_int, dp, C.POINTER(C.c_char_p), C.c_int]),
        "dpg_gpu_launches_per_rhs": (C.c_int, [vp]),
        "dpg_gpu_time_rk_steps": (C.c_int, [vp, C.c_double, C.c_int, dp]),
        "dpg_newton_params_default": (None, [C.POINTER(NewtonParams)]),
        "dpg_gpu_newton_solve": (C.c_int, [vp, C.POINTER(NewtonParams), C.POINTER(NewtonStats)]),
        "dpg_gpu_jacobian_apply": (C.c_int, [vp, dp, dp]),
        "dpg_gpu_get_tiles": (C.c_int, [vp, C.POINTER(TileConfig)]),
        "dpg_gpu_set_tiles": (C.c_int, [vp, C.POINTER(TileConfig)]),
        "dpg_gpu_autotune": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(TileConfig), dp]),
        "dpg_gpu_mlp_enable": (C.c_int, [vp, C.c_int, C.c_int, C.c_uint64]),
        "dpg_gpu_mlp_train": (C.c_int, [vp, C.c_int, C.c_int, C.c_double, dp]),
        "dpg_gpu_mlp_samples": (C.c_int, [vp]),
        "dpg_gpu_mlp_params": (C.c_int, [vp, C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_int64)]),
        "dpg_gpu_mlp_loss_grad": (C.c_int, [vp, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float), dp,
                                            C.POINTER(C.c_float)]),
        "dpg_gpu_mlp_dims": (C.c_int, [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "dpg_gpu_mlp_set_wait_limit": (C.c_int, [vp, C.c_longlong]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _check(status: int, what: str) -> None:
    if status != DPG_OK:
        raise DpgError(status, what + " (" + load_library().dpg_status_string(status).decode() + ")")


@dataclass
class Config:
    """Structured periodic DG problem (mirrors the keys of a control file)."""
    d: int = 2
    p: int = 2
    n_elem: tuple = (16, 16, 1)
    lo: tuple = (-5.0, -5.0, 0.0)
    hi: tuple = (5.0, 5.0, 2.5)
    jitter: float = 0.0
    seed: int = 0
    pde: str = "euler"
    num_flux: str = "Roe-Pike"
    test_case: str = "isentropic_vortex"
    vortex: tuple = (5.0, 0.0, 0.0, 1.0, 1.0, 1.0, 0.0, 1.0)
    b_adv: tuple = (1.0, 0.5, 0.0)
    # boundaries, viscosity, curved geometry
    element: str = "tp"                    # "tp" (QUAD in 2D, HEX in 3D), "tri" (2D) or "tet" (3D): periodic advection
    bc: tuple = ("periodic",) * 6          # box sides x-, x+, y-, y+, z-, z+ (annulus: inner, outer wall)
    mesh: str = "box"                      # "box" or "annulus" (n_elem[0] radial x n_elem[1] azimuthal, r in lo[0]..hi[0])
    mu: float = 0.0
    Pr: float = 0.72
    omega: float = 0.0
    bc_state: tuple = (1.0, 1.0, 0.0, 0.0, 1.0)
    wall_p: float = 1.0
    wall_T: float = 1.0
    # mixed orders: p_max > p draws each volume's order uniformly from p .. p_max (seeded by p_seed)
    p_max: int = 0
    p_seed: int = 0

    def to_params(self) -> SimParams:
        prm = SimParams()
        load_library().dpg_sim_params_default(C.byref(prm))
        prm.d = self.d
        prm.e_type = {"tri": TRI, "tet": TET}.get(self.element, QUAD if self.d == 2 else HEX)
        prm.p = self.p
        for a in range(3):
            prm.n_elem[a] = int(self.n_elem[a]) if a < len(self.n_elem) else 1
            prm.lo[a] = float(self.lo[a])
            prm.hi[a] = float(self.hi[a])
        prm.jitter = self.jitter
        prm.seed = self.seed
        prm.pde_index = {"euler": PDE_EULER, "advection": PDE_ADVECTION, "navier_stokes": PDE_NAVIER_STOKES}[self.pde]
        prm.num_flux = {"Roe-Pike": NUM_FLUX_ROE_PIKE, "Lax-Friedrichs": NUM_FLUX_LAX_FRIEDRICHS,
                        "upwind": NUM_FLUX_UPWIND}[self.num_flux]
        prm.test_case = {"isentropic_vortex": TC_ISENTROPIC_VORTEX, "advection_sine": TC_ADVECTION_SINE,
                         "free_stream": TC_FREE_STREAM, "taylor_couette": TC_TAYLOR_COUETTE,
                         "periodic_vortex": TC_PERIODIC_VORTEX}[self.test_case]
        for i in range(8):
            prm.vortex[i] = self.vortex[i]
        for i in range(3):
            prm.b_adv[i] = self.b_adv[i]
        for k in range(6):
            b = self.bc[k] if k < len(self.bc) else "periodic"
            prm.bc_side[k] = BC_CODES[b] if isinstance(b, str) else int(b)
        prm.mesh_kind = {"box": MESH_BOX, "annulus": MESH_ANNULUS}[self.mesh]
        prm.num_flux_2nd = NUM_FLUX_BR2_STABLE if self.pde == "navier_stokes" else 0
        prm.mu, prm.Pr, prm.omega = float(self.mu), float(self.Pr), float(self.omega)
        for i in range(5):
            prm.bc_state[i] = float(self.bc_state[i])
        prm.wall_p, prm.wall_T = float(self.wall_p), float(self.wall_T)
        prm.p_max, prm.p_seed = int(self.p_max), int(self.p_seed)
        return prm


class Simulation:
    """Host simulation (mesh, operators, geometry, sol_coef).  Pure host code."""

    def __init__(self, cfg: Config | None = None, ctrl: str | None = None, msh: str | None = None):
        """From a Config (structured periodic box), a control file, or a gmsh 2.2 mesh file with a Config for the
        rest of the problem (its n_elem / lo / hi / jitter unused)."""
        lib = load_library()
        h = C.c_void_p()
        # the problem's parameters and mesh file, for callers that rebuild the same problem elsewhere
        self.cfg = None if ctrl is not None else (cfg or Config())
        self.msh = msh if ctrl is None else None
        if ctrl is not None:
            _check(lib.dpg_sim_create_from_ctrl(ctrl.encode(), C.byref(h)), "dpg_sim_create_from_ctrl")
        elif msh is not None:
            prm = (cfg or Config()).to_params()
            _check(lib.dpg_sim_create_from_gmsh(C.byref(prm), msh.encode(), C.byref(h)), "dpg_sim_create_from_gmsh")
        else:
            prm = (cfg or Config()).to_params()
            _check(lib.dpg_sim_create(C.byref(prm), C.byref(h)), "dpg_sim_create")
        self._adopt(h)

    @classmethod
    def from_reference_lists(cls, cfg: "Config", xyz_ve: np.ndarray, face_volume: np.ndarray, face_ind_lf: np.ndarray,
                             face_bc: np.ndarray | None = None, sol_coef=None,
                             p_ref: np.ndarray | None = None) -> "Simulation":
        """From the reference's volume and face lists (dpg_sim_create_from_lists): xyz_ve [n_vol, 2^d, d],
        face_volume / face_ind_lf [n_face, 2] (neigh_info[0..1]; volume -1 on side 1 of a boundary face), face_bc
        [n_face] (Face::bc), sol_coef [n_vol, n_s * n_var] (or a list of per-volume arrays) or None, p_ref [n_vol]
        (Solver_Volume_T::p_ref of an adapted mesh) or None."""
        lib = load_library()
        xyz = np.ascontiguousarray(xyz_ve, np.float64)
        fv = np.ascontiguousarray(face_volume, np.int32)
        fl = np.ascontiguousarray(face_ind_lf, np.int32)
        fb = np.zeros(len(fv), np.int32) if face_bc is None else np.ascontiguousarray(face_bc, np.int32)
        if sol_coef is None:
            sc = None
        elif isinstance(sol_coef, (list, tuple)):
            sc = [np.ascontiguousarray(a, np.float64) for a in sol_coef]
        else:
            sc = np.ascontiguousarray(sol_coef, np.float64).reshape(len(xyz), -1)
        vols = (RefVolume * len(xyz))()
        for v in range(len(xyz)):
            vols[v].xyz_ve = xyz[v].ctypes.data_as(C.POINTER(C.c_double))
            vols[v].sol_coef = sc[v].ctypes.data_as(C.POINTER(C.c_double)) if sc is not None else None
            vols[v].p_ref = int(p_ref[v]) if p_ref is not None else 0
        faces = (RefFace * len(fv))()
        for f in range(len(fv)):
            faces[f].volume[0], faces[f].volume[1] = int(fv[f, 0]), int(fv[f, 1])
            faces[f].ind_lf[0], faces[f].ind_lf[1] = int(fl[f, 0]), int(fl[f, 1])
            faces[f].bc = int(fb[f])
        prm = cfg.to_params()
        h = C.c_void_p()
        _check(lib.dpg_sim_create_from_lists(C.byref(prm), len(xyz), vols, len(fv), faces, C.byref(h)),
               "dpg_sim_create_from_lists")
        obj = cls.__new__(cls)
        obj.cfg, obj.msh = cfg, None
        obj._adopt(h)
        return obj

    def _adopt(self, h) -> None:
        lib = load_library()
        self.handle = h
        info = (C.c_int64 * 10)()
        _check(lib.dpg_sim_info(h, info), "dpg_sim_info")
        (self.d, self.n_var, self.n_vol, self.n_face, self.n_dof, self.n_s, self.n_c, self.n_fc, self.p,
         self.e_type) = [int(x) for x in info]

    def close(self) -> None:
        if self.handle:
            load_library().dpg_sim_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def write_restart(self, path: str) -> None:
        """Restart file of the current sol_coef (gmsh mesh + Bezier coefficients, the reference's format)."""
        _check(load_library().dpg_sim_write_restart(self.handle, path.encode()), "write_restart")

    def write_vtk(self, path: str) -> None:
        """VTK XML unstructured grid (.vtu) of the current sol_coef, one piece per volume (the reference's output)."""
        _check(load_library().dpg_sim_write_vtk(self.handle, path.encode()), "write_vtk")

    def read_restart(self, path: str) -> None:
        """sol_coef from a restart file (evaluated at this mesh's solution nodes)."""
        _check(load_library().dpg_sim_read_restart(self.handle, path.encode()), "read_restart")

    def sol_coef(self) -> np.ndarray:
        a = np.empty(self.n_dof, np.float64)
        _check(load_library().dpg_sim_get_sol_coef(self.handle, _dptr(a)), "get_sol_coef")
        return a

    def set_sol_coef(self, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a, np.float64)
        _check(load_library().dpg_sim_set_sol_coef(self.handle, _dptr(a)), "set_sol_coef")

    def l2_error(self, t: float) -> np.ndarray:
        e = np.zeros(5, np.float64)
        _check(load_library().dpg_sim_l2_error(self.handle, t, _dptr(e), 5), "l2_error")
        return e[: self.n_var]

    def max_wave_speed(self) -> float:
        return float(load_library().dpg_sim_max_wave_speed(self.handle))

    def cfl_dt(self, cfl: float, h: float) -> float:
        """dt = CFL * h / (max(|V|+c) * (2p+1))."""
        return cfl * h / (self.max_wave_speed() * (2 * self.p + 1))


class GpuContext:
    """Device state of one simulation (dpg_gpu_* calls)."""

    def __init__(self, sim: Simulation):
        lib = load_library()
        h = C.c_void_p()
        _check(lib.dpg_gpu_create(sim.handle, C.byref(h)), "dpg_gpu_create")
        self.handle = h
        self.sim = sim
        self.n_dof = sim.n_dof

    def close(self) -> None:
        if self.handle:
            load_library().dpg_gpu_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_precision(self, mode: int, n_slices: int = 0) -> None:
        _check(load_library().dpg_gpu_set_precision(self.handle, mode, n_slices), "set_precision")

    def write_restart(self, path: str) -> None:
        """Restart file of the device state (through the simulation's host copy)."""
        self.sim.set_sol_coef(self.download())
        self.sim.write_restart(path)

    def write_vtk(self, path: str) -> None:
        """VTK XML unstructured grid (.vtu) of the current sol_coef, one piece per volume (the reference's output)."""
        _check(load_library().dpg_sim_write_vtk(self.handle, path.encode()), "write_vtk")

    def read_restart(self, path: str) -> None:
        """Device state from a restart file (evaluated at this mesh's solution nodes)."""
        self.sim.read_restart(path)
        self.upload(self.sim.sol_coef())

    def set_positivity(self, on: bool) -> None:
        """Positivity limiter after every RK stage / Newton update (Euler; on by default, as in the reference)."""
        _check(load_library().dpg_gpu_set_positivity(self.handle, int(on)), "set_positivity")

    def enforce_positivity(self) -> None:
        """The positivity limiter on the context's state (enforce_positivity_highorder on every volume)."""
        _check(load_library().dpg_gpu_enforce_positivity(self.handle), "enforce_positivity")

    def positivity_update(self, du: np.ndarray) -> None:
        """Newton update u += relax du with the per-volume under-relaxation, then the limiter."""
        du = np.ascontiguousarray(du, np.float64)
        _check(load_library().dpg_gpu_positivity_update(self.handle, _dptr(du)), "positivity_update")

    def upload(self, sol: np.ndarray) -> None:
        sol = np.ascontiguousarray(sol, np.float64)
        _check(load_library().dpg_gpu_upload_sol_coef(self.handle, _dptr(sol)), "upload")

    def download(self) -> np.ndarray:
        a = np.empty(self.n_dof, np.float64)
        _check(load_library().dpg_gpu_download_sol_coef(self.handle, _dptr(a)), "download")
        return a

    def rhs(self) -> np.ndarray:
        a = np.empty(self.n_dof, np.float64)
        _check(load_library().dpg_gpu_download_rhs(self.handle, _dptr(a)), "download_rhs")
        return a

    def compute_rhs(self) -> float:
        m = C.c_double()
        _check(load_library().dpg_gpu_compute_rhs(self.handle, C.byref(m)), "compute_rhs")
        return m.value

    def rk_step(self, dt: float, n_steps: int = 1) -> float:
        m = C.c_double()
        _check(load_library().dpg_gpu_rk_step(self.handle, dt, n_steps, C.byref(m)), "rk_step")
        return m.value

    def rk_step_host(self, sol: np.ndarray, dt: float, n_steps: int = 1) -> float:
        m = C.c_double()
        _check(load_library().dpg_gpu_rk_step_host(self.handle, _dptr(sol), dt, n_steps, C.byref(m)), "rk_step_host")
        return m.value

    def solve_explicit(self, t0: float, t_final: float, dt: float) -> tuple[int, float]:
        n = C.c_int()
        m = C.c_double()
        _check(load_library().dpg_gpu_solve_explicit(self.handle, t0, t_final, dt, C.byref(n), C.byref(m)),
               "solve_explicit")
        return n.value, m.value

    def newton_solve(self, precond: int = PRECOND_BLOCK_JACOBI, tol: float = 1e-10, forcing: np.ndarray | None = None,
                     **kw) -> NewtonStats:
        lib = load_library()
        prm = NewtonParams()
        lib.dpg_newton_params_default(C.byref(prm))
        prm.precond = precond
        prm.tol = tol
        if forcing is not None:
            forcing = np.ascontiguousarray(forcing, np.float64)
            prm.forcing = _dptr(forcing)
        for k, v in kw.items():
            setattr(prm, k, v)
        st = NewtonStats()
        _check(lib.dpg_gpu_newton_solve(self.handle, C.byref(prm), C.byref(st)), "newton_solve")
        return st

    def jacobian_apply(self, v: np.ndarray) -> np.ndarray:
        """dF/du . v at the context's state (F = m_inv rhs), analytic linearisation in FP64."""
        v = np.ascontiguousarray(v, np.float64)
        out = np.empty_like(v)
        _check(load_library().dpg_gpu_jacobian_apply(self.handle, _dptr(v), _dptr(out)), "jacobian_apply")
        return out

    def mlp_enable(self, hidden: int = 256, capacity: int = 65536, seed: int = 0) -> None:
        _check(load_library().dpg_gpu_mlp_enable(self.handle, hidden, capacity, seed), "mlp_enable")

    def mlp_train(self, epochs: int, batch: int = 256, lr: float = 1e-3) -> float:
        loss = C.c_double()
        _check(load_library().dpg_gpu_mlp_train(self.handle, epochs, batch, lr, C.byref(loss)), "mlp_train")
        return loss.value

    def mlp_samples(self) -> int:
        return int(load_library().dpg_gpu_mlp_samples(self.handle))

    def mlp_set_wait_limit(self, polls: int) -> None:
        """Test hook: poll limit of the bounded waits in the network's tensor-core GEMMs (negative: default)."""
        _check(load_library().dpg_gpu_mlp_set_wait_limit(self.handle, int(polls)), "mlp_set_wait_limit")

    def mlp_dims(self) -> tuple:
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        _check(load_library().dpg_gpu_mlp_dims(self.handle, C.byref(a), C.byref(b), C.byref(c)), "mlp_dims")
        return a.value, b.value, c.value

    def mlp_params(self, set_to: np.ndarray | None = None) -> np.ndarray:
        lib = load_library()
        n = C.c_int64()
        _check(lib.dpg_gpu_mlp_params(self.handle, None, None, C.byref(n)), "mlp_params")
        fp = C.POINTER(C.c_float)
        if set_to is not None:
            s = np.ascontiguousarray(set_to, np.float32)
            _check(lib.dpg_gpu_mlp_params(self.handle, None, s.ctypes.data_as(fp), C.byref(n)), "mlp_params")
        out = np.empty(n.value, np.float32)
        _check(lib.dpg_gpu_mlp_params(self.handle, out.ctypes.data_as(fp), None, C.byref(n)), "mlp_params")
        return out

    def mlp_loss_grad(self, x: np.ndarray, target: np.ndarray) -> tuple[float, np.ndarray]:
        lib = load_library()
        fp = C.POINTER(C.c_float)
        x = np.ascontiguousarray(x, np.float32)
        target = np.ascontiguousarray(target, np.float32)
        n = C.c_int64()
        _check(lib.dpg_gpu_mlp_params(self.handle, None, None, C.byref(n)), "mlp_params")
        g = np.empty(n.value, np.float32)
        loss = C.c_double()
        _check(lib.dpg_gpu_mlp_loss_grad(self.handle, x.shape[0], x.ctypes.data_as(fp), target.ctypes.data_as(fp),
                                         C.byref(loss), g.ctypes.data_as(fp)), "mlp_loss_grad")
        return loss.value, g

    def tiles(self) -> dict:
        """The split-precision block configuration in use (elements per block, FP64 share, face block warps)."""
        t = TileConfig()
        _check(load_library().dpg_gpu_get_tiles(self.handle, C.byref(t)), "get_tiles")
        return t.as_dict()

    def set_tiles(self, elems_per_block: int, fp64_share_eighths: int, face_block_warps: int) -> None:
        t = TileConfig(elems_per_block, fp64_share_eighths, face_block_warps)
        _check(load_library().dpg_gpu_set_tiles(self.handle, C.byref(t)), "set_tiles")

    def autotune(self, n_rep: int = 10, force: bool = False) -> tuple[dict, float]:
        """Times candidate block configurations on the current state and keeps the fastest; returns it and its
        time per residual (ms).  Cached per process for the same device, element shape and mesh size."""
        t = TileConfig()
        ms = C.c_double()
        _check(load_library().dpg_gpu_autotune(self.handle, n_rep, int(force), C.byref(t), C.byref(ms)), "autotune")
        return t.as_dict(), ms.value

    def kernel_times(self, n_rep: int = 10) -> dict:
        ms = (C.c_double * 8)()
        names = (C.c_char_p * 8)()
        _check(load_library().dpg_gpu_kernel_times(self.handle, n_rep, ms, names, 8), "kernel_times")
        return {names[i].decode(): ms[i] for i in range(4) if names[i]}
