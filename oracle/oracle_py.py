"""ctypes binding of the CPU oracle (oracle_setup.c + oracle_dg.c).  Test infrastructure only.

The oracle builds its problem -- mesh, operators, geometry, connectivity, initial state -- from the problem
parameters alone (``Problem``), with its own code; it neither imports nor loads the library under test.  It is
compiled by ``build_oracle()`` (plain gcc), which the benchmark's CPU legs call instead of the library's build.
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess
from dataclasses import dataclass

import numpy as np

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(ORACLE_DIR)
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", "liboracle_dg.so")
_lib = None

# reference codes (definitions_test_case.h, definitions_numerical_flux.h), the same integers as the library's
PDE_ADVECTION, PDE_EULER, PDE_NAVIER_STOKES = 1, 3, 4
NUM_FLUX = {"upwind": 11, "Roe-Pike": 31, "Lax-Friedrichs": 32}
PDE = {"advection": PDE_ADVECTION, "euler": PDE_EULER, "navier_stokes": PDE_NAVIER_STOKES}
TEST_CASE = {"isentropic_vortex": 1, "advection_sine": 2, "free_stream": 3, "taylor_couette": 4, "periodic_vortex": 5}
BC = {"periodic": 0, "riemann": 101, "slipwall": 102, "noslip_adiabatic": 111, "noslip_all_rotating": 113}
MESH = {"box": 0, "annulus": 1}


def build_oracle(force: bool = False) -> str:
    """Compiles oracle/*.c into oracle/_build/liboracle_dg.so (gcc, no CUDA)."""
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    src = sorted(glob.glob(os.path.join(ORACLE_DIR, "*.c")))
    hdr = (glob.glob(os.path.join(ORACLE_DIR, "*.h")) + glob.glob(os.path.join(ORACLE_DIR, "*.inc"))
           + glob.glob(os.path.join(ROOT, "include", "*.h")))
    if force or not os.path.exists(ORACLE_LIB) or any(os.path.getmtime(s) > os.path.getmtime(ORACLE_LIB)
                                                       for s in src + hdr):
        cmd = ["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-fPIC", "-shared", "-pthread",
               "-I" + os.path.join(ROOT, "include"), *src, "-o", ORACLE_LIB, "-lm"]
        proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if proc.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + proc.stdout)
    return ORACLE_LIB


class OracleParams(C.Structure):
    """struct oracle_params (oracle_dg.h)."""
    _fields_ = [("d", C.c_int), ("p", C.c_int), ("n_elem", C.c_int * 3), ("lo", C.c_double * 3),
                ("hi", C.c_double * 3), ("jitter", C.c_double), ("seed", C.c_uint64), ("pde_index", C.c_int),
                ("num_flux", C.c_int), ("test_case", C.c_int), ("vortex", C.c_double * 8), ("b_adv", C.c_double * 3),
                ("bc_side", C.c_int * 6), ("mesh_kind", C.c_int), ("mu", C.c_double), ("Pr", C.c_double),
                ("omega", C.c_double), ("bc_state", C.c_double * 5), ("wall_p", C.c_double), ("wall_T", C.c_double),
                ("e_type", C.c_int), ("p_max", C.c_int), ("p_seed", C.c_uint64), ("vrule_n", C.c_int * 9),
                ("vrule", C.POINTER(C.c_double) * 9), ("frule_n", C.c_int * 9), ("frule", C.POINTER(C.c_double) * 9)]


@dataclass
class Problem:
    """Problem parameters of the oracle (the same keys as the library's Config)."""
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
    bc: tuple = ("periodic",) * 6
    mesh: str = "box"
    mu: float = 0.0
    Pr: float = 0.72
    omega: float = 0.0
    bc_state: tuple = (1.0, 1.0, 0.0, 0.0, 1.0)
    wall_p: float = 1.0
    wall_T: float = 1.0
    element: str = "tp"                      # "tp" (QUAD / HEX), "tri" (2D cells split into two triangles) or
                                             # "tet" (3D cells split into six tetrahedra)
    p_max: int = 0                           # mixed orders: each volume's order drawn from p .. p_max
    p_seed: int = 0
    vol_rules: dict = None                   # TRI / TET: {p: [n][d + 2] barycentric points and weights summing
                                             # to 1}, the volume cubature of order p (default: Stroud's rule)
    face_rules: dict = None                  # TET: {p: [n][4] barycentric points on a face and weights summing to
                                             # 1}, a symmetric face cubature of order p (default: symmetrised Stroud)

    @classmethod
    def like(cls, cfg) -> "Problem":
        """The same problem from any object with these attribute names (e.g. the library's Config)."""
        return cls(**{k: getattr(cfg, k) for k in cls.__dataclass_fields__ if hasattr(cfg, k)})

    def params(self) -> OracleParams:
        prm = OracleParams()
        prm.d, prm.p = int(self.d), int(self.p)
        for a in range(3):
            prm.n_elem[a] = int(self.n_elem[a]) if a < len(self.n_elem) else 1
            prm.lo[a], prm.hi[a] = float(self.lo[a]), float(self.hi[a])
        prm.jitter, prm.seed = float(self.jitter), int(self.seed)
        prm.pde_index, prm.num_flux = PDE[self.pde], NUM_FLUX[self.num_flux]
        prm.test_case = TEST_CASE[self.test_case]
        for i in range(8):
            prm.vortex[i] = float(self.vortex[i])
        for i in range(3):
            prm.b_adv[i] = float(self.b_adv[i])
        for k in range(6):
            b = self.bc[k] if k < len(self.bc) else "periodic"
            prm.bc_side[k] = BC[b] if isinstance(b, str) else int(b)
        prm.mesh_kind = MESH[self.mesh]
        prm.mu, prm.Pr, prm.omega = float(self.mu), float(self.Pr), float(self.omega)
        for i in range(5):
            prm.bc_state[i] = float(self.bc_state[i])
        prm.wall_p, prm.wall_T = float(self.wall_p), float(self.wall_T)
        prm.e_type = {"tri": 2, "tet": 4}.get(self.element, 0)   # DPG_TRI, DPG_TET; 0: tensor-product
        prm.p_max, prm.p_seed = int(self.p_max), int(self.p_seed)
        prm._keep = []
        for pk, r in (self.vol_rules or {}).items():
            a = np.ascontiguousarray(np.asarray(r, dtype=np.float64))
            assert a.ndim == 2 and a.shape[1] == int(self.d) + 2 and 1 <= int(pk) <= 8
            prm._keep.append(a)
            prm.vrule_n[int(pk)] = a.shape[0]
            prm.vrule[int(pk)] = a.ctypes.data_as(C.POINTER(C.c_double))
        for pk, r in (self.face_rules or {}).items():
            a = np.ascontiguousarray(np.asarray(r, dtype=np.float64))
            assert a.ndim == 2 and a.shape[1] == 4 and 1 <= int(pk) <= 8
            prm._keep.append(a)
            prm.frule_n[int(pk)] = a.shape[0]
            prm.frule[int(pk)] = a.ctypes.data_as(C.POINTER(C.c_double))
        return prm


def load_oracle() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(ORACLE_LIB):
        build_oracle()
    lib = C.CDLL(ORACLE_LIB)
    dp = C.POINTER(C.c_double)
    vp = C.c_void_p
    sig = {
        "oracle_sim_structured": (C.c_int, [C.POINTER(OracleParams), C.POINTER(vp)]),
        "oracle_sim_gmsh": (C.c_int, [C.POINTER(OracleParams), C.c_char_p, C.POINTER(vp)]),
        "oracle_sim_free": (None, [vp]),
        "oracle_initial_solution": (None, [vp, dp]),
        "oracle_l2_error": (C.c_int, [vp, dp, C.c_double, dp]),
        "oracle_nodes_gl": (None, [C.c_int, dp, dp]),
        "oracle_nodes_gll": (None, [C.c_int, dp, dp]),
        "oracle_create": (vp, [vp]),
        "oracle_destroy": (None, [vp]),
        "oracle_set_threads": (None, [vp, C.c_int]),
        "oracle_compute_rhs": (C.c_double, [vp, dp, dp]),
        "oracle_compute_rhs_unscaled": (C.c_double, [vp, dp, dp]),
        "oracle_rk_step": (C.c_double, [vp, dp, C.c_double, C.c_int]),
        "oracle_enforce_positivity": (C.c_int, [vp, dp]),
        "oracle_set_positivity": (None, [vp, C.c_int]),
        "oracle_positivity_relaxation": (C.c_int, [vp, dp, dp, dp]),
        "oracle_cs_jvp": (C.c_double, [vp, dp, dp, C.c_double, dp, dp]),
        "oracle_flux_euler": (None, [C.c_int, dp, dp]),
        "oracle_numflux_euler_roe_pike": (None, [C.c_int, dp, dp, dp, dp]),
        "oracle_numflux_euler_lax_friedrichs": (None, [C.c_int, dp, dp, dp, dp]),
        "oracle_numflux_advection_upwind": (C.c_double, [C.c_int, dp, C.c_double, C.c_double, dp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))


def nodes(kind: str, n: int) -> tuple[np.ndarray, np.ndarray]:
    """The oracle's 1D nodes and weights: kind 'GL' or 'GLL'."""
    x, w = np.zeros(n), np.zeros(n)
    fn = load_oracle().oracle_nodes_gl if kind == "GL" else load_oracle().oracle_nodes_gll
    fn(n, _p(x), _p(w))
    return x, w


class Oracle:
    """FP64 restatement of compute_rhs_dg / time_step_ssp_rk_33 on the oracle's own set-up of a problem.

    ``source`` is a ``Problem``, an object with the same attributes (the library's ``Config``), or a library
    ``Simulation``, of which only its parameters (``cfg``) and its mesh file name (``msh``) are used.
    ``data_model`` (advanced): the address of an existing include/dpg_simulation.h data model to run the residual
    restatement on instead -- the tests use it to check the library's set-up through the residual.
    """

    def __init__(self, source=None, msh: str | None = None, threads: int = 1, data_model: int | None = None):
        self.lib = load_oracle()
        self.sim_h = None
        if data_model is None:
            if source is not None and hasattr(source, "handle") and hasattr(source, "cfg"):
                msh = msh or getattr(source, "msh", None)
                source = source.cfg
            if source is None:
                raise ValueError("the oracle needs the problem's parameters")
            prob = source if isinstance(source, Problem) else Problem.like(source)
            prm = prob.params()
            h = C.c_void_p()
            rc = (self.lib.oracle_sim_gmsh(C.byref(prm), msh.encode(), C.byref(h)) if msh
                  else self.lib.oracle_sim_structured(C.byref(prm), C.byref(h)))
            if rc != 0:
                raise RuntimeError(f"oracle set-up failed ({rc})")
            self.sim_h = h
            model = h.value
            self.problem = prob
        else:
            model = data_model
            self.problem = None
        self.model = model
        self.h = self.lib.oracle_create(model)
        from . import oracle_layout as L  # sizes of the data model

        self.layout = L.read(model)
        self.n_vol = self.layout["n_vol"]
        self.n_dof = self.layout["n_dof"]
        if threads > 1:
            self.lib.oracle_set_threads(self.h, int(threads))

    def close(self):
        if self.h:
            self.lib.oracle_destroy(self.h)
            self.h = None
        if self.sim_h:
            self.lib.oracle_sim_free(self.sim_h)
            self.sim_h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_threads(self, n: int) -> None:
        self.lib.oracle_set_threads(self.h, int(n))

    def initial_solution(self) -> np.ndarray:
        """The oracle's own initial state (the test case at the solution nodes)."""
        sol = np.empty(self.n_dof, np.float64)
        self.lib.oracle_initial_solution(self.model, _p(sol))
        return sol

    def l2_error(self, sol: np.ndarray, t: float) -> np.ndarray:
        """L2 errors against the exact solution at time t (rho, u, v, (w), p or u)."""
        sol = np.ascontiguousarray(sol, np.float64)
        err = np.zeros(5, np.float64)
        self.lib.oracle_l2_error(self.model, _p(sol), t, _p(err))
        return err[: self.layout["n_var"]]

    def compute_rhs(self, sol: np.ndarray) -> tuple[float, np.ndarray]:
        sol = np.ascontiguousarray(sol, np.float64)
        rhs = np.empty_like(sol)
        m = self.lib.oracle_compute_rhs(self.h, _p(sol), _p(rhs))
        return m, rhs

    def compute_rhs_unscaled(self, sol: np.ndarray) -> tuple[float, np.ndarray]:
        sol = np.ascontiguousarray(sol, np.float64)
        rhs = np.empty_like(sol)
        m = self.lib.oracle_compute_rhs_unscaled(self.h, _p(sol), _p(rhs))
        return m, rhs

    def jvp_complex_step(self, u: np.ndarray, v: np.ndarray, h: float = 1e-30) -> tuple[np.ndarray, np.ndarray]:
        """dF/du(u) v of the scaled residual F = m_inv rhs by the complex step Im F(u + i h v) / h, and F(u)."""
        u = np.ascontiguousarray(u, np.float64)
        v = np.ascontiguousarray(v, np.float64)
        jv, f = np.empty_like(u), np.empty_like(u)
        self.lib.oracle_cs_jvp(self.h, _p(u), _p(v), h, _p(jv), _p(f))
        return jv, f

    def rk_step(self, sol: np.ndarray, dt: float, n_steps: int) -> float:
        assert sol.dtype == np.float64 and sol.flags["C_CONTIGUOUS"]
        return self.lib.oracle_rk_step(self.h, _p(sol), dt, n_steps)

    def set_positivity(self, on: bool) -> None:
        self.lib.oracle_set_positivity(self.h, int(on))

    def enforce_positivity(self, sol: np.ndarray) -> int:
        """enforce_positivity_highorder on every volume, in place; 0, or -1 where an average is below EPS_PHYS."""
        assert sol.dtype == np.float64 and sol.flags["C_CONTIGUOUS"]
        return self.lib.oracle_enforce_positivity(self.h, _p(sol))

    def positivity_relaxation(self, u: np.ndarray, du: np.ndarray) -> tuple[int, np.ndarray]:
        """compute_relaxation per volume for the Newton update du at u."""
        u = np.ascontiguousarray(u, np.float64)
        du = np.ascontiguousarray(du, np.float64)
        relax = np.empty(self.n_vol, np.float64)
        rc = self.lib.oracle_positivity_relaxation(self.h, _p(u), _p(du), _p(relax))
        return rc, relax
