"""ctypes binding of the CPU oracle (oracle_dg.c).  Test infrastructure only."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

ORACLE_LIB = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "liboracle_dg.so")
_lib = None


def load_oracle() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(ORACLE_LIB):
        raise RuntimeError(f"{ORACLE_LIB} missing: build it with __graft_entry__.build()")
    lib = C.CDLL(ORACLE_LIB)
    dp = C.POINTER(C.c_double)
    lib.oracle_create.restype = C.c_void_p
    lib.oracle_create.argtypes = [C.c_void_p]
    lib.oracle_destroy.restype = None
    lib.oracle_destroy.argtypes = [C.c_void_p]
    lib.oracle_compute_rhs.restype = C.c_double
    lib.oracle_compute_rhs.argtypes = [C.c_void_p, dp, dp]
    lib.oracle_compute_rhs_unscaled.restype = C.c_double
    lib.oracle_compute_rhs_unscaled.argtypes = [C.c_void_p, dp, dp]
    lib.oracle_rk_step.restype = C.c_double
    lib.oracle_rk_step.argtypes = [C.c_void_p, dp, C.c_double, C.c_int]
    lib.oracle_flux_euler.restype = None
    lib.oracle_enforce_positivity.restype = C.c_int
    lib.oracle_enforce_positivity.argtypes = [C.c_void_p, dp]
    lib.oracle_set_positivity.restype = None
    lib.oracle_set_positivity.argtypes = [C.c_void_p, C.c_int]
    lib.oracle_positivity_relaxation.restype = C.c_int
    lib.oracle_positivity_relaxation.argtypes = [C.c_void_p, dp, dp, dp]
    lib.oracle_flux_euler.argtypes = [C.c_int, dp, dp]
    lib.oracle_numflux_euler_roe_pike.restype = None
    lib.oracle_numflux_euler_roe_pike.argtypes = [C.c_int, dp, dp, dp, dp]
    lib.oracle_numflux_euler_lax_friedrichs.restype = None
    lib.oracle_numflux_euler_lax_friedrichs.argtypes = [C.c_int, dp, dp, dp, dp]
    lib.oracle_numflux_advection_upwind.restype = C.c_double
    lib.oracle_numflux_advection_upwind.argtypes = [C.c_int, dp, C.c_double, C.c_double, dp]
    _lib = lib
    return lib


def _p(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """FP64 serial restatement of compute_rhs_dg / time_step_ssp_rk_33 on a dpgsolver_gb300.Simulation."""

    def __init__(self, sim):
        self.lib = load_oracle()
        self.sim = sim
        self.h = self.lib.oracle_create(sim.handle)
        self.n_vol = sim.n_vol

    def close(self):
        if self.h:
            self.lib.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

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
