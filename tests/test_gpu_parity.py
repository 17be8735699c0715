"""GPU residual vs the CPU oracle on the same seeded inputs, through the C ABI.

Tolerance: FP64 path, max |rhs_gpu - rhs_oracle| <= 1e-11 * max |rhs_oracle| (rounding-order differences in
K-term sums whose terms exceed the result; the required parity bound for floating point is 1e-10 relative).
"""
import math

import numpy as np
import pytest

import dpgsolver_gb300 as dg
from oracle import Oracle

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-11

CASES = [
    dict(d=2, p=1, n_elem=(5, 4, 1)),
    dict(d=2, p=2, n_elem=(6, 6, 1)),
    dict(d=2, p=3, n_elem=(4, 5, 1), num_flux="Lax-Friedrichs"),
    dict(d=2, p=4, n_elem=(3, 3, 1), jitter=0.2, seed=5),
    dict(d=3, p=1, n_elem=(3, 3, 2)),
    dict(d=3, p=2, n_elem=(4, 3, 2), jitter=0.15, seed=2),
    dict(d=3, p=3, n_elem=(4, 4, 2)),
    dict(d=3, p=3, n_elem=(3, 3, 3), num_flux="Lax-Friedrichs"),
    dict(d=2, p=3, n_elem=(6, 6, 1), pde="advection", num_flux="upwind", test_case="advection_sine",
         lo=(0, 0, 0), hi=(1, 1, 1), jitter=0.1, seed=1),
    dict(d=3, p=2, n_elem=(3, 3, 3), pde="advection", num_flux="upwind", test_case="advection_sine",
         lo=(0, 0, 0), hi=(1, 1, 1), b_adv=(1.0, 0.5, 0.25)),
]


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("case", CASES, ids=lambda c: "-".join(f"{k}{v}" for k, v in c.items() if k in ("d", "p", "num_flux", "jitter")))
def test_rhs_matches_oracle(case):
    sim = dg.Simulation(dg.Config(**case))
    orc = Oracle(sim)
    ctx = dg.GpuContext(sim)
    rng = np.random.default_rng(11)
    sol = sim.sol_coef()
    # perturb the state so that every coefficient matters (keeps density/pressure positive)
    sol = sol * (1.0 + 1e-2 * rng.standard_normal(sol.shape))
    ctx.upload(sol)
    m_gpu = ctx.compute_rhs()
    m_ref, rhs_ref = orc.compute_rhs(sol)
    assert _rel(ctx.rhs(), rhs_ref) <= FP64_TOL
    assert abs(m_gpu - m_ref) <= FP64_TOL * m_ref


@pytest.mark.parametrize("case", [CASES[1], CASES[6], CASES[8]], ids=["quad-p2", "hex-p3", "adv-p3"])
def test_rk3_steps_match_oracle(case):
    sim = dg.Simulation(dg.Config(**case))
    orc = Oracle(sim)
    ctx = dg.GpuContext(sim)
    sol = sim.sol_coef()
    dt = 0.25 * sim.cfl_dt(0.4, 10.0 / case["n_elem"][0])
    m_gpu = ctx.rk_step(dt, 3)
    ref = sol.copy()
    m_ref = orc.rk_step(ref, dt, 3)
    assert _rel(ctx.download(), ref) <= FP64_TOL
    assert abs(m_gpu - m_ref) <= 1e-10 * m_ref


def test_solve_explicit_shortens_last_step():
    case = dict(d=2, p=2, n_elem=(6, 6, 1))
    sim = dg.Simulation(dg.Config(**case))
    orc = Oracle(sim)
    ctx = dg.GpuContext(sim)
    dt, tf = 0.03, 0.1
    n, _ = ctx.solve_explicit(0.0, tf, dt)
    assert n == 4
    ref = sim.sol_coef()
    orc.rk_step(ref, dt, 3)
    orc.rk_step(ref, tf - 3 * dt, 1)
    assert _rel(ctx.download(), ref) <= FP64_TOL


def test_host_buffer_entry_point():
    sim = dg.Simulation(dg.Config(d=3, p=2, n_elem=(3, 3, 2)))
    orc = Oracle(sim)
    ctx = dg.GpuContext(sim)
    sol = sim.sol_coef()
    ref = sol.copy()
    ctx.rk_step_host(sol, 0.01, 2)
    orc.rk_step(ref, 0.01, 2)
    assert _rel(sol, ref) <= FP64_TOL


def test_nonfinite_state_is_reported():
    sim = dg.Simulation(dg.Config(d=2, p=2, n_elem=(4, 4, 1)))
    ctx = dg.GpuContext(sim)
    sol = sim.sol_coef()
    sol[7] = np.nan
    ctx.upload(sol)
    with pytest.raises(dg.DpgError) as ei:
        ctx.compute_rhs()
    assert ei.value.status == dg.api.DPG_ERR_NONFINITE
