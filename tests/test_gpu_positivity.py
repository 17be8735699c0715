"""Positivity limiter and Newton under-relaxation on the GPU against the oracle (enforce_positivity_highorder,
solve.c:187-233, after every RK stage; compute_relaxation + update_coef_s_v, solve_implicit.c:724-731, 821-873).

Tolerances (max-norm, relative to the state's largest entry): volumes the limiter corrects 1e-10 (a density
correction leaves a Bezier coefficient at density EPS_PHYS, where m / rho carries the rounding of rho at ~1e-3
relative into the pressure correction: two restatements agree to ~3e-12); volumes it does not correct: the GPU leaves
them bit-identical where its FP32 screen clears them, the oracle (as the reference) round-trips them through the
Bezier and primitive forms (1e-13).
"""
import numpy as np
import pytest

import dpgsolver_gb300 as dg
from oracle import Oracle
from positivity_support import EPS_PHYS, bezier_prim_min, blocks, perturbed_state
from tests_support import sim_arrays

pytestmark = pytest.mark.gpu

CASES = [dict(d=2, p=1, n_elem=(8, 8, 1)), dict(d=2, p=2, n_elem=(6, 6, 1)), dict(d=2, p=4, n_elem=(4, 4, 1)),
         dict(d=3, p=1, n_elem=(6, 6, 2)), dict(d=3, p=2, n_elem=(6, 6, 2)), dict(d=3, p=3, n_elem=(6, 6, 2)),
         dict(d=3, p=4, n_elem=(4, 4, 2))]
IDS = [f"d{c['d']}-p{c['p']}" for c in CASES]
LIMITED_TOL = 1e-10


def _gpu_limited(sim, u):
    ctx = dg.GpuContext(sim)
    ctx.upload(u)
    ctx.enforce_positivity()
    return ctx.download()


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_limiter_matches_oracle(case):
    sim = dg.Simulation(dg.Config(**case))
    u, picked = perturbed_state(sim)
    g = _gpu_limited(sim, u)
    o = u.copy()
    assert Oracle(sim).enforce_positivity(o) == 0
    scale = np.max(np.abs(u))
    assert np.max(np.abs(g - o)) <= LIMITED_TOL * scale
    a = sim_arrays(sim)
    for e in picked:   # corrected: positive Bezier minima again
        assert min(bezier_prim_min(blocks(sim, g)[e], a["ccSB0_vs_vs"], sim.d)) >= EPS_PHYS - 1e-13 * scale
    mask = np.ones(sim.n_vol, bool)
    mask[picked] = False
    assert np.max(np.abs(blocks(sim, g)[mask] - blocks(sim, u)[mask])) <= 1e-13 * scale


def test_limiter_acts_on_a_coarse_interpolant():
    """3x3x3 HEX p2 vortex: the interpolant itself has negative Bezier coefficients in some volumes."""
    sim = dg.Simulation(dg.Config(d=3, p=2, n_elem=(3, 3, 3)))
    u = sim.sol_coef()
    g = _gpu_limited(sim, u)
    o = u.copy()
    assert Oracle(sim).enforce_positivity(o) == 0
    assert np.max(np.abs(g - o)) <= LIMITED_TOL * np.max(np.abs(u))
    assert np.max(np.abs(g - u)) > 1e-3   # the limiter did act


def test_limiter_leaves_a_positive_state_bit_identical():
    """The screen clears every volume of a resolved vortex (the bench's situation): no volume is rewritten."""
    sim = dg.Simulation(dg.Config(d=3, p=3, n_elem=(12, 12, 4), lo=(-5, -5, 0), hi=(5, 5, 2.5)))
    u = sim.sol_coef()
    assert np.array_equal(_gpu_limited(sim, u), u)


def test_vanishing_average_is_an_error_and_leaves_the_volume():
    sim = dg.Simulation(dg.Config(d=2, p=2, n_elem=(4, 4, 1)))
    u = sim.sol_coef().copy()
    blocks(sim, u)[5, 0, :] = -0.2
    ctx = dg.GpuContext(sim)
    ctx.upload(u)
    with pytest.raises(dg.DpgError) as ei:
        ctx.enforce_positivity()
    assert ei.value.status == dg.api.DPG_ERR_NONFINITE
    assert np.array_equal(blocks(sim, ctx.download())[5], blocks(sim, u)[5])
    ctx.upload(sim.sol_coef())   # the error is reported once; the context stays usable
    ctx.enforce_positivity()
    ctx.compute_rhs()


@pytest.mark.parametrize("prec", [(dg.PREC_FP64, 0), (dg.PREC_BF16_SLICED, 7)], ids=["fp64", "sliced7"])
@pytest.mark.parametrize("case", [dict(d=3, p=2, n_elem=(3, 3, 3)), dict(d=2, p=2, n_elem=(6, 6, 1))],
                         ids=["coarse-hex-p2", "quad-p2-perturbed"])
def test_rk_steps_with_the_limiter_match_oracle(case, prec):
    """The coarse HEX interpolant needs the limiter at every stage; the perturbed QUAD state is limited first (a step
    starts with a residual of its input state, which a negative nodal density makes non-finite, in the reference as
    here) and leaves the limiter work on the stages' small coefficients."""
    sim = dg.Simulation(dg.Config(**case))
    if case["d"] == 3:
        u = sim.sol_coef()
    else:
        u = perturbed_state(sim)[0]
        assert Oracle(sim).enforce_positivity(u) == 0
    dt = sim.cfl_dt(0.2, 10.0 / case["n_elem"][0])
    ctx = dg.GpuContext(sim)
    ctx.set_precision(*prec)
    ctx.upload(u)
    ctx.rk_step(dt, 2)
    o = u.copy()
    Oracle(sim).rk_step(o, dt, 2)
    err = np.max(np.abs(ctx.download() - o)) / np.max(np.abs(o))
    assert err <= 1e-9, err


def test_limiter_switch():
    sim = dg.Simulation(dg.Config(d=3, p=2, n_elem=(3, 3, 3)))
    u = sim.sol_coef()
    dt = sim.cfl_dt(0.2, 10.0 / 3)
    ctx = dg.GpuContext(sim)
    ctx.set_positivity(False)
    ctx.upload(u)
    ctx.rk_step(dt, 1)
    ora = Oracle(sim)
    ora.set_positivity(False)
    o = u.copy()
    ora.rk_step(o, dt, 1)
    assert np.max(np.abs(ctx.download() - o)) <= 1e-11 * np.max(np.abs(o))
    adv = dg.GpuContext(dg.Simulation(dg.Config(d=2, p=2, n_elem=(4, 4, 1), pde="advection", num_flux="upwind",
                                                test_case="advection_sine", lo=(0, 0, 0), hi=(1, 1, 1))))
    with pytest.raises(dg.DpgError) as ei:
        adv.set_positivity(True)
    assert ei.value.status == dg.api.DPG_ERR_UNSUPPORTED


@pytest.mark.parametrize("case", CASES[1:2] + CASES[4:6], ids=IDS[1:2] + IDS[4:6])
def test_relaxed_newton_update_matches_oracle(case):
    sim = dg.Simulation(dg.Config(**case))
    u = sim.sol_coef()
    d = sim.d
    rng = np.random.default_rng(2)
    du = 0.05 * rng.standard_normal(u.shape) * np.max(np.abs(u))
    db = blocks(sim, du)
    db[1, 0, :] = -1.3 * blocks(sim, u)[1, 0, :]
    db[3, d + 1, :] = -3.0 * blocks(sim, u)[3, d + 1, :]
    ora = Oracle(sim)
    rc, relax = ora.positivity_relaxation(u, du)
    assert rc == 0 and relax[1] < 1.0 and relax[3] < 1.0
    o = (blocks(sim, u) + relax[:, None, None] * db).reshape(-1).copy()
    assert ora.enforce_positivity(o) == 0
    ctx = dg.GpuContext(sim)
    ctx.upload(u)
    ctx.positivity_update(du)
    assert np.max(np.abs(ctx.download() - o)) <= LIMITED_TOL * np.max(np.abs(o))
