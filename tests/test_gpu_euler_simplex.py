"""The Euler equations on TRI and TET volumes on the GPU against the oracle's own set-up with the reference's
Witherden-Vincent rules (periodic isentropic vortex on jittered split boxes, Roe-Pike flux).

- FP64 residual and three SSP-RK3 steps (the positivity limiter after every stage, as the reference's Euler step)
  within 1e-11 of the oracle (2e-11 at p = 4), TRI p = 1..4 and TET p = 1..4;
- a state whose Bezier pressure average is negative stops the step with DPG_ERR_NONFINITE, as the reference stops
  ("Average pressure approaching 0.0"), on a mesh too coarse for the vortex (TET p = 2 at 3 x 3 x 2 cells);
- the dense simplex limiter (k_positivity_dense) against the oracle's enforce_positivity on states with planted
  negative Bezier coefficients (1e-10, the tolerance of the tensor-product limiter's test) and bit-identical on the
  volumes it leaves alone;
- the split-precision (tcgen05) path with S = 7 within 1e-10 of the oracle where its instantiations cover the
  shapes (TRI p = 1..4, TET p = 1..3)."""
import numpy as np
import pytest

import dpgsolver_gb300 as dg
from oracle import Oracle, Problem
from positivity_support import EPS_PHYS, bezier_prim_min, blocks, perturbed_state
from test_euler_simplex import CASES, IDS, cfg
from tests_support import oracle_rules, sim_arrays

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("element,p", CASES, ids=IDS)
def test_residual_and_steps_match_the_oracle(element, p):
    c = cfg(element, p)
    sim = dg.Simulation(dg.Config(**c))
    orc = Oracle(Problem(**c, **oracle_rules(element, p, sim)))
    u = orc.initial_solution()
    ctx = dg.GpuContext(sim)
    ctx.upload(u)
    m = ctx.compute_rhs()
    m_ref, r_ref = orc.compute_rhs(u)
    tol = 2e-11 if p == 4 else 1e-11   # order 4: the two set-ups' bases round differently
    assert _rel(ctx.rhs(), r_ref) <= tol
    assert abs(m - m_ref) <= tol * m_ref
    dt = 0.02 / p
    ctx.rk_step(dt, 3)
    orc.rk_step(u, dt, 3)
    assert _rel(ctx.download(), u) <= tol


@pytest.mark.parametrize("element,p", [("tri", 2), ("tri", 4), ("tet", 2), ("tet", 3)],
                         ids=["tri-p2", "tri-p4", "tet-p2", "tet-p3"])
def test_dense_limiter_matches_the_oracle(element, p):
    sim = dg.Simulation(dg.Config(**cfg(element, p)))
    u, picked = perturbed_state(sim)
    o = u.copy()
    assert Oracle(sim).enforce_positivity(o) == 0   # the planted state keeps positive averages (no stop)
    ctx = dg.GpuContext(sim)
    ctx.upload(u)
    ctx.enforce_positivity()
    g = ctx.download()
    scale = np.max(np.abs(u))
    assert np.max(np.abs(g - o)) <= 1e-10 * scale
    a = sim_arrays(sim)
    for e in picked:
        assert min(bezier_prim_min(blocks(sim, g)[e], a["ccSB0_vs_vs"], sim.d)) >= EPS_PHYS - 1e-13 * scale
    mask = np.ones(sim.n_vol, bool)
    mask[picked] = False
    assert np.array_equal(blocks(sim, g)[mask], blocks(sim, u)[mask])


@pytest.mark.parametrize("element,p", CASES[:7], ids=IDS[:7])
def test_split_precision(element, p):
    c = cfg(element, p)
    sim = dg.Simulation(dg.Config(**c))
    orc = Oracle(Problem(**c, **oracle_rules(element, p, sim)))
    u = orc.initial_solution()
    _, r_ref = orc.compute_rhs(u)
    ctx = dg.GpuContext(sim)
    ctx.set_precision(dg.PREC_BF16_SLICED, 7)
    ctx.upload(u)
    ctx.compute_rhs()
    assert _rel(ctx.rhs(), r_ref) <= 1e-10


def test_negative_average_stops_like_the_reference():
    sim = dg.Simulation(dg.Config(**cfg("tet", 2, (3, 3, 2))))
    u = sim.sol_coef()
    assert Oracle(sim).enforce_positivity(u.copy()) == -1
    ctx = dg.GpuContext(sim)
    ctx.upload(u)
    with pytest.raises(dg.DpgError) as e:
        ctx.enforce_positivity()
    assert e.value.status == dg.api.DPG_ERR_NONFINITE
