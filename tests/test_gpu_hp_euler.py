"""Mixed orders for the Euler equations on the GPU (`kernels_hp.cu`, every order in each launch, and the dense
positivity limiter launched per order group) against the oracle's own mixed-order set-up: residual and three SSP-RK3
steps with the limiter after every stage within 1e-11 on QUAD, HEX, TRI and TET meshes (the HEX case's coarse
interpolant has negative Bezier coefficients, so the limiter acts there)."""
import numpy as np
import pytest

import dpgsolver_gb300 as dg
from oracle import Oracle, Problem
from test_hp_euler import CASES, IDS, problem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("element,d,n,p_max", CASES, ids=IDS)
def test_residual_and_steps_match_the_oracle(element, d, n, p_max):
    c, kw = problem(element, d, n, p_max)
    sim = dg.Simulation(dg.Config(**c))
    orc = Oracle(Problem(**c, **kw))
    u = orc.initial_solution()
    ctx = dg.GpuContext(sim)
    ctx.upload(u)
    ctx.compute_rhs()
    _, r_ref = orc.compute_rhs(u)
    assert np.max(np.abs(ctx.rhs() - r_ref)) <= 1e-11 * np.max(np.abs(r_ref))
    ctx.rk_step(0.005, 3)
    orc.rk_step(u, 0.005, 3)
    assert np.max(np.abs(ctx.download() - u)) <= 1e-11 * np.max(np.abs(u))
