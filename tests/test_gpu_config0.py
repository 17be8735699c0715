"""The plain-method vortex case on the GPU and the observed L2 convergence order of the GPU path.

- Config 0: 2D Euler isentropic vortex, 16x16 QUAD p=2, Roe-Pike, SSP-RK3 at CFL 0.4 to t = 10 (dt rounded down
  to a whole number of steps, the same steps for the oracle): the FP64 form's final state against the
  oracle's, and the L2 errors against the exact advected vortex of both GPU forms against the oracle's
  ("within 1e-10 relative of the FP64 oracle": FP64 form 1e-10, S = 7 split precision 1e-8 for the L2 error
  values, the split state differing from the FP64 one at the 1e-10 level after ~700 steps).
- Convergence: the reference's criterion (test_integration_convergence_support.c:49,508-528: observed order
  >= p + 1 - 0.165) for the GPU path in both forms, QUAD p = 1..3 and HEX p = 2, 3.
"""
import math

import numpy as np
import pytest

import dpgsolver_gb300 as dg
from oracle import Oracle

pytestmark = pytest.mark.gpu


def test_config0_to_t10():
    cfg = dg.Config(d=2, p=2, n_elem=(16, 16, 1))
    sim = dg.Simulation(cfg)
    u0 = sim.sol_coef()
    dt = sim.cfl_dt(0.4, 10.0 / 16)
    t_final = 10.0
    n_steps = int(math.ceil(t_final / dt))
    dt = t_final / n_steps

    o = u0.copy()
    Oracle(sim).rk_step(o, dt, n_steps)
    sim.set_sol_coef(o)
    l2_ref = sim.l2_error(t_final)

    ctx = dg.GpuContext(sim)
    results = {}
    for name, mode, s in [("fp64", dg.PREC_FP64, 0), ("sliced7", dg.PREC_BF16_SLICED, 7)]:
        ctx.set_precision(mode, s)
        ctx.upload(u0)
        ctx.rk_step(dt, n_steps)
        u = ctx.download()
        sim.set_sol_coef(u)
        results[name] = (u, sim.l2_error(t_final))
    u64, l2_64 = results["fp64"]
    assert np.max(np.abs(u64 - o)) <= 1e-10 * np.max(np.abs(o))
    assert np.max(np.abs(l2_64 - l2_ref) / l2_ref[np.argmax(l2_ref)]) <= 1e-10
    _, l2_s7 = results["sliced7"]
    assert np.max(np.abs(l2_s7 - l2_ref)) <= 1e-8 * np.max(l2_ref), (l2_s7, l2_ref)
    assert np.max(l2_ref) < 0.05   # the vortex is resolved: the errors compared are discretisation errors


def _l2_after(cfg, mode, s, t_final):
    sim = dg.Simulation(cfg)
    ctx = dg.GpuContext(sim)
    ctx.set_precision(mode, s)
    h = 10.0 / cfg.n_elem[0]
    dt = sim.cfl_dt(0.4, h)
    n_steps = int(math.ceil(t_final / dt))
    ctx.rk_step(t_final / n_steps, n_steps)
    sim.set_sol_coef(ctx.download())
    return sim.l2_error(t_final)[0]   # density


@pytest.mark.parametrize("prec", [(dg.PREC_FP64, 0), (dg.PREC_BF16_SLICED, 7)], ids=["fp64", "sliced7"])
@pytest.mark.parametrize("d,p", [(2, 1), (2, 2), (2, 3), (3, 2), (3, 3)])
def test_convergence_order(d, p, prec):
    ns = (8, 16, 32) if d == 2 else (6, 12, 24)
    e = []
    for n in ns:
        cfg = dg.Config(d=d, p=p, n_elem=(n, n, 2), lo=(-5.0, -5.0, 0.0), hi=(5.0, 5.0, 2.5))
        e.append(_l2_after(cfg, *prec, 0.5))
    order = math.log(e[1] / e[2], 2)
    assert order >= p + 1 - 0.165, (d, p, e, order)
