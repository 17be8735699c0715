"""Mixed orders on the GPU (kernels_hp.cu: volumes grouped by order, three launches per residual), 2D linear
advection with the upwind flux on periodic jittered meshes, against the oracle's own mixed-order set-up.

- residual <= 1e-11 relative (max-norm) and SSP-RK3 steps <= 1e-11 on TRI and QUAD meshes with orders 1..4 and
  HEX meshes with orders 1..3;
- at the advection configuration's size (64 x 64 cells split into 8,192 TRIs, jitter 0.1 h, orders uniform in
  {1, 2, 3, 4}) the residual <= 1e-11;
- the GPU path's L2 error converges at order >= p_min + 1 - 0.165 with orders drawn from {p_min, p_min + 1};
- split precision, the linearisation and the implicit solve are refused (one-order meshes only)."""
import numpy as np
import pytest

import dpgsolver_gb300 as dg
from oracle import Oracle

pytestmark = pytest.mark.gpu


def _cfg(element, p, p_max, n, jitter=0.1, seed=3, p_seed=11):
    return dg.Config(d=2, p=p, p_max=p_max, p_seed=p_seed, n_elem=(n[0], n[1], 1), element=element, pde="advection",
                     num_flux="upwind", test_case="advection_sine", lo=(0, 0, 0), hi=(1, 1, 1), jitter=jitter,
                     seed=seed, b_adv=(1.0, 0.5, 0.0))


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("element,n", [("tri", (7, 6)), ("tp", (6, 5))])
def test_residual_and_steps_match_the_oracle(element, n):
    cfg = _cfg(element, 1, 4, n)
    sim = dg.Simulation(cfg)
    orc = Oracle(cfg)
    u = orc.initial_solution()
    ctx = dg.GpuContext(sim)
    ctx.upload(u)
    m = ctx.compute_rhs()
    m_ref, r_ref = orc.compute_rhs(u)
    assert _rel(ctx.rhs(), r_ref) <= 1e-11
    assert abs(m - m_ref) <= 1e-11 * m_ref
    dt = 1e-3
    ctx.rk_step(dt, 3)
    orc.rk_step(u, dt, 3)
    assert _rel(ctx.download(), u) <= 1e-11


def test_hex_mixed_orders_match_the_oracle():
    kw = dict(d=3, p=1, p_max=3, p_seed=4, n_elem=(4, 3, 3), lo=(0, 0, 0), hi=(1, 1, 1), pde="advection",
              num_flux="upwind", test_case="advection_sine", jitter=0.1, seed=3, b_adv=(1.0, 0.5, 0.25))
    cfg = dg.Config(**kw)
    sim = dg.Simulation(cfg)
    orc = Oracle(cfg)
    u = orc.initial_solution()
    ctx = dg.GpuContext(sim)
    ctx.upload(u)
    ctx.compute_rhs()
    _, r_ref = orc.compute_rhs(u)
    assert _rel(ctx.rhs(), r_ref) <= 1e-11
    ctx.rk_step(1e-3, 2)
    orc.rk_step(u, 1e-3, 2)
    assert _rel(ctx.download(), u) <= 1e-11


def test_at_the_configuration_size():
    cfg = _cfg("tri", 1, 4, (64, 64), seed=7, p_seed=5)
    sim = dg.Simulation(cfg)
    orc = Oracle(cfg, threads=16)
    u = orc.initial_solution()
    ctx = dg.GpuContext(sim)
    ctx.upload(u)
    ctx.compute_rhs()
    _, r_ref = orc.compute_rhs(u)
    assert sim.n_vol == 8192
    assert _rel(ctx.rhs(), r_ref) <= 1e-11


@pytest.mark.parametrize("element,p", [("tri", 1), ("tri", 2), ("tp", 2)])
def test_gpu_convergence_order(element, p):
    errs = []
    for n in (8, 16):
        sim = dg.Simulation(_cfg(element, p, p + 1, (n, n)))
        ctx = dg.GpuContext(sim)
        tf = 0.1
        dt = 0.1 * (1.0 / n) / (1.2 * (2 * (p + 1) + 1))
        ns = int(np.ceil(tf / dt))
        ctx.rk_step(tf / ns, ns)
        sim.set_sol_coef(ctx.download())
        errs.append(sim.l2_error(tf)[0])
    order = np.log2(errs[0] / errs[1])
    assert order >= p + 1 - 0.165, (errs, order)


def test_refusals():
    ctx = dg.GpuContext(dg.Simulation(_cfg("tp", 1, 3, (4, 4))))
    with pytest.raises(dg.DpgError) as e:
        ctx.set_precision(dg.PREC_BF16_SLICED, 7)
    assert e.value.status == dg.api.DPG_ERR_UNSUPPORTED
    with pytest.raises(dg.DpgError) as e:
        ctx.newton_solve(dg.PRECOND_BLOCK_JACOBI, tol=1e-10)
    assert e.value.status == dg.api.DPG_ERR_UNSUPPORTED
