"""TRI elements on the GPU (FP64 path): 2D linear advection with the upwind flux on periodic jittered boxes of cells
split into two triangles, against the oracle's own TRI set-up (monomial Vandermonde basis, its own nodes, cubature
and geometry) on the same parameters.

- residual <= 1e-11 relative (max-norm), p = 1..4, and at the advection configuration's size (64 x 64 cells =
  8,192 triangles, jitter 0.1 h);
- SSP-RK3 steps <= 1e-11;
- the GPU path's L2 error converges at order >= p + 1 - 0.165 (the reference's criterion) for p = 1, 2, 3;
- the split-precision (tcgen05) modes on TRI meet the tensor-product meshes' tolerances against the oracle (S = 7:
  1e-10), up to 8,192 triangles."""
import numpy as np
import pytest

import dpgsolver_gb300 as dg
from oracle import Oracle

pytestmark = pytest.mark.gpu


def _cfg(p, n=(6, 5), jitter=0.1, seed=3):
    return dg.Config(d=2, p=p, n_elem=(n[0], n[1], 1), element="tri", pde="advection", num_flux="upwind",
                     test_case="advection_sine", lo=(0, 0, 0), hi=(1, 1, 1), jitter=jitter, seed=seed,
                     b_adv=(1.0, 0.5, 0.0))


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_tri_residual_and_steps_match_the_oracle(p):
    cfg = _cfg(p)
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


def test_tri_at_the_configuration_size():
    cfg = _cfg(3, (64, 64), seed=7)
    sim = dg.Simulation(cfg)
    orc = Oracle(cfg, threads=16)
    u = orc.initial_solution()
    ctx = dg.GpuContext(sim)
    ctx.upload(u)
    ctx.compute_rhs()
    _, r_ref = orc.compute_rhs(u)
    assert sim.n_vol == 8192
    assert _rel(ctx.rhs(), r_ref) <= 1e-11


@pytest.mark.parametrize("p", [1, 2, 3])
def test_tri_gpu_convergence_order(p):
    errs = []
    for n in (8, 16):
        sim = dg.Simulation(_cfg(p, (n, n)))
        ctx = dg.GpuContext(sim)
        tf = 0.1
        dt = 0.1 * (1.0 / n) / (1.2 * (2 * p + 1))
        ns = int(np.ceil(tf / dt))
        ctx.rk_step(tf / ns, ns)
        sim.set_sol_coef(ctx.download())
        errs.append(sim.l2_error(tf)[0])
    order = np.log2(errs[0] / errs[1])
    assert order >= p + 1 - 0.165, (errs, order)


SPLIT_MODES = [("sliced7", dg.PREC_BF16_SLICED, 7, 1e-10), ("sliced5", dg.PREC_BF16_SLICED, 5, 1e-8),
               ("tf32x3", dg.PREC_TF32X3, 0, 1e-3), ("bf16x3", dg.PREC_BF16X3, 0, 5e-3)]


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_tri_split_precision_matches_the_oracle(p):
    """The tensor-core path on triangles (the operators are dense, any element type of one order): residuals of the
    split modes against the oracle with the tolerances of the tensor-product meshes, S = 7 SSP-RK3 steps within
    1e-10 (odd face-node counts per element: the trace rows start on 8-byte boundaries)."""
    cfg = _cfg(p)
    sim = dg.Simulation(cfg)
    orc = Oracle(cfg)
    u = orc.initial_solution()
    _, r_ref = orc.compute_rhs(u)
    ctx = dg.GpuContext(sim)
    for name, mode, s, tol in SPLIT_MODES:
        ctx.set_precision(mode, s)
        ctx.upload(u)
        ctx.compute_rhs()
        assert _rel(ctx.rhs(), r_ref) <= tol, (name, p)
    ctx.set_precision(dg.PREC_BF16_SLICED, 7)
    ctx.upload(u)
    ctx.rk_step(1e-3, 3)
    u2 = u.copy()
    orc.rk_step(u2, 1e-3, 3)
    assert _rel(ctx.download(), u2) <= 1e-10


def test_tri_split_at_the_configuration_size():
    cfg = _cfg(4, (64, 64), seed=7)
    sim = dg.Simulation(cfg)
    orc = Oracle(cfg, threads=16)
    u = orc.initial_solution()
    ctx = dg.GpuContext(sim)
    ctx.set_precision(dg.PREC_BF16_SLICED, 7)
    ctx.upload(u)
    ctx.compute_rhs()
    _, r_ref = orc.compute_rhs(u)
    assert _rel(ctx.rhs(), r_ref) <= 1e-10
