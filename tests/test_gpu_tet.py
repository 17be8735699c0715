"""TET elements on the GPU: 3D linear advection with the upwind flux on periodic jittered boxes of cells split into
six tetrahedra, against the oracle's own TET set-up (barycentric-monomial basis, Stroud's conical product rule, a
symmetrised face rule, its own mesh and geometry).

- FP64 residual and SSP-RK3 steps <= 1e-11 relative for p = 1..4, and on a mesh of orders 1..4 (`kernels_hp.cu`);
- the split-precision (tcgen05) path for p = 1, 2, 3 (the shapes of its compiled instantiations): S = 7 residual
  within 1e-10 of the oracle;
- the GPU path's L2 error converges at order >= p + 1 - 0.165 for p = 1, 2."""
import numpy as np
import pytest

import dpgsolver_gb300 as dg
from oracle import Oracle

pytestmark = pytest.mark.gpu


def _cfg(p, n=(4, 3, 3), **kw):
    return dg.Config(d=3, p=p, n_elem=n, element="tet", pde="advection", num_flux="upwind", test_case="advection_sine",
                     lo=(0, 0, 0), hi=(1, 1, 1), jitter=0.1, seed=3, b_adv=(1.0, 0.5, 0.25), **kw)


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("p,p_max", [(1, 0), (2, 0), (3, 0), (4, 0), (1, 4)], ids=["p1", "p2", "p3", "p4", "p1-4"])
def test_tet_residual_and_steps_match_the_oracle(p, p_max):
    cfg = _cfg(p, p_max=p_max, p_seed=4)
    sim = dg.Simulation(cfg)
    orc = Oracle(cfg)
    u = orc.initial_solution()
    ctx = dg.GpuContext(sim)
    ctx.upload(u)
    m = ctx.compute_rhs()
    m_ref, r_ref = orc.compute_rhs(u)
    assert _rel(ctx.rhs(), r_ref) <= 1e-11
    assert abs(m - m_ref) <= 1e-11 * m_ref
    ctx.rk_step(1e-3, 3)
    orc.rk_step(u, 1e-3, 3)
    assert _rel(ctx.download(), u) <= 1e-11


@pytest.mark.parametrize("p", [1, 2, 3])
def test_tet_split_precision(p):
    cfg = _cfg(p)
    sim = dg.Simulation(cfg)
    orc = Oracle(cfg)
    u = orc.initial_solution()
    _, r_ref = orc.compute_rhs(u)
    ctx = dg.GpuContext(sim)
    ctx.set_precision(dg.PREC_BF16_SLICED, 7)
    ctx.upload(u)
    ctx.compute_rhs()
    assert _rel(ctx.rhs(), r_ref) <= 1e-10


@pytest.mark.parametrize("p", [1, 2])
def test_tet_gpu_convergence_order(p):
    errs = []
    for n in (6, 12):
        sim = dg.Simulation(_cfg(p, (n, n, n)))
        ctx = dg.GpuContext(sim)
        tf = 0.05
        dt = 0.1 * (1.0 / n) / (1.2 * (2 * p + 1))
        ns = int(np.ceil(tf / dt))
        ctx.rk_step(tf / ns, ns)
        sim.set_sol_coef(ctx.download())
        errs.append(sim.l2_error(tf)[0])
    order = np.log2(errs[0] / errs[1])
    assert order >= p + 1 - 0.165, (errs, order)
