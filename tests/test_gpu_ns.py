"""The general FP64 chain (boundary faces, BR2 Navier-Stokes, curved annulus) on the GPU against the CPU oracle, which
builds the same problems with its own set-up.

Tolerances: residuals and RK states <= 1e-11 relative (max-norm), as for the periodic FP64 path.  Jacobian-vector
products (forward-mode tangents of the same kernels) against central differences of the ORACLE residual,
(F(u + h v) - F(u - h v)) / 2h with h = 1e-6 relative to the state: <= 1e-6 relative (the difference quotient's own
truncation and rounding error is ~1e-8 here).
"""
import numpy as np
import pytest

import dpgsolver_gb300 as dg
from oracle import Oracle

pytestmark = pytest.mark.gpu

TC = dict(d=2, mesh="annulus", lo=(1.0, 0, 0), hi=(2.0, 0, 0), pde="navier_stokes", mu=5e-3, omega=0.5,
          test_case="taylor_couette", bc=("noslip_all_rotating", "noslip_adiabatic"))
CASES = [
    dict(d=2, p=2, n_elem=(5, 4, 1), lo=(0, 0, 0), hi=(2, 1, 1), jitter=0.15, seed=3, bc=("periodic", "periodic", "slipwall", "slipwall")),
    dict(d=2, p=3, n_elem=(4, 4, 1), lo=(-5, -5, 0), hi=(5, 5, 1), bc=("riemann", "riemann", "slipwall", "riemann"),
         bc_state=(1.0, 1.0, 1.0, 0.0, 1.0), num_flux="Lax-Friedrichs"),
    dict(d=3, p=2, n_elem=(3, 2, 2), lo=(-5, -5, 0), hi=(5, 5, 2.5), jitter=0.1, seed=1,
         bc=("slipwall", "slipwall", "periodic", "periodic", "riemann", "riemann")),
    dict(TC, p=2, n_elem=(3, 12, 1)),
    dict(TC, p=3, n_elem=(4, 16, 1)),
    dict(d=2, p=3, n_elem=(4, 3, 1), lo=(0, 0, 0), hi=(1, 1, 1), jitter=0.1, seed=2, pde="navier_stokes", mu=1e-2,
         test_case="isentropic_vortex", vortex=(0.5, 0.5, 0.5, 1.0, 0.3, 0.0, 0.0, 1.0),
         bc=("periodic", "periodic", "noslip_adiabatic", "noslip_adiabatic")),
    dict(d=3, p=2, n_elem=(3, 2, 2), lo=(0, 0, 0), hi=(1, 1, 1), jitter=0.1, seed=4, pde="navier_stokes", mu=1e-2,
         test_case="isentropic_vortex", vortex=(0.5, 0.5, 0.5, 1.0, 0.3, 0.2, 0.1, 1.0),
         bc=("periodic",) * 4 + ("noslip_adiabatic", "noslip_adiabatic")),
]


def _ids(c):
    return f"{c.get('pde', 'euler')}-d{c['d']}-p{c['p']}-{c.get('mesh', 'box')}"


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _state(orc, seed=11, amp=1e-2):
    u = orc.initial_solution()
    return u * (1.0 + amp * np.random.default_rng(seed).standard_normal(u.shape))


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_general_residual_matches_oracle(case):
    sim = dg.Simulation(dg.Config(**case))
    orc = Oracle(sim)
    ctx = dg.GpuContext(sim)
    u = _state(orc)
    ctx.upload(u)
    m_gpu = ctx.compute_rhs()
    m_ref, r_ref = orc.compute_rhs(u)
    assert _rel(ctx.rhs(), r_ref) <= 1e-11
    assert abs(m_gpu - m_ref) <= 1e-11 * m_ref


@pytest.mark.parametrize("case", [CASES[0], CASES[4]], ids=["euler-walls", "ns-annulus"])
def test_general_rk_steps_match_oracle(case):
    sim = dg.Simulation(dg.Config(**case))
    orc = Oracle(sim)
    ctx = dg.GpuContext(sim)
    u = orc.initial_solution()
    ctx.upload(u)
    dt = 1e-3
    ctx.rk_step(dt, 3)
    ref = u.copy()
    orc.rk_step(ref, dt, 3)
    assert _rel(ctx.download(), ref) <= 1e-11


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_jacobian_vector_product_against_oracle_differences(case):
    sim = dg.Simulation(dg.Config(**case))
    orc = Oracle(sim)
    ctx = dg.GpuContext(sim)
    u = _state(orc, 5)
    ctx.upload(u)
    rng = np.random.default_rng(9)
    v = rng.standard_normal(u.shape) * np.abs(u)
    jv = ctx.jacobian_apply(v)
    h = 1e-6
    _, fp = orc.compute_rhs(u + h * v)
    _, fm = orc.compute_rhs(u - h * v)
    fd = (fp - fm) / (2 * h)
    assert _rel(jv, fd) <= 1e-6


def test_split_precision_refuses_the_general_chain():
    sim = dg.Simulation(dg.Config(**CASES[0]))
    ctx = dg.GpuContext(sim)
    with pytest.raises(dg.DpgError) as e:
        ctx.set_precision(dg.PREC_BF16_SLICED, 7)
    assert e.value.status == dg.api.DPG_ERR_UNSUPPORTED


def test_periodic_jvp_against_oracle_differences():
    """The periodic Euler path's tangents (kernels_fp64.cu) against the oracle's central differences."""
    for case in (dict(d=2, p=3, n_elem=(4, 4, 1), jitter=0.1, seed=2), dict(d=3, p=2, n_elem=(3, 3, 2))):
        sim = dg.Simulation(dg.Config(**case))
        orc = Oracle(sim)
        ctx = dg.GpuContext(sim)
        u = _state(orc, 7)
        ctx.upload(u)
        v = np.random.default_rng(4).standard_normal(u.shape) * np.abs(u)
        jv = ctx.jacobian_apply(v)
        h = 1e-6
        fd = (orc.compute_rhs(u + h * v)[1] - orc.compute_rhs(u - h * v)[1]) / (2 * h)
        assert _rel(jv, fd) <= 1e-6


def test_newton_taylor_couette_converges_to_the_oracle_steady_state():
    """Implicit Newton-GMRES (block-Jacobi) on the curved annulus from the reference's uniform-pressure initial state
    to ||F||_inf <= 1e-10; the oracle's residual at the converged state is at the same level."""
    cfg = dg.Config(**dict(TC, p=2, n_elem=(3, 12, 1)))
    sim = dg.Simulation(cfg)
    orc = Oracle(sim)
    ctx = dg.GpuContext(sim)
    ctx.upload(orc.initial_solution())
    st = ctx.newton_solve(dg.PRECOND_BLOCK_JACOBI, tol=1e-10, dtau0=1.0, max_newton=200)
    assert st.residual_final <= 1e-10
    m_ref, _ = orc.compute_rhs(ctx.download())
    assert m_ref <= 2e-10, m_ref
