"""The GPU's analytic linearisation against the oracle's complex-step derivatives.

dpg_gpu_jacobian_apply carries forward-mode tangents through the FP64 formulas; the oracle evaluates its own residual
on complex states, Im F(u + i h v) / h with h = 1e-30 (oracle_cs.c).  Both are exact to rounding, so they agree at
the level of the reference's linearisation test, which compares its assembled Jacobians with complex-step ones at
4e-13 (test_integration_linearization.c).  Cases: the periodic Euler path (Roe-Pike, Lax-Friedrichs; straight and
jittered QUAD/HEX), linear advection (upwind), the general chain with slip-wall and Riemann boundaries, and BR2
Navier-Stokes on the curved annulus with rotating and adiabatic no-slip walls.  The state is the oracle's initial
state with a seeded additive perturbation: away from the kinks of |lambda| where both sides' traces agree, and with
no velocity exactly at rest at a wall, where a branch of the entropy fix would be decided by rounding."""
import numpy as np
import pytest

import dpgsolver_gb300 as dg
from oracle import Oracle

pytestmark = pytest.mark.gpu

TOL = 4e-13   # test_integration_linearization.c: complex-step vs assembled Jacobian

CASES = {
    "quad-p3-roe-jittered": dict(d=2, p=3, n_elem=(4, 4, 1), jitter=0.1, seed=2),
    "quad-p2-lf": dict(d=2, p=2, n_elem=(4, 3, 1), num_flux="Lax-Friedrichs"),
    "hex-p2-roe": dict(d=3, p=2, n_elem=(3, 2, 2)),
    "hex-p1-lf-jittered": dict(d=3, p=1, n_elem=(3, 3, 2), num_flux="Lax-Friedrichs", jitter=0.1, seed=5),
    "advection-p3-upwind": dict(d=2, p=3, n_elem=(4, 4, 1), pde="advection", num_flux="upwind",
                                test_case="advection_sine", lo=(0, 0, 0), hi=(1, 1, 1)),
    "walls-riemann-slip": dict(d=2, p=3, n_elem=(4, 3, 1), lo=(0, 0, 0), hi=(2, 1, 1), jitter=0.1, seed=2,
                               test_case="free_stream", vortex=(0, 0, 0, 1.0, 0.7, 0.3, 0, 1.0),
                               bc=("riemann", "riemann", "slipwall", "riemann"), bc_state=(1.0, 0.7, 0.3, 0.0, 1.0)),
    "hex-slip-walls": dict(d=3, p=2, n_elem=(2, 3, 2), lo=(0, 0, 0), hi=(1, 1, 1), jitter=0.1, seed=2,
                           test_case="free_stream", vortex=(0, 0, 0, 1.0, 0.0, 0.3, 0.2, 1.0),
                           bc=("slipwall", "slipwall") + ("periodic",) * 4),
    "ns-annulus-p2": dict(d=2, p=2, n_elem=(3, 12, 1), mesh="annulus", lo=(1.0, 0, 0), hi=(2.0, 0, 0),
                          pde="navier_stokes", mu=5e-3, Pr=0.72, omega=0.5, test_case="taylor_couette",
                          bc=("noslip_all_rotating", "noslip_adiabatic")),
    "ns-hex-p2-walls": dict(d=3, p=2, n_elem=(3, 2, 2), lo=(0, 0, 0), hi=(1, 1, 1), jitter=0.1, seed=4,
                            pde="navier_stokes", mu=1e-2, test_case="isentropic_vortex",
                            vortex=(0.5, 0.5, 0.5, 1.0, 0.3, 0.2, 0.1, 1.0),
                            bc=("periodic",) * 4 + ("noslip_adiabatic", "noslip_adiabatic")),
    "ns-annulus-p3": dict(d=2, p=3, n_elem=(2, 8, 1), mesh="annulus", lo=(1.0, 0, 0), hi=(2.0, 0, 0),
                          pde="navier_stokes", mu=5e-2, Pr=0.72, omega=0.5, test_case="taylor_couette",
                          bc=("noslip_all_rotating", "noslip_adiabatic")),
}


@pytest.mark.parametrize("case", list(CASES.values()), ids=list(CASES))
def test_jacobian_vector_product_matches_complex_step(case):
    sim = dg.Simulation(dg.Config(**case))
    orc = Oracle(sim)
    ctx = dg.GpuContext(sim)
    rng = np.random.default_rng(11)
    u0 = orc.initial_solution()
    u = u0 + 1e-2 * np.max(np.abs(u0)) * rng.standard_normal(u0.shape)
    ctx.upload(u)
    for k in range(2):
        v = rng.standard_normal(u.shape) * (np.abs(u) if k else 1.0)
        jv = ctx.jacobian_apply(v)
        cs, f = orc.jvp_complex_step(u, v)
        err = np.max(np.abs(jv - cs)) / np.max(np.abs(cs))
        assert err <= TOL, (k, err)
    # the complex evaluation's real part is the oracle's residual
    _, r = orc.compute_rhs(u)
    assert np.max(np.abs(f - r)) <= 1e-13 * np.max(np.abs(r))
