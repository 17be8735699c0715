"""Analytic linearisation of the residual on the GPU (forward-mode tangents of the FP64 formulas).

The reference checks its assembled Jacobians against complex-step derivatives (test_integration_linearization, 4e-13
relative).  Here dF/du . v (F = m_inv rhs) from dpg_gpu_jacobian_apply is checked
- exactly, by Euler's theorem: the Euler flux, the Roe-Pike and Lax-Friedrichs fluxes and the linear advection flux
  are homogeneous of degree 1 in the conservative state, so J(u) u = F(u) (scaling the state changes neither the
  velocity nor the sound speed: no branch switches along u);
- against central differences of the FP64 residual along random directions (truncation ~h^2: a 1e-7 bound);
- for exact linearity in v; and in the implicit solver:
the tangent Jacobian converges the steady free-stream problem in no more Newton steps than the finite-difference
one, to the same state.

The comparison state is the initial solution plus a small random perturbation: the interpolated initial state has
identical traces on both sides of every face, where the Roe-Pike |lambda| and the Lax-Friedrichs max wave speed sit
exactly on their kinks (C^1 but not C^2 there), so central differences would converge only to first order.
"""
import numpy as np
import pytest

import dpgsolver_gb300 as dg

pytestmark = pytest.mark.gpu

CASES = [
    dict(d=2, p=2, n_elem=(4, 4, 1)),                                   # Euler, Roe-Pike
    dict(d=2, p=3, n_elem=(3, 3, 1), num_flux="Lax-Friedrichs"),
    dict(d=3, p=1, n_elem=(3, 3, 2)),
    dict(d=3, p=2, n_elem=(2, 2, 2), num_flux="Lax-Friedrichs"),
    dict(d=2, p=3, n_elem=(4, 4, 1), pde="advection", num_flux="upwind", test_case="advection_sine",
         lo=(0, 0, 0), hi=(1, 1, 1)),
]


def _residual(ctx, u):
    ctx.upload(u)
    ctx.compute_rhs()
    return ctx.rhs()


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"d{c['d']}-p{c['p']}-{c.get('num_flux', 'Roe-Pike')}")
def test_jacobian_matches_central_differences(case):
    sim = dg.Simulation(dg.Config(**case))
    ctx = dg.GpuContext(sim)
    rng = np.random.default_rng(3)
    u0 = sim.sol_coef()
    u = u0 + 1e-3 * np.max(np.abs(u0)) * rng.standard_normal(u0.shape)   # a generic state (see above)
    v = rng.standard_normal(u.shape)
    ctx.upload(u)
    jv = ctx.jacobian_apply(v)
    h = 1e-5 * np.max(np.abs(u)) / np.max(np.abs(v))
    fd = (_residual(ctx, u + h * v) - _residual(ctx, u - h * v)) / (2 * h)
    err = np.max(np.abs(jv - fd)) / np.max(np.abs(jv))
    assert err <= 1e-7, err


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"d{c['d']}-p{c['p']}-{c.get('num_flux', 'Roe-Pike')}")
def test_jacobian_times_state_is_the_residual(case):
    sim = dg.Simulation(dg.Config(**case))
    ctx = dg.GpuContext(sim)
    u0 = sim.sol_coef()
    u = u0 + 1e-2 * np.max(np.abs(u0)) * np.random.default_rng(11).standard_normal(u0.shape)
    F = _residual(ctx, u)
    ju = ctx.jacobian_apply(u)
    # rounding of the O(|terms|) sums: relative to the largest term of F, not to F (which may be small)
    ref = np.max(np.abs(ctx.jacobian_apply(np.abs(u)))) + np.max(np.abs(F))
    assert np.max(np.abs(ju - F)) <= 1e-12 * ref


def test_jacobian_is_linear_in_the_direction():
    sim = dg.Simulation(dg.Config(d=2, p=2, n_elem=(4, 4, 1)))
    ctx = dg.GpuContext(sim)
    ctx.upload(sim.sol_coef())
    rng = np.random.default_rng(5)
    v, w = rng.standard_normal((2, sim.sol_coef().size))
    jv, jw = ctx.jacobian_apply(v), ctx.jacobian_apply(w)
    assert np.array_equal(ctx.jacobian_apply(2.0 * v), 2.0 * jv)   # power-of-two scaling is exact
    jvw = ctx.jacobian_apply(v + w)
    assert np.max(np.abs(jvw - (jv + jw))) <= 1e-12 * np.max(np.abs(jvw))


def test_newton_with_the_tangent_jacobian():
    from test_gpu_implicit import _problem, _oracle_residual
    sim, ctx, u_star, forcing, u0 = _problem()
    res = {}
    for name, jac in (("tangent", dg.JACOBIAN_TANGENT), ("fd", dg.JACOBIAN_FD)):
        ctx.upload(u0)
        st = ctx.newton_solve(dg.PRECOND_BLOCK_JACOBI, tol=1e-10, forcing=forcing, dtau0=10.0, max_newton=40,
                              jacobian=jac)
        assert st.residual_final <= 1e-10, name
        res[name] = (st.newton_iterations, st.gmres_iterations, ctx.download())
    assert res["tangent"][0] <= res["fd"][0]
    assert _oracle_residual(sim, res["tangent"][2], forcing) <= 1e-9
    # both solves reach the same steady state
    assert np.max(np.abs(res["tangent"][2] - res["fd"][2])) <= 1e-8 * np.max(np.abs(u_star))
