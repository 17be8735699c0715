"""Checks of the oracle's boundary conditions and Navier-Stokes (BR2) restatement that need no library.

* Free-stream preservation: a uniform flow parallel to slip walls, or matching the Riemann boundary's external
  state, has a zero residual (to rounding) on jittered meshes, as in test_integration_free_stream.
* Taylor-Couette: the residual of the BR2 discretisation on the curved annulus, evaluated at the interpolated steady
  solution of the compressible equations (velocity c (1/r - r/r_o^2), the reference's temperature profile, and the
  pressure of the radial balance dp/dr = rho V^2 / r, integrated here by Gauss-Legendre quadrature), converges under
  refinement at an order near p.  The reference's own Taylor-Couette solution keeps the pressure uniform
  (solution_taylor_couette_T.c notes it is "nearly uniform"); it is not a steady state of the compressible
  equations, and the residual there stays at rho V^2 / r.
"""
import numpy as np
import pytest

from oracle import Oracle, Problem
from oracle import oracle_layout as L

RI, RO, OMEGA, MU, PR, GAMMA = 1.0, 2.0, 0.5, 5e-3, 0.72, 1.4


@pytest.mark.parametrize("bc", [("periodic", "periodic", "slipwall", "slipwall"),
                                ("periodic", "periodic", "riemann", "riemann"),
                                ("riemann", "riemann", "slipwall", "riemann")])
def test_free_stream_preserved_with_walls(bc):
    pr = Problem(d=2, p=3, n_elem=(4, 3, 1), lo=(0, 0, 0), hi=(2, 1, 1), jitter=0.1, seed=2, test_case="free_stream",
                 vortex=(0, 0, 0, 1.0, 0.7, 0.0, 0, 1.0), bc=bc, bc_state=(1.0, 0.7, 0.0, 0.0, 1.0))
    o = Oracle(pr)
    m, _ = o.compute_rhs(o.initial_solution())
    assert m < 1e-12


def test_free_stream_preserved_3d_slip_walls():
    pr = Problem(d=3, p=2, n_elem=(2, 3, 2), lo=(0, 0, 0), hi=(1, 1, 1), jitter=0.1, seed=2, test_case="free_stream",
                 vortex=(0, 0, 0, 1.0, 0.0, 0.3, 0.2, 1.0), bc=("slipwall", "slipwall") + ("periodic",) * 4)
    o = Oracle(pr)
    m, _ = o.compute_rhs(o.initial_solution())
    assert m < 1e-12


def _tc_problem(p, n):
    return Problem(d=2, p=p, n_elem=(n, 4 * n, 1), mesh="annulus", lo=(RI, 0, 0), hi=(RO, 0, 0), pde="navier_stokes",
                   mu=MU, Pr=PR, omega=OMEGA, test_case="taylor_couette", bc=("noslip_all_rotating", "noslip_adiabatic"))


def tc_steady_state(orc):
    """The compressible Taylor-Couette steady state at the oracle's solution nodes (sol_coef layout)."""
    c = OMEGA / (1 / RI ** 2 - 1 / RO ** 2)
    kappa = MU * (GAMMA / (GAMMA - 1)) / PR
    vt = lambda r: c * (1 / r - r / RO ** 2)
    temp = lambda r: 1.0 - 2 * c * c / RO ** 2 * MU / kappa * np.log(r / RI) - c * c * MU / kappa * (1 / r ** 2 - 1 / RI ** 2)
    xg, wg = np.polynomial.legendre.leggauss(40)

    def logp(r):
        x = 0.5 * (r - RI) * xg + 0.5 * (r + RI)
        return 0.5 * (r - RI) * np.sum(wg * vt(x) ** 2 / (temp(x) * x))

    A = L.arrays(orc.model)
    rst, ve = A["rst_vs"], A["xyz_ve"][:, :4, :2]
    w = lambda k, r: 0.5 * (1 + r) if k else 0.5 * (1 - r)
    phi = np.array([[w(k & 1, x[0]) * w(k >> 1, x[1]) for k in range(4)] for x in rst])
    rr, tt = phi @ ve[:, :, 0].T, phi @ ve[:, :, 1].T
    pres = np.exp(np.vectorize(logp)(rr))
    rho, v = pres / temp(rr), vt(rr)
    u = np.stack([rho, -rho * np.sin(tt) * v, rho * np.cos(tt) * v, pres / (GAMMA - 1) + 0.5 * rho * v * v])
    return np.ascontiguousarray(u.transpose(2, 0, 1).reshape(-1))


@pytest.mark.parametrize("p,order", [(2, 1.5), (3, 2.7)])
def test_taylor_couette_residual_converges(p, order):
    res = []
    for n in (4, 8, 16):
        o = _tc_problem(p, n)
        orc = Oracle(o)
        m, _ = orc.compute_rhs(tc_steady_state(orc))
        res.append(m)
    rates = np.log2(np.array(res[:-1]) / np.array(res[1:]))
    assert np.all(rates > order), (res, rates)


def test_uniform_pressure_solution_is_not_steady():
    """The reference's Taylor-Couette initial state leaves the radial balance out: residual ~ rho V^2 / r."""
    orc = Oracle(_tc_problem(3, 8))
    m, _ = orc.compute_rhs(orc.initial_solution())
    assert 0.2 < m < 0.3


@pytest.mark.parametrize("case", [
    dict(d=2, p=3, n_elem=(3, 3, 1), jitter=0.1, seed=2),
    dict(d=3, p=2, n_elem=(2, 2, 2), num_flux="Lax-Friedrichs"),
    dict(d=2, p=2, n_elem=(4, 3, 1), lo=(0, 0, 0), hi=(2, 1, 1), test_case="free_stream",
         vortex=(0, 0, 0, 1.0, 0.7, 0.3, 0, 1.0), bc=("riemann", "riemann", "slipwall", "riemann"),
         bc_state=(1.0, 0.7, 0.3, 0.0, 1.0)),
    dict(d=2, p=2, n_elem=(2, 8, 1), mesh="annulus", lo=(RI, 0, 0), hi=(RO, 0, 0), pde="navier_stokes", mu=MU, Pr=PR,
         omega=OMEGA, test_case="taylor_couette", bc=("noslip_all_rotating", "noslip_adiabatic"))],
    ids=["quad-roe", "hex-lf", "riemann-slip", "ns-annulus"])
def test_complex_step_linearisation(case):
    """The oracle's complex-step product (oracle_cs.c): real part = the residual, linear in v, and the limit of
    central differences (the error falls ~4x when h halves).  The state is perturbed additively, so that no
    velocity sits exactly at zero: at a wall where the flow is at rest the Roe-Pike entropy fix switches at the
    state itself (a term like |V_n| V_n), and central differences converge only at first order there; the flow
    crosses the Riemann boundaries (no switch between inflow and outflow states within the differences)."""
    orc = Oracle(Problem(**case))
    rng = np.random.default_rng(1)
    u0 = orc.initial_solution()
    u = u0 + 1e-2 * np.max(np.abs(u0)) * rng.standard_normal(u0.shape)
    v, w = rng.standard_normal(u.shape), rng.standard_normal(u.shape)
    jv, f = orc.jvp_complex_step(u, v)
    jw, _ = orc.jvp_complex_step(u, w)
    jvw, _ = orc.jvp_complex_step(u, 2.0 * v - 3.0 * w)
    _, r = orc.compute_rhs(u)
    scale = np.max(np.abs(jv))
    assert np.max(np.abs(f - r)) <= 1e-14 * np.max(np.abs(r))
    assert np.max(np.abs(jvw - (2.0 * jv - 3.0 * jw))) <= 1e-13 * scale
    errs = []
    for h in (2e-5, 1e-5):
        fd = (orc.compute_rhs(u + h * v)[1] - orc.compute_rhs(u - h * v)[1]) / (2 * h)
        errs.append(np.max(np.abs(fd - jv)) / scale)
    assert errs[1] < 1e-5 and 3.0 < errs[0] / errs[1] < 5.0, errs
