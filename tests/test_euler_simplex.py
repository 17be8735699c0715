"""The Euler equations on TRI and TET volumes (periodic isentropic vortex on jittered split boxes), CPU checks.

- the Bezier operators of the positivity limiter on simplices: ccBS0 holds the Bernstein polynomials of degree p at
  the solution nodes (the basis of constructor_basis_si_bezier, bases.c:572-608: nonnegative, a partition of unity,
  equal as sets per node to B_a(l) = p!/a! l^a evaluated here), ccSB0 its inverse;
- the oracle's own set-up (its own nodes, bases, geometry and faces) with the reference's Witherden-Vincent rules
  (TRI volumes p <= 4, TET volumes p <= 3 and faces, from the golden fixture; the Euler integrands are not polynomial,
  so the rule is part of the discretisation) gives the library's residual (5e-12, 2e-11 at p = 4 where the two
  bases' Vandermonde matrices round differently); TET p = 4 with the library's
  collapsed volume rule handed to the oracle."""
import ctypes as C
import itertools
from math import factorial

import numpy as np
import pytest

import dpgsolver_gb300 as dg
from oracle import Oracle, Problem
from tests_support import DpgSim, oracle_rules, sim_arrays

CASES = [("tri", p) for p in (1, 2, 3, 4)] + [("tet", p) for p in (1, 2, 3, 4)]
IDS = [f"{e}-p{p}" for e, p in CASES]


def cfg(element, p, n=None, **kw):
    d = 2 if element == "tri" else 3
    n = n or ((6, 6, 1) if d == 2 else (6, 6, 3))   # TET: at 3 x 3 x 2 cells the p >= 2 interpolant of the vortex
                                                       # has negative Bezier pressure averages (the reference stops)
    return dict(d=d, p=p, n_elem=n, element=element, pde="euler", num_flux="Roe-Pike", test_case="isentropic_vortex",
                lo=(-5, -5, 0), hi=(5, 5, 1 if d == 2 else 2.5), jitter=0.1, seed=3, **kw)


def _bary(element, x):
    s3, s6 = np.sqrt(3.0), np.sqrt(6.0)
    V = (np.array([[-1.0, -1 / s3], [1.0, -1 / s3], [0.0, 2 / s3]]) if element == "tri" else
         np.array([[-1.0, -1 / s3, -1 / s6], [1.0, -1 / s3, -1 / s6], [0.0, 2 / s3, -1 / s6], [0.0, 0.0, 3 / s6]]))
    l = np.linalg.solve((V[1:] - V[0]).T, (x - V[0]).T).T
    return np.column_stack([1 - l.sum(axis=1), l])


@pytest.mark.parametrize("element,p", CASES, ids=IDS)
def test_bezier_operators(element, p):
    sim = dg.Simulation(dg.Config(**cfg(element, p)))
    a = sim_arrays(sim)
    n_s, d = sim.n_s, sim.d
    BS, SB = a["ccBS0_vs_vs"].reshape(n_s, n_s), a["ccSB0_vs_vs"].reshape(n_s, n_s)
    assert np.min(BS) >= -1e-15 and np.max(np.abs(BS.sum(axis=1) - 1)) <= 1e-14
    assert np.max(np.abs(BS @ SB - np.eye(n_s))) <= 1e-11
    lam = _bary(element, a["rst_vs"].reshape(n_s, d))
    idx = [al for al in itertools.product(range(p + 1), repeat=d + 1) if sum(al) == p]
    ref = np.array([[factorial(p) / np.prod([factorial(k) for k in al]) * np.prod(l ** np.array(al)) for al in idx]
                    for l in lam])
    assert np.max(np.abs(np.sort(ref, axis=1) - np.sort(BS, axis=1))) <= 1e-13


@pytest.mark.parametrize("element,p", CASES, ids=IDS)
def test_oracle_set_up_gives_the_library_residual(element, p):
    c = cfg(element, p)
    sim = dg.Simulation(dg.Config(**c))
    own = Oracle(Problem(**c, **oracle_rules(element, p, sim)))
    u = sim.sol_coef()
    assert np.max(np.abs(own.initial_solution() - u)) <= 1e-13
    _, r1 = own.compute_rhs(u)
    _, r2 = Oracle(data_model=dg.load_library().dpg_sim_view(sim.handle)).compute_rhs(u)
    tol = 2e-11 if p == 4 else 5e-12   # order 4: the two bases' Vandermonde matrices round differently
    assert np.max(np.abs(r1 - r2)) <= tol * np.max(np.abs(r1))


def test_refusals():
    with pytest.raises(dg.DpgError):   # boundary faces: the simplex meshes are periodic boxes
        dg.Simulation(dg.Config(**cfg("tri", 2, bc=("slipwall",) * 4)))
