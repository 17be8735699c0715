"""Positivity limiter and Newton under-relaxation: the Bezier operators of the host data model and the oracle's
restatement of enforce_positivity_highorder (solve.c:187-233) / compute_relaxation (solve_implicit.c:821-873),
checked against the Bernstein definition (bases.c:1013-1019) and an independent numpy restatement (CPU only)."""
import math

import numpy as np
import pytest

import dpgsolver_gb300 as dg
from oracle import Oracle
from positivity_support import (EPS_PHYS, bezier_prim_min, blocks, limit_volume, perturbed_state, relaxation)
from tests_support import sim_arrays

# vortex meshes whose initial Bezier coefficients are positive (on coarser 3D meshes, e.g. 3x3x3 p2, the interpolant's
# coefficients are not, and the limiter acts on the initial state itself: test_limiter_acts_on_a_coarse_interpolant)
CASES = [dict(d=2, p=2, n_elem=(6, 6, 1)), dict(d=2, p=4, n_elem=(4, 4, 1)), dict(d=3, p=2, n_elem=(6, 6, 2)),
         dict(d=3, p=3, n_elem=(6, 6, 2))]
IDS = [f"d{c['d']}-p{c['p']}" for c in CASES]
LIMITED_TOL = 1e-10   # two restatements of the limiter on volumes it corrects (see below)


def _bernstein(p, i, r):
    return math.comb(p, i) * (0.5 * (1 + r)) ** i * (0.5 * (1 - r)) ** (p - i)


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_bezier_operators(case):
    sim = dg.Simulation(dg.Config(**case))
    a = sim_arrays(sim)
    p, d, n1 = a["p"], a["d"], a["p"] + 1
    gll = a["rst_vs"][:n1, 0]   # the first n1 solution nodes run along x (GLL nodes, x index fastest)
    assert np.all(np.diff(gll) > 0) and gll[0] == -1.0 and gll[-1] == 1.0
    B1 = np.array([[_bernstein(p, i, r) for i in range(n1)] for r in gll])
    assert np.allclose(a["bez1"], B1, rtol=0, atol=1e-15)
    # tensor-product ordering of the reference (Bernstein index i fastest, as the solution nodes)
    BS = B1
    for _ in range(d - 1):
        BS = np.kron(B1, BS)
    assert np.allclose(a["ccBS0_vs_vs"], BS, rtol=0, atol=1e-15)
    assert np.allclose(a["ccBS0_vs_vs"].sum(axis=1), 1.0, rtol=0, atol=1e-14)   # partition of unity
    n_s = a["ccBS0_vs_vs"].shape[0]
    assert np.allclose(a["ccSB0_vs_vs"] @ a["ccBS0_vs_vs"], np.eye(n_s), rtol=0, atol=1e-12)
    assert np.allclose(a["bez1_inv"] @ a["bez1"], np.eye(n1), rtol=0, atol=1e-13)


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_oracle_limiter_on_a_positive_state_is_a_round_trip(case):
    sim = dg.Simulation(dg.Config(**case))
    u = sim.sol_coef().copy()
    u0 = u.copy()
    assert Oracle(sim).enforce_positivity(u) == 0
    assert np.max(np.abs(u - u0)) <= 1e-13 * np.max(np.abs(u0))


@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_oracle_limiter_matches_numpy_and_restores_positivity(case):
    sim = dg.Simulation(dg.Config(**case))
    a = sim_arrays(sim)
    SB, BS, d = a["ccSB0_vs_vs"], a["ccBS0_vs_vs"], sim.d
    u, picked = perturbed_state(sim)
    before = [bezier_prim_min(blocks(sim, u)[e], SB, d) for e in picked]
    assert all(min(m) < 0.0 for m in before)          # every perturbed volume needs the limiter
    ref = u.copy()
    rb = blocks(sim, ref)
    for e in range(sim.n_vol):
        rb[e], ok = limit_volume(rb[e], SB, BS, d)
        assert ok
    ora = u.copy()
    assert Oracle(sim).enforce_positivity(ora) == 0
    scale = np.max(np.abs(u))
    # the density correction leaves a coefficient at density EPS_PHYS, where the primitive velocity m / rho carries
    # the rounding of rho (1e-16 absolute) at 1e-3 relative into the pressure correction: the two restatements agree
    # to ~3e-12 there (measured), to rounding elsewhere
    assert np.max(np.abs(ora - ref)) <= LIMITED_TOL * scale
    for e in picked:
        rho_min, p_min = bezier_prim_min(blocks(sim, ora)[e], SB, d)
        assert rho_min >= EPS_PHYS - 1e-13 * scale and p_min >= EPS_PHYS - 1e-13 * scale
    # untouched volumes change by rounding only
    mask = np.ones(sim.n_vol, bool)
    mask[picked] = False
    assert np.max(np.abs(blocks(sim, ora)[mask] - blocks(sim, u)[mask])) <= 1e-13 * scale


def test_limiter_acts_on_a_coarse_interpolant():
    """3x3x3 HEX p2 vortex: the interpolant's Bezier coefficients have negative density and pressure in some volumes;
    the oracle limits exactly those (numpy restatement), leaving positive minima."""
    sim = dg.Simulation(dg.Config(d=3, p=2, n_elem=(3, 3, 3)))
    a = sim_arrays(sim)
    SB, BS, d = a["ccSB0_vs_vs"], a["ccBS0_vs_vs"], sim.d
    u = sim.sol_coef().copy()
    need = [e for e in range(sim.n_vol) if min(bezier_prim_min(blocks(sim, u)[e], SB, d)) < EPS_PHYS]
    assert len(need) >= 1
    ref = u.copy()
    for e in range(sim.n_vol):
        blocks(sim, ref)[e], _ = limit_volume(blocks(sim, ref)[e], SB, BS, d)
    ora = u.copy()
    assert Oracle(sim).enforce_positivity(ora) == 0
    scale = np.max(np.abs(u))
    assert np.max(np.abs(ora - ref)) <= LIMITED_TOL * scale
    for e in need:
        assert min(bezier_prim_min(blocks(sim, ora)[e], SB, d)) >= EPS_PHYS - 1e-13 * scale


def test_oracle_limiter_stops_on_a_vanishing_average():
    sim = dg.Simulation(dg.Config(d=2, p=2, n_elem=(4, 4, 1)))
    u = sim.sol_coef().copy()
    blocks(sim, u)[5, 0, :] = -0.2              # negative density everywhere in volume 5
    v = u.copy()
    assert Oracle(sim).enforce_positivity(v) == -1
    assert np.array_equal(blocks(sim, v)[5], blocks(sim, u)[5])


@pytest.mark.parametrize("case", CASES[:3], ids=IDS[:3])
def test_oracle_relaxation_matches_numpy(case):
    sim = dg.Simulation(dg.Config(**case))
    a = sim_arrays(sim)
    SB, d = a["ccSB0_vs_vs"], sim.d
    u = sim.sol_coef().copy()
    rng = np.random.default_rng(2)
    du = 0.05 * rng.standard_normal(u.shape) * np.max(np.abs(u))
    db = blocks(sim, du)
    db[1, 0, :] = -1.3 * blocks(sim, u)[1, 0, :]        # density average of u + du negative: relax 1/2 at most
    db[3, d + 1, :] = -3.0 * blocks(sim, u)[3, d + 1, :]  # energy (and pressure) average negative
    rc, relax = Oracle(sim).positivity_relaxation(u, du)
    assert rc == 0
    ref = np.array([relaxation(blocks(sim, u)[e], db[e], SB, d) for e in range(sim.n_vol)])
    assert np.array_equal(relax, ref)
    assert relax[1] < 1.0 and relax[3] < 1.0 and np.sum(relax < 1.0) >= 2
