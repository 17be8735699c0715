"""Edge sizes of the GPU path.

- Meshes one element wide (a face joins an element to itself through the periodic boundary, so both sides of a
  face are the same volume) and a single element: FP64 form and S = 7 split precision against the oracle, and RK
  steps (the limiter may act on such coarse interpolants, hence the positivity tests' 1e-9 for the steps).
- A mesh 16x the bench workload (80x80x20 HEX p=3, 128,000 volumes, 41 M DOF): size-independent properties --
  free-stream preservation and discrete conservation of the residual -- for both forms.
"""
import numpy as np
import pytest

import dpgsolver_gb300 as dg
from oracle import Oracle
from tests_support import sim_arrays

pytestmark = pytest.mark.gpu

THIN = [dict(d=2, p=2, n_elem=(1, 1, 1)), dict(d=2, p=3, n_elem=(1, 4, 1)), dict(d=3, p=2, n_elem=(1, 1, 1)),
        dict(d=3, p=3, n_elem=(2, 1, 3))]


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("case", THIN, ids=lambda c: "d{}-p{}-{}x{}x{}".format(c["d"], c["p"], *c["n_elem"]))
def test_meshes_one_element_wide(case):
    sim = dg.Simulation(dg.Config(**case))
    ora = Oracle(sim)
    u = sim.sol_coef()
    _, ref = ora.compute_rhs(u)
    ctx = dg.GpuContext(sim)
    for mode, s, tol in [(dg.PREC_FP64, 0, 1e-11), (dg.PREC_BF16_SLICED, 7, 1e-10)]:
        ctx.set_precision(mode, s)
        ctx.upload(u)
        ctx.compute_rhs()
        assert _rel(ctx.rhs(), ref) <= tol, mode
    ctx.set_precision(dg.PREC_FP64, 0)
    ctx.upload(u)
    dt = 1e-3
    ctx.rk_step(dt, 2)
    o = u.copy()
    ora.rk_step(o, dt, 2)
    assert _rel(ctx.download(), o) <= 1e-9


BIG = dict(d=3, p=3, n_elem=(80, 80, 20), lo=(-5.0, -5.0, 0.0), hi=(5.0, 5.0, 2.5))


@pytest.fixture(scope="module")
def big():
    sim = dg.Simulation(dg.Config(**BIG))
    return sim, dg.GpuContext(sim)


@pytest.mark.parametrize("prec", [(dg.PREC_FP64, 0), (dg.PREC_BF16_SLICED, 7)], ids=["fp64", "sliced7"])
def test_large_mesh_conservation(big, prec):
    """Sum over all basis functions of M rhs (the unscaled residual) vanishes on a periodic mesh: with M = detJ M_ref
    per affine volume, sum_j c_j detJ_e rhs_ej = 0 per variable, c = column sums of M_ref."""
    sim, ctx = big
    ctx.set_precision(*prec)
    ctx.upload(sim.sol_coef())
    ctx.compute_rhs()
    rhs = ctx.rhs().reshape(sim.n_vol, sim.n_var, sim.n_s)
    a = sim_arrays(sim)
    c = np.linalg.inv(a["m_inv_ref"]).sum(axis=0)                       # [n_s]
    detj = a["jacobian_det_vc"].reshape(sim.n_vol, sim.n_c)[:, 0]      # affine volumes
    terms = rhs * c[None, None, :] * detj[:, None, None]
    tot = terms.sum(axis=(0, 2))
    # relative to the largest variable's term scale (w-momentum is zero for this vortex: its sums are rounding);
    # measured (FP64 form): |tot| <= 4e-11 against a scale of 40
    assert np.all(np.abs(tot) <= 1e-9 * np.abs(terms).sum(axis=(0, 2)).max()), tot


@pytest.mark.parametrize("prec", [(dg.PREC_FP64, 0), (dg.PREC_BF16_SLICED, 7)], ids=["fp64", "sliced7"])
def test_large_mesh_free_stream(prec):
    sim = dg.Simulation(dg.Config(**BIG, test_case="free_stream"))
    ctx = dg.GpuContext(sim)
    ctx.set_precision(*prec)
    # round-off of O(1) fluxes scaled by 1/detJ (~4000 here) through the lift: ~1e-10 absolute
    assert ctx.compute_rhs() < 1e-9
    u = sim.sol_coef()
    ctx.rk_step(1e-3, 1)
    assert np.max(np.abs(ctx.download() - u)) < 1e-11
