"""Split-precision (tcgen05) residual vs the CPU oracle and vs the FP64 GPU form.

Tolerances (max |rhs - rhs_oracle| / max |rhs_oracle|): exponent-aligned BF16 slices with S = 6, 7: 1e-10 (the
floating-point parity bound of this path); S = 5: 1e-8; S = 4: 1e-6; TF32x3: 1e-3; BF16x3: 5e-3.
"""
import numpy as np
import pytest

import dpgsolver_gb300 as dg
from oracle import Oracle

pytestmark = pytest.mark.gpu

MODES = [("sliced7", dg.PREC_BF16_SLICED, 7, 1e-10), ("sliced6", dg.PREC_BF16_SLICED, 6, 1e-10),
         ("sliced5", dg.PREC_BF16_SLICED, 5, 1e-8), ("sliced4", dg.PREC_BF16_SLICED, 4, 1e-6),
         ("tf32x3", dg.PREC_TF32X3, 0, 1e-3), ("bf16x3", dg.PREC_BF16X3, 0, 5e-3)]

CASES = [
    dict(d=2, p=2, n_elem=(6, 6, 1)),
    dict(d=2, p=4, n_elem=(5, 4, 1), num_flux="Lax-Friedrichs"),
    dict(d=3, p=1, n_elem=(3, 3, 2)),
    dict(d=3, p=2, n_elem=(4, 3, 2)),
    dict(d=3, p=3, n_elem=(4, 4, 3)),
    dict(d=2, p=3, n_elem=(6, 6, 1), pde="advection", num_flux="upwind", test_case="advection_sine",
         lo=(0, 0, 0), hi=(1, 1, 1)),
]


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"d{c['d']}-p{c['p']}-{c.get('pde', 'euler')}")
def test_split_modes_match_oracle(case):
    sim = dg.Simulation(dg.Config(**case))
    _, ref = Oracle(sim).compute_rhs(sim.sol_coef())
    ctx = dg.GpuContext(sim)
    for name, mode, s, tol in MODES:
        ctx.set_precision(mode, s)
        ctx.compute_rhs()
        err = _rel(ctx.rhs(), ref)
        assert err <= tol, (name, err)


def test_sliced7_rk_matches_fp64_full_size():
    """3D Euler vortex 32x32x8 HEX p3: 10 SSP-RK3 steps, sliced S=7 state within 1e-10 of the FP64 GPU form."""
    sim = dg.Simulation(dg.Config(d=3, p=3, n_elem=(32, 32, 8), lo=(-5, -5, 0), hi=(5, 5, 2.5)))
    ctx = dg.GpuContext(sim)
    u0 = sim.sol_coef()
    dt = sim.cfl_dt(0.4, 10.0 / 32)
    ctx.rk_step(dt, 10)
    u64 = ctx.download()
    ctx.set_precision(dg.PREC_BF16_SLICED, 7)
    ctx.upload(u0)
    ctx.rk_step(dt, 10)
    assert _rel(ctx.download(), u64) <= 1e-10


def test_split_requires_affine_geometry():
    sim = dg.Simulation(dg.Config(d=2, p=2, n_elem=(4, 4, 1), jitter=0.2, seed=1))
    ctx = dg.GpuContext(sim)
    with pytest.raises(dg.DpgError) as ei:
        ctx.set_precision(dg.PREC_BF16_SLICED, 6)
    assert ei.value.status == dg.api.DPG_ERR_UNSUPPORTED


def test_invalid_slice_count_rejected():
    sim = dg.Simulation(dg.Config(d=2, p=2, n_elem=(4, 4, 1)))
    ctx = dg.GpuContext(sim)
    with pytest.raises(dg.DpgError):
        ctx.set_precision(dg.PREC_BF16_SLICED, 9)


@pytest.mark.parametrize("case", [CASES[0], CASES[4]], ids=["quad-p2", "hex-p3"])
def test_residual_scales_with_the_state(case):
    """Exponent handling far from unit magnitudes: the Euler flux and the Roe-Pike flux are homogeneous of degree 1
    in the conservative state (velocity and sound speed do not change), so scaling the state by 2^k scales the
    residual by 2^k -- exactly in the FP64 form (power-of-two factors round nothing), and to the split modes'
    own rounding (the per-row digit scales, exponent bounds and double-float fluxes all move by k)."""
    sim = dg.Simulation(dg.Config(**case))
    u = sim.sol_coef()
    ctx = dg.GpuContext(sim)
    for mode, s, tol in [(dg.PREC_FP64, 0, 0.0), (dg.PREC_BF16_SLICED, 7, 1e-13), (dg.PREC_BF16_SLICED, 5, 1e-13)]:
        ctx.set_precision(mode, s)
        ctx.upload(u)
        ctx.compute_rhs()
        r1 = ctx.rhs()
        for k in (-40, 40):
            ctx.upload(np.ldexp(u, k))
            ctx.compute_rhs()
            rk = np.ldexp(ctx.rhs(), -k)
            err = float(np.max(np.abs(rk - r1)) / np.max(np.abs(r1)))
            assert err <= tol, (mode, s, k, err)
