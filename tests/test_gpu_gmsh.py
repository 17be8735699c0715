"""The GPU residual path on meshes read from gmsh files (the reference's own periodic QUAD mesh and a generated
periodic HEX mesh with rotated and mirrored elements): FP64 form and S = 7 split precision against the oracle on the
same host data (1e-11 / 1e-10, the path's bounds), and RK steps."""
import os

import numpy as np
import pytest

import dpgsolver_gb300 as dg
from gmsh_writer import write_box_msh
from oracle import Oracle

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def _meshes(tmp_path):
    quad = (dg.Config(d=2, p=3, vortex=(1.0, 0.0, 0.0, 1.0, 0.5, 0.25, 0.0, 1.0)),
            os.path.join(GOLDEN, "straight_2d_quad_periodic.msh"))
    hex_msh = str(tmp_path / "hex.msh")
    write_box_msh(hex_msh, 3, (6, 5, 3), (-5.0, -5.0, 0.0), (5.0, 5.0, 2.5), rotate_seed=5, mirror_every=4,
                  shuffle_seed=9)
    return [quad, (dg.Config(d=3, p=3), hex_msh)]


def test_residual_and_steps_on_gmsh_meshes(tmp_path):
    for cfg, msh in _meshes(tmp_path):
        sim = dg.Simulation(cfg, msh=msh)
        ora = Oracle(sim)
        u = sim.sol_coef()
        _, ref = ora.compute_rhs(u)
        ctx = dg.GpuContext(sim)
        modes = [(dg.PREC_FP64, 0, 1e-11)] + ([(dg.PREC_BF16_SLICED, 7, 1e-10)] if cfg.d == 3 else [])
        for mode, s, tol in modes:
            ctx.set_precision(mode, s)
            ctx.upload(u)
            ctx.compute_rhs()
            assert _rel(ctx.rhs(), ref) <= tol, (msh, mode)
        dt = 1e-3
        ctx.set_precision(dg.PREC_FP64, 0)
        ctx.upload(u)
        ctx.rk_step(dt, 2)
        o = u.copy()
        ora.rk_step(o, dt, 2)
        assert _rel(ctx.download(), o) <= 1e-11, msh


def test_walls_from_physical_tags_on_the_gpu(tmp_path):
    """A generated mesh whose boundary elements carry slip-wall and Riemann tags (bc_base + BC_*): the general chain
    against the oracle's own set-up of the same file (1e-11), and RK steps."""
    cfg = dg.Config(d=2, p=3, n_elem=(5, 4, 1), lo=(0.0, 0.0, 0.0), hi=(2.0, 1.0, 1.0), test_case="free_stream",
                    vortex=(0, 0, 0, 1.0, 0.7, 0.3, 0, 1.0), bc=("riemann", "riemann", "slipwall", "slipwall"),
                    bc_state=(1.0, 0.7, 0.3, 0.0, 1.0))
    msh = str(tmp_path / "walls.msh")
    write_box_msh(msh, 2, (5, 4), (0.0, 0.0), (2.0, 1.0), rotate_seed=2, mirror_every=3, shuffle_seed=1,
                  side_tags={(0, 0): 10101, (0, 1): 10101, (1, 0): 10102, (1, 1): 10102}, periodic_dirs=[])
    sim = dg.Simulation(cfg, msh=msh)
    ora = Oracle(cfg, msh=msh)
    u = sim.sol_coef() * (1.0 + 1e-2 * np.random.default_rng(4).standard_normal(sim.n_dof))
    _, ref = ora.compute_rhs(u)
    ctx = dg.GpuContext(sim)
    ctx.upload(u)
    ctx.compute_rhs()
    assert _rel(ctx.rhs(), ref) <= 1e-11
    ctx.rk_step(1e-3, 3)
    o = u.copy()
    ora.rk_step(o, 1e-3, 3)
    assert _rel(ctx.download(), o) <= 1e-11
