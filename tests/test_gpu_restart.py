"""Restart of a GPU run: the device state after some RK steps written to a restart file and read back into a fresh
context of the same problem continues identically (the same state to the restart file's 16 significant digits)."""
import numpy as np
import pytest

import dpgsolver_gb300 as dg

pytestmark = pytest.mark.gpu


def test_gpu_restart_round_trip(tmp_path):
    cfg = dg.Config(d=3, p=3, n_elem=(6, 6, 2), lo=(-5, -5, 0), hi=(5, 5, 2.5))
    ctx = dg.GpuContext(dg.Simulation(cfg))
    ctx.set_precision(dg.PREC_BF16_SLICED, 7)
    ctx.rk_step(1e-2, 5)
    u = ctx.download()
    path = str(tmp_path / "restart.msh")
    ctx.write_restart(path)
    other = dg.GpuContext(dg.Simulation(cfg))
    other.read_restart(path)
    assert np.max(np.abs(other.download() - u)) <= 1e-13 * np.max(np.abs(u))
