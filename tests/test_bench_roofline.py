"""The benchmark's roofline arithmetic on CPU: algorithmic bytes per launch from the operand sizes of the workload,
achieved = bytes / CUDA-event time, frac = achieved / the measured HBM peak, traffic = the ncu summary's DRAM bytes
per element times the elements, the dominant kernel is the slowest one."""
import os
import sys

import pytest

import dpgsolver_gb300 as dg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


@pytest.fixture(scope="module")
def sim():
    return dg.Simulation(dg.Config(**bench.WORKLOAD))


def test_algorithmic_bytes_of_the_bench_workload(sim):
    split = bench._bytes_per_element(sim, True)
    # HEX p3 Euler: n_s = n_c = 64, 6 faces of 16 nodes, 5 variables
    assert split["trace"] == 64 * 5 * 8 + 9 * 8 + 96 * 5 * 8 + 3 * 64 * 5 * 8 + 5 * 4
    assert split["volume"] == (96 + 3 * 64) * 5 * 8 + 5 * 32 + 8 + 64 * 5 * 8
    assert split["positivity"] == 64 * 5 * 8
    fp64 = bench._bytes_per_element(sim, False)
    assert set(fp64) == {"trace", "face", "volume", "positivity"}


def test_algorithmic_work_per_residual(sim):
    """One residual of the 32x32x8 HEX p3 Euler workload: 16 B per DOF of state, 4,608 B of metrics per volume,
    16 x 4 doubles per face (about 92 MB), and 327,680 flop per volume (1,024 flop per DOF, 2.68 GFLOP)."""
    b, f = bench._algorithmic_per_residual(sim)
    assert sim.n_dof == 2621440 and sim.n_face == 3 * 8192
    assert b == 2621440 * 16 + 8192 * 64 * 9 * 8 + 24576 * 16 * 4 * 8
    assert 91e6 < b < 93e6
    assert f == 8192 * 327680


def test_roofline_fields(sim):
    kt = {"trace": 0.09, "face": 0.04, "volume": 0.095, "positivity": 0.014}
    peaks = {"hbm_gbs": 6683.8}
    roof = bench._roofline(sim, kt, dg.PREC_BF16_SLICED, peaks, "measured")
    assert roof["kernel"] == "residual (ks_interp + ks_face + ks_lift)"
    assert roof["bound"] == "hbm" and roof["unit"] == "GB/s"
    alg, _ = bench._algorithmic_per_residual(sim)
    assert roof["algorithmic_bytes_per_launch"] == alg
    assert roof["achieved"] == pytest.approx(alg / 0.225e-3 / 1e9)
    assert roof["frac"] == pytest.approx(roof["achieved"] / 6683.8)
    traffic = bench._ncu_traffic()
    if traffic is not None:
        assert roof["traffic"] == pytest.approx(sum(traffic[k] for k in ("ks_interp", "ks_face", "ks_lift")) * sim.n_vol)
    assert set(roof["kernels"]) == {"ks_interp", "ks_face", "ks_lift", "k_positivity"}
    assert roof["kernels"]["ks_lift"]["design_bytes"] == bench._bytes_per_element(sim, True)["volume"] * sim.n_vol


def test_cfl_dt_matches_library(sim):
    """The reference arm's time step (computed without the library) equals the library's cfl_dt."""
    dt = bench._cfl_dt(sim.sol_coef(), sim.n_vol, sim.n_var)
    assert dt == pytest.approx(sim.cfl_dt(0.4, 10.0 / 32), rel=1e-14)
