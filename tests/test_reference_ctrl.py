"""The reference's own control files: dpg_sim_create_from_ctrl on
input/testing/control_files/euler/periodic_vortex/TEST_Euler_PeriodicVortex_QUAD__ml2__p2.ctrl with the test case's
input_files/euler/periodic/periodic_vortex/test_case.data and solution.data, copied unchanged under
golden/reference_input/ in the reference's relative layout (golden/make_golden.py).

The reference generates its meshes with gmsh from input/meshes/n-cube/2d.geo; gmsh is not run here, so the test
writes the same mesh -- [-1, 1]^2, 2^(ml+1) = 8 QUAD elements per direction for ml 2, periodic in x and y -- with
the test suite's gmsh writer at the path the reference assembles from the control file (mesh_name_assemble,
simulation.c:624-640): ../meshes/n-cube/euler/periodic/periodic_vortex/straight__2d__quad_ml2.msh.  The loaded
problem must equal the same problem set up from a Config and that mesh, and its initial state must equal the
oracle's own restatement of the Gaussian periodic vortex (solution_euler_periodic_vortex.c)."""
import ctypes as C
import os
import shutil

import numpy as np
import pytest

import dpgsolver_gb300 as dg
from gmsh_writer import write_box_msh
from oracle import Oracle, Problem
from oracle import oracle_layout as L

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_input")
CTRL_REL = os.path.join("testing", "control_files", "euler", "periodic_vortex",
                        "TEST_Euler_PeriodicVortex_QUAD__ml2__p2.ctrl")
MESH_REL = os.path.join("testing", "control_files", "euler", "meshes", "n-cube", "euler", "periodic",
                        "periodic_vortex", "straight__2d__quad_ml2.msh")
VORTEX = (0.165, 0.7853981633974483, 0.5916079783099616, 1.0, 1.0, 1.0)   # solution.data: r_v theta V_inf p_inf t_inf Rg


def _tree(tmp_path, mesh=True):
    root = tmp_path / "input"
    shutil.copytree(GOLDEN, root)
    msh = root / MESH_REL
    if mesh:
        msh.parent.mkdir(parents=True)
        write_box_msh(str(msh), 2, (8, 8), (-1.0, -1.0), (1.0, 1.0), rotate_seed=5, shuffle_seed=9)
    return root, str(root / CTRL_REL), str(msh)


def _config():
    return dg.Config(d=2, p=2, num_flux="Roe-Pike", test_case="periodic_vortex", vortex=VORTEX + (0.0, 0.0))


def test_reference_control_file_loads_the_periodic_vortex(tmp_path):
    _, ctrl, msh = _tree(tmp_path)
    sim = dg.Simulation(ctrl=ctrl)
    assert (sim.d, sim.p, sim.n_vol, sim.n_var) == (2, 2, 64, 4)
    s = L.model(dg.load_library().dpg_sim_view(sim.handle))
    assert s.test_case == dg.api.TC_PERIODIC_VORTEX
    assert (s.dt, s.time_final) == (0.0025, 0.20)                  # test_case.data
    assert s.ind_num_flux[0] == 31                                   # num_flux_1st Roe-Pike
    assert (s.solver_proc, s.solver_type_e) == (100, 102)            # explicit, ssp_rk_33
    assert tuple(s.vortex[:6]) == VORTEX

    same = dg.Simulation(_config(), msh=msh)
    assert np.array_equal(sim.sol_coef(), same.sol_coef())
    orc = Oracle(data_model=dg.load_library().dpg_sim_view(sim.handle))
    m_ctrl, r_ctrl = orc.compute_rhs(sim.sol_coef())
    m_same, r_same = Oracle(data_model=dg.load_library().dpg_sim_view(same.handle)).compute_rhs(same.sol_coef())
    assert np.array_equal(r_ctrl, r_same) and m_ctrl == m_same


def test_periodic_vortex_initial_state_matches_the_oracle(tmp_path):
    """The library's periodic vortex against the oracle's restatement on the oracle's own set-up of the same mesh."""
    _, ctrl, msh = _tree(tmp_path)
    sim = dg.Simulation(ctrl=ctrl)
    pr = Problem(d=2, p=2, num_flux="Roe-Pike", test_case="periodic_vortex", vortex=VORTEX + (0.0, 0.0))
    orc = Oracle(pr, msh=msh)
    u_orc = orc.initial_solution()
    u_lib = sim.sol_coef()
    assert np.max(np.abs(u_orc - u_lib)) <= 1e-13 * np.max(np.abs(u_orc))
    m_o, r_o = orc.compute_rhs(u_orc)
    m_l, r_l = Oracle(data_model=dg.load_library().dpg_sim_view(sim.handle)).compute_rhs(u_lib)
    assert np.max(np.abs(r_o - r_l)) <= 1e-12 * np.max(np.abs(r_o))
    # the vortex centre moves with V_inf along theta and wraps with period 2 sqrt(2) on the 45 degree diagonal
    e_early = sim.l2_error(0.0)
    assert np.all(e_early < 1e-2)
    assert np.max(np.abs(sim.l2_error(2 * np.sqrt(2) / VORTEX[2]) - e_early)) < 1e-12


def test_missing_solution_parameters_and_mesh_are_reported(tmp_path):
    root, ctrl, msh = _tree(tmp_path)
    lib = dg.load_library()
    h = C.c_void_p()
    os.remove(msh)
    assert lib.dpg_sim_create_from_ctrl(ctrl.encode(), C.byref(h)) == dg.api.DPG_ERR_IO
    write_box_msh(msh, 2, (8, 8), (-1.0, -1.0), (1.0, 1.0))
    sol = root / "input_files" / "euler" / "periodic" / "periodic_vortex" / "solution.data"
    text = sol.read_text()
    sol.write_text("\n".join(l for l in text.splitlines() if not l.startswith("Rg")))
    assert lib.dpg_sim_create_from_ctrl(ctrl.encode(), C.byref(h)) == dg.api.DPG_ERR_IO
    sol.write_text(text)
    assert lib.dpg_sim_create_from_ctrl(ctrl.encode(), C.byref(h)) == dg.api.DPG_OK
    lib.dpg_sim_destroy(h)


@pytest.mark.parametrize("edit", [("fe_method 1", "fe_method 2"), ("mesh_type        quad", "mesh_type        wedge"),
                                  ("basis_sol   lagrange", "basis_sol   bezier")])
def test_methods_outside_this_path_are_refused(tmp_path, edit):
    _, ctrl, _ = _tree(tmp_path)
    text = open(ctrl).read()
    assert edit[0] in text
    open(ctrl, "w").write(text.replace(edit[0], edit[1]))
    h = C.c_void_p()
    assert dg.load_library().dpg_sim_create_from_ctrl(ctrl.encode(), C.byref(h)) == dg.api.DPG_ERR_UNSUPPORTED


def test_input_directory_from_the_environment(tmp_path, monkeypatch):
    root, ctrl, _ = _tree(tmp_path)
    away = tmp_path / "elsewhere"
    shutil.move(str(root / "input_files"), str(away / "input_files"))
    h = C.c_void_p()
    lib = dg.load_library()
    assert lib.dpg_sim_create_from_ctrl(ctrl.encode(), C.byref(h)) == dg.api.DPG_ERR_IO
    monkeypatch.setenv("DPG_INPUT_DIR", str(away))
    assert lib.dpg_sim_create_from_ctrl(ctrl.encode(), C.byref(h)) == dg.api.DPG_OK
    lib.dpg_sim_destroy(h)


@pytest.mark.gpu
def test_reference_control_file_runs_to_time_final_on_the_gpu(tmp_path):
    """The loaded case marched with its own time_step to its own time_final (80 SSP-RK3 steps) on the GPU, against
    the oracle's march of the same problem: state and L2 errors equal within 1e-10 (FP64 rounding order only)."""
    _, ctrl, msh = _tree(tmp_path)
    sim = dg.Simulation(ctrl=ctrl)
    s = L.model(dg.load_library().dpg_sim_view(sim.handle))
    n_steps = int(round(s.time_final / s.dt))
    orc = Oracle(Problem(d=2, p=2, num_flux="Roe-Pike", test_case="periodic_vortex", vortex=VORTEX + (0.0, 0.0)),
                 msh=msh)
    u = orc.initial_solution()
    ctx = dg.GpuContext(sim)
    ctx.upload(sim.sol_coef())
    ctx.rk_step(s.dt, n_steps)
    orc.rk_step(u, s.dt, n_steps)
    got = ctx.download()
    assert np.max(np.abs(got - u)) <= 1e-10 * np.max(np.abs(u))
    sim.set_sol_coef(got)
    assert np.allclose(sim.l2_error(s.time_final), orc.l2_error(u, s.time_final), rtol=1e-10, atol=1e-14)
