"""Restart files (the reference's format: gmsh 2.2 mesh + $SolutionCoefficients of Bezier coefficients,
restart_writers.c; read back as set_sol_restart_T does, restart_T.c): same-mesh round trips, a restart onto a mesh of
higher order and onto a finer, non-nested mesh (a state that the coarse space holds exactly must come back exactly),
the file layout and the error cases."""
import numpy as np
import pytest

import dpgsolver_gb300 as dg
from tests_support import solution_node_xyz


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("cfg", [dict(d=2, p=3, n_elem=(5, 4, 1), jitter=0.2, seed=3),
                                 dict(d=3, p=2, n_elem=(3, 3, 2)),
                                 dict(d=2, p=2, n_elem=(4, 4, 1), pde="advection", num_flux="upwind",
                                      test_case="advection_sine", lo=(0, 0, 0), hi=(1, 1, 1))],
                         ids=["quad-p3-jitter", "hex-p2", "quad-advection"])
def test_round_trip_on_the_same_mesh(tmp_path, cfg):
    sim = dg.Simulation(dg.Config(**cfg))
    u = sim.sol_coef() * (1.0 + 0.01 * np.random.default_rng(1).standard_normal(sim.n_dof))   # discontinuous
    sim.set_sol_coef(u)
    path = str(tmp_path / "restart.msh")
    sim.write_restart(path)
    other = dg.Simulation(dg.Config(**cfg))
    other.read_restart(path)
    assert _rel(other.sol_coef(), u) <= 1e-13


def test_file_layout(tmp_path):
    sim = dg.Simulation(dg.Config(d=2, p=2, n_elem=(3, 2, 1)))
    path = tmp_path / "r.msh"
    sim.write_restart(str(path))
    lines = path.read_text().splitlines()
    assert lines[:3] == ["$MeshFormat", "2.2 0 8", "$EndMeshFormat"]
    i = lines.index("$Nodes")
    assert int(lines[i + 1]) == 4 * 3          # distinct vertices of the 3x2 box (periodic images kept apart)
    j = lines.index("$Elements")
    assert int(lines[j + 1]) == 6 and all(l.split()[1:5] == ["3", "2", "0", "0"] for l in lines[j + 2:j + 8])
    k = lines.index("$SolutionCoefficients")
    assert int(lines[k + 1]) == 6
    head = lines[k + 2].split()
    assert head[:4] == ["1", "2", "9", "4"] and len(head) == 4 + 9 * 4
    assert lines[-1] == "$EndSolutionCoefficients"


def _linear_state(sim, coef):
    """Nodal values of u_v(x) = c0 + c . x per variable (held exactly by every Q_p space on multilinear volumes)."""
    x = solution_node_xyz(sim)                                    # [n_vol, n_s, d]
    out = np.empty((sim.n_vol, sim.n_var, sim.n_s))
    for v in range(sim.n_var):
        out[:, v, :] = coef[v][0] + np.einsum("vsd,d->vs", x, np.asarray(coef[v][1:sim.d + 1]))
    return out.reshape(-1)


@pytest.mark.parametrize("d", [2, 3])
def test_restart_onto_a_finer_mesh_of_higher_order(tmp_path, d):
    n0 = (3, 3, 2) if d == 3 else (4, 3, 1)
    n1 = (5, 4, 3) if d == 3 else (7, 6, 1)
    # straight boxes: every node of the fine mesh lies inside the coarse mesh (a jittered periodic mesh has wavy
    # boundaries, so nodes there are found at their periodic images, where a linear -- non-periodic -- field differs;
    # jittered meshes are covered by the same-mesh round trip)
    coarse = dg.Simulation(dg.Config(d=d, p=2, n_elem=n0))
    rng = np.random.default_rng(4)
    coef = [rng.uniform(0.5, 1.5, 1 + d) for _ in range(coarse.n_var)]
    coarse.set_sol_coef(_linear_state(coarse, coef))
    path = str(tmp_path / "coarse.msh")
    coarse.write_restart(path)
    fine = dg.Simulation(dg.Config(d=d, p=3, n_elem=n1))
    fine.read_restart(path)
    assert _rel(fine.sol_coef(), _linear_state(fine, coef)) <= 1e-12


def test_missing_file_and_foreign_mesh(tmp_path):
    sim = dg.Simulation(dg.Config(d=2, p=2, n_elem=(3, 3, 1)))
    with pytest.raises(dg.DpgError) as ei:
        sim.read_restart(str(tmp_path / "none.msh"))
    assert ei.value.status == dg.api.DPG_ERR_IO
    small = dg.Simulation(dg.Config(d=2, p=2, n_elem=(2, 2, 1), lo=(0, 0, 0), hi=(1, 1, 1)))
    small.write_restart(str(tmp_path / "small.msh"))
    with pytest.raises(dg.DpgError) as ei:          # nodes of [-5, 5]^2 outside the restart mesh's [0, 1]^2
        sim.read_restart(str(tmp_path / "small.msh"))
    assert ei.value.status == dg.api.DPG_ERR_UNSUPPORTED


def test_inverse_mapping_against_the_reference_fixture():
    """The inverse of the multilinear volume map used to locate nodes in a restart mesh, on the reference's own
    test data (input/testing/unit/inverse_mapping/quad.data, test_unit_inverse_mapping.c): points of the standard
    element mapped forward by a random, the standard and the symmetric quadrilateral must map back to their
    symmetric reference coordinates within the reference's tolerance, 1e3 EPS."""
    import ctypes as C
    import json
    import os

    gold = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                       "reference_goldens.json")))["inverse_mapping_quad"]
    fn = dg.load_library().dpg_p1_inverse_map
    fn.restype = C.c_int
    dp = C.POINTER(C.c_double)
    fn.argtypes = [C.c_int, dp, dp, dp]
    rst = np.array(gold["rst_std"])                      # [n, 2] in [0, 1]^2
    phi = np.stack([(1 - rst[:, 0]) * (1 - rst[:, 1]), rst[:, 0] * (1 - rst[:, 1]),
                    (1 - rst[:, 0]) * rst[:, 1], rst[:, 0] * rst[:, 1]], axis=1)
    expect = 2.0 * rst - 1.0                             # the symmetric element's coordinates
    for name in ("ve_random", "ve_std", "ve_symm"):
        ve = np.zeros((4, 3))
        ve[:, :2] = np.array(gold[name])
        xyz = phi @ ve
        ve_c = np.ascontiguousarray(ve)
        for i in range(len(rst)):
            y = np.ascontiguousarray(xyz[i])
            r = np.zeros(3)
            ok = fn(2, ve_c.ctypes.data_as(dp), y.ctypes.data_as(dp), r.ctypes.data_as(dp))
            assert ok == 1, (name, i)
            assert np.max(np.abs(r[:2] - expect[i])) <= 1e3 * 1e-15, (name, i, r[:2], expect[i])
