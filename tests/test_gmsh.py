"""gmsh 2.2 reader of the host set-up (the reference's mesh input, mesh_readers.c): the reference's own periodic QUAD
mesh file and generated periodic QUAD / HEX meshes with rotated and mirrored element vertex orders and shuffled node
numbers give the residual of the structured box mesh (volumes and nodes matched by their coordinates); meshes
outside this path (non-periodic boundaries, triangles) and unreadable files are refused with a status."""
import json
import os

import numpy as np
import pytest

import dpgsolver_gb300 as dg
from gmsh_writer import write_box_msh
from oracle import Oracle
from tests_support import match_volumes, remap_state, sim_arrays

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REF_MSH = os.path.join(GOLDEN, "straight_2d_quad_periodic.msh")


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def _same_residual(cfg, msh, tol):
    sim = dg.Simulation(cfg, msh=msh)
    box = dg.Simulation(cfg)
    assert (sim.n_vol, sim.n_face) == (box.n_vol, box.n_face)
    vol, perm = match_volumes(box, sim, tol=1e-9)
    _, r_box = Oracle(box).compute_rhs(box.sol_coef())
    _, r_msh = Oracle(sim).compute_rhs(sim.sol_coef())
    assert _rel(remap_state(box, sim, sim.sol_coef(), vol, perm), box.sol_coef()) <= tol
    assert _rel(remap_state(box, sim, r_msh, vol, perm), r_box) <= tol
    return sim, box


def test_reference_mesh_file():
    """input/testing/integration/mesh/straight_2d_quad_periodic.msh: 2x2 QUAD on [-1, 1]^2 (its centre lines at
    -2.75e-12), periodic through $Periodic; residual and face normals as the structured 2x2 box."""
    cfg = dg.Config(d=2, p=2, n_elem=(2, 2, 1), lo=(-1.0, -1.0, 0.0), hi=(1.0, 1.0, 0.0),
                    vortex=(1.0, 0.0, 0.0, 1.0, 0.5, 0.25, 0.0, 1.0))
    sim, _ = _same_residual(cfg, REF_MSH, 1e-9)
    gold = json.load(open(os.path.join(GOLDEN, "reference_goldens.json")))
    ref = np.array(gold["geom_straight_2d_quad_periodic_normals"]).reshape(-1, 2)
    ours = sim_arrays(sim)["normals_fc"]
    assert sorted({tuple(np.round(r, 9)) for r in ref}) == sorted(
        {tuple(np.round(o, 9)) for o in np.concatenate([ours, -ours])})


@pytest.mark.parametrize("d,p,n", [(2, 2, (5, 4, 1)), (2, 3, (3, 3, 1)), (3, 2, (3, 2, 2)), (3, 3, (2, 2, 2)),
                                   (2, 2, (1, 3, 1)), (3, 2, (1, 1, 1))],
                         ids=["quad-p2", "quad-p3", "hex-p2", "hex-p3", "quad-one-wide", "hex-single"])
def test_generated_meshes_with_rotated_and_mirrored_elements(tmp_path, d, p, n):
    lo, hi = (-5.0, -5.0, 0.0), (5.0, 5.0, 2.5)
    cfg = dg.Config(d=d, p=p, n_elem=n, lo=lo, hi=hi)
    msh = str(tmp_path / "box.msh")
    write_box_msh(msh, d, n, lo, hi, rotate_seed=7, mirror_every=3, shuffle_seed=11)
    _same_residual(cfg, msh, 1e-12)


def test_control_file_with_mesh_path(tmp_path):
    msh_dir = tmp_path / "meshes"
    msh_dir.mkdir()
    write_box_msh(str(msh_dir / "box.msh"), 2, (4, 4), (-5.0, -5.0), (5.0, 5.0), rotate_seed=3)
    ctrl = tmp_path / "case.ctrl"
    ctrl.write_text("pde_name euler\ndimension 2\nmesh_format gmsh\nmesh_type quad\nmesh_path meshes/box.msh\n"
                    "p_ref 2\nnum_flux_1st Roe-Pike\ntest_case isentropic_vortex\n")
    sim = dg.Simulation(ctrl=str(ctrl))
    box = dg.Simulation(dg.Config(d=2, p=2, n_elem=(4, 4, 1)))
    vol, perm = match_volumes(box, sim)
    _, r_box = Oracle(box).compute_rhs(box.sol_coef())
    _, r_msh = Oracle(data_model=dg.load_library().dpg_sim_view(sim.handle)).compute_rhs(sim.sol_coef())
    assert _rel(remap_state(box, sim, r_msh, vol, perm), r_box) <= 1e-12


@pytest.mark.parametrize("kind", ["no-periodic", "triangle", "missing"])
def test_meshes_outside_the_path_are_refused(tmp_path, kind):
    msh = str(tmp_path / "bad.msh")
    if kind == "no-periodic":
        write_box_msh(msh, 2, (3, 3), (0.0, 0.0), (1.0, 1.0), periodic=False)
        status = dg.api.DPG_ERR_UNSUPPORTED
    elif kind == "triangle":
        write_box_msh(msh, 2, (3, 3), (0.0, 0.0), (1.0, 1.0), add_triangle=True)
        status = dg.api.DPG_ERR_UNSUPPORTED
    else:
        msh = str(tmp_path / "none.msh")
        status = dg.api.DPG_ERR_IO
    with pytest.raises(dg.DpgError) as ei:
        dg.Simulation(dg.Config(d=2, p=2), msh=msh)
    assert ei.value.status == status


def test_reference_mesh_connectivity():
    """The reference's finite-element connectivity of the same mesh (input/testing/integration/fe/
    TEST_straight_2d_quad_periodic.fe.data): every volume's vertices in tensor-product order and the set of faces as
    pairs of (volume, local face) sides, periodic faces included, as the gmsh reader builds them."""
    import ctypes as C
    from tests_support import DpgSim, _arr

    gold = json.load(open(os.path.join(GOLDEN, "reference_goldens.json")))["fe_straight_2d_quad_periodic"]
    sim = dg.Simulation(dg.Config(d=2, p=2), msh=REF_MSH)
    s = C.cast(sim.handle, C.POINTER(DpgSim)).contents
    xyz = _arr(s.xyz_ve, s.n_vol * 8 * 3).reshape(s.n_vol, 8, 3)[:, :4, :2]
    assert np.max(np.abs(xyz - np.array(gold["xyz_ve"]))) <= 1e-11   # the file's centre lines sit at -2.75e-12
    fv = _arr(s.face_vol, 2 * s.n_face, np.int32).reshape(-1, 2)
    fl = _arr(s.face_lf, 2 * s.n_face, np.int32).reshape(-1, 2)
    ours = {frozenset({(int(fv[f, 0]), int(fl[f, 0])), (int(fv[f, 1]), int(fl[f, 1]))}) for f in range(s.n_face)}
    ref = {frozenset({tuple(a), tuple(b)}) for a, b in gold["faces"]}
    assert ours == ref


def test_reference_face_normals_face_by_face():
    """The geometry fixture's unit normals (TEST_straight_2d_quad_periodic.geom.data, outward from each face's first
    side), face by face: faces matched through the connectivity fixture's (volume, local face) sides, the sign
    following which side this library lists first."""
    import ctypes as C
    from tests_support import DpgSim, _arr

    gold = json.load(open(os.path.join(GOLDEN, "reference_goldens.json")))
    fe = gold["fe_straight_2d_quad_periodic"]
    sim = dg.Simulation(dg.Config(d=2, p=2), msh=REF_MSH)
    s = C.cast(sim.handle, C.POINTER(DpgSim)).contents
    fv = _arr(s.face_vol, 2 * s.n_face, np.int32).reshape(-1, 2)
    fl = _arr(s.face_lf, 2 * s.n_face, np.int32).reshape(-1, 2)
    ours = sim_arrays(sim)["normals_fc"].reshape(s.n_face, sim.n_fc, 2)
    side = {(int(fv[f, k]), int(fl[f, k])): (f, k) for f in range(s.n_face) for k in range(2)}
    for i, (a, b) in enumerate(fe["faces"]):
        f, k = side[tuple(a)]
        assert side[tuple(b)] == (f, 1 - k)
        ref = np.array(gold["geom_straight_2d_quad_periodic_normals"][i]).reshape(-1, 2)
        assert ref.shape == ours[f].shape
        assert np.max(np.abs((1.0 if k == 0 else -1.0) * ours[f] - ref)) <= 1e-12, (i, ours[f], ref)


def test_control_file_with_another_mesh_format(tmp_path):
    ctrl = tmp_path / "case.ctrl"
    ctrl.write_text("pde_name euler\ndimension 2\nmesh_format other\nmesh_type quad\np_ref 2\n")
    with pytest.raises(dg.DpgError) as ei:
        dg.Simulation(ctrl=str(ctrl))
    assert ei.value.status == dg.api.DPG_ERR_UNSUPPORTED


WALL_CASES = {
    "quad-p2-slip-x": (dict(d=2, p=2, n_elem=(4, 3, 1), lo=(0.0, 0.0, 0.0), hi=(2.0, 1.0, 1.0), test_case="free_stream",
                            vortex=(0, 0, 0, 1.0, 0.4, 0.3, 0, 1.0), bc=("slipwall", "slipwall", "periodic", "periodic")),
                       {(0, 0): 10102, (0, 1): 10102}, [1]),
    "quad-p3-riemann-slip": (dict(d=2, p=3, n_elem=(3, 4, 1), lo=(0.0, 0.0, 0.0), hi=(1.0, 2.0, 1.0),
                                  test_case="free_stream", vortex=(0, 0, 0, 1.0, 0.7, 0.3, 0, 1.0),
                                  bc=("riemann", "riemann", "slipwall", "riemann"), bc_state=(1.0, 0.7, 0.3, 0.0, 1.0)),
                             {(0, 0): 10101, (0, 1): 20101, (1, 0): 10102, (1, 1): 10101}, []),
    "hex-p2-walls-z": (dict(d=3, p=2, n_elem=(2, 2, 3), lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.5),
                            test_case="free_stream", vortex=(0, 0, 0, 1.0, 0.3, 0.2, 0.4, 1.0),
                            bc=("periodic",) * 4 + ("riemann", "slipwall"), bc_state=(1.0, 0.3, 0.2, 0.4, 1.0)),
                       {(2, 0): 10101, (2, 1): 10102}, [0, 1]),
}


@pytest.mark.parametrize("name", list(WALL_CASES))
def test_boundary_conditions_from_physical_tags(tmp_path, name):
    """Boundary lines / quadrilaterals tagged bc_base + BC_* (straight 10000, curved 20000 numbering) give the
    boundary faces of the structured box with the same conditions: same residual after matching volumes (library
    set-up), and the oracle's own set-up of the mesh file gives the library's residual."""
    case, tags, per = WALL_CASES[name]
    d = case["d"]
    cfg = dg.Config(**case)
    msh = str(tmp_path / "walls.msh")
    write_box_msh(msh, d, case["n_elem"][:d], case["lo"][:d], case["hi"][:d], rotate_seed=4, mirror_every=3,
                  shuffle_seed=8, side_tags=tags, periodic_dirs=per)
    sim = dg.Simulation(cfg, msh=msh)
    box = dg.Simulation(cfg)
    assert (sim.n_vol, sim.n_face) == (box.n_vol, box.n_face)
    vol, perm = match_volumes(box, sim, tol=1e-9)
    u = box.sol_coef() * (1.0 + 1e-3 * np.random.default_rng(3).standard_normal(box.n_dof))
    ub = u.reshape(box.n_vol, box.n_var, box.n_s)
    u_msh = np.empty_like(ub)
    u_msh[vol[:, None], :, perm] = ub.transpose(0, 2, 1)
    u_msh = u_msh.reshape(-1)
    _, r_box = Oracle(box).compute_rhs(u)
    _, r_msh = Oracle(data_model=dg.load_library().dpg_sim_view(sim.handle)).compute_rhs(u_msh)
    assert _rel(remap_state(box, sim, r_msh, vol, perm), r_box) <= 1e-12
    _, r_own = Oracle(cfg, msh=msh).compute_rhs(u_msh)
    assert _rel(r_own, r_msh) <= 1e-12


def test_unsupported_boundary_condition_tags_are_refused(tmp_path):
    msh = str(tmp_path / "sup.msh")
    write_box_msh(msh, 2, (3, 3), (0.0, 0.0), (1.0, 1.0), side_tags={(0, 0): 10105, (0, 1): 10105}, periodic_dirs=[1])
    cfg = dg.Config(d=2, p=2, lo=(0, 0, 0), hi=(1, 1, 1), test_case="free_stream",
                    vortex=(0, 0, 0, 1.0, 0.4, 0.3, 0, 1.0), bc=("slipwall", "slipwall", "periodic", "periodic"))
    with pytest.raises(dg.DpgError) as ei:
        dg.Simulation(cfg, msh=msh)
    assert ei.value.status == dg.api.DPG_ERR_UNSUPPORTED
