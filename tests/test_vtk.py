"""Visualisation output (dpg_sim_write_vtk), the reference's serial .vtu of output_visualization_vtk_sol
(visualization.c:302-350): one piece per volume with equally spaced points of the volume's order, linear sub-cells,
point data index / p_ref and the solution.

- the file parses as VTK XML; every piece has (p+1)^d (TRI: (p+1)(p+2)/2) points and p^d (TRI: p^2) cells whose
  sub-cells cover the element: their areas sum to the element's area (jittered QUAD, TRI, mixed orders);
- a polynomial state of the element's order is reproduced exactly at the points (1e-12), the points are the
  geometry map of the equally spaced reference nodes (corner points are the vertices);
- Euler: primitive variables and zero errors for the exact initial state interpolated as the reference does."""
import ctypes as C
import xml.etree.ElementTree as ET

import numpy as np
import pytest

import dpgsolver_gb300 as dg
from tests_support import DpgSim


def _pieces(path):
    root = ET.parse(path).getroot()
    assert root.tag == "VTKFile" and root.get("type") == "UnstructuredGrid"
    out = []
    for pc in root.iter("Piece"):
        arrs = {}
        for da in pc.iter("DataArray"):
            txt = (da.text or "").split()
            arrs[da.get("Name") or "Points"] = np.array(txt, dtype=float if da.get("type").startswith("Float") else int)
        out.append((int(pc.get("NumberOfPoints")), int(pc.get("NumberOfCells")), arrs))
    return out


def _area(pts, conn, typ):
    a = 0.0
    if typ == 5:
        for t in conn.reshape(-1, 3):
            p0, p1, p2 = pts[t]
            a += 0.5 * abs((p1[0] - p0[0]) * (p2[1] - p0[1]) - (p2[0] - p0[0]) * (p1[1] - p0[1]))
    else:
        for q in conn.reshape(-1, 4):
            x, y = pts[q, 0], pts[q, 1]
            a += 0.5 * abs(np.dot(x, np.roll(y, -1)) - np.dot(y, np.roll(x, -1)))
    return a


CASES = {
    "quad-p3-jittered": dict(d=2, p=3, n_elem=(3, 2, 1), lo=(0, 0, 0), hi=(1, 1, 1), jitter=0.1, seed=2,
                             pde="advection", num_flux="upwind", test_case="advection_sine"),
    "tri-p2": dict(d=2, p=2, n_elem=(3, 3, 1), element="tri", lo=(0, 0, 0), hi=(1, 1, 1), jitter=0.1, seed=2,
                   pde="advection", num_flux="upwind", test_case="advection_sine"),
    "tri-mixed-1-4": dict(d=2, p=1, p_max=4, p_seed=3, n_elem=(3, 3, 1), element="tri", lo=(0, 0, 0), hi=(1, 1, 1),
                          jitter=0.1, seed=2, pde="advection", num_flux="upwind", test_case="advection_sine"),
}


@pytest.mark.parametrize("case", list(CASES.values()), ids=list(CASES))
def test_pieces_cover_the_mesh_and_reproduce_polynomials(tmp_path, case):
    sim = dg.Simulation(dg.Config(**case))
    s = C.cast(sim.handle, C.POINTER(DpgSim)).contents
    n_vol = sim.n_vol
    vp = np.ctypeslib.as_array(s.vol_p, shape=(n_vol,)).copy()
    off = np.ctypeslib.as_array(s.vol_dof_off, shape=(n_vol + 1,)).copy()
    tri = case.get("element") == "tri"
    # a state that is, on every volume, the polynomial q(x, y) = 1 + x - 2 y + x y (degree 2, total degree 2):
    # exactly representable for p >= 2 (TRI) / p >= 1 with the xy term (QUAD); at the solution nodes
    u = np.empty(sim.n_dof)
    xs = _solution_nodes(sim, s)
    for v in range(n_vol):
        x, y = xs[v][:, 0], xs[v][:, 1]
        u[off[v]:off[v + 1]] = 1 + x - 2 * y + (x * y if (not tri or vp[v] >= 2) else 0.0)
    sim.set_sol_coef(u)
    path = str(tmp_path / "sol.vtu")
    sim.write_vtk(path)
    pieces = _pieces(path)
    assert len(pieces) == n_vol
    total = 0.0
    for v, (n_pt, n_cell, a) in enumerate(pieces):
        p = int(vp[v])
        assert n_pt == ((p + 1) * (p + 2) // 2 if tri else (p + 1) ** 2)
        assert n_cell == p * p
        assert np.all(a["index"] == v) and np.all(a["p_ref"] == p)
        pts = a["Points"].reshape(-1, 3)
        conn = a["connectivity"]
        assert conn.min() >= 0 and conn.max() < n_pt
        total += _area(pts, conn, int(a["types"][0]))
        x, y = pts[:, 0], pts[:, 1]
        q = 1 + x - 2 * y + (x * y if (not tri or p >= 2) else 0.0)
        assert np.max(np.abs(a["u"] - q)) <= 1e-12
        xv = np.ctypeslib.as_array(s.xyz_ve, shape=(n_vol * 24,)).reshape(n_vol, 8, 3)[v]
        corners = [0, p, (p + 1) * (p + 2) // 2 - 1] if tri else [0, p, (p + 1) * p, (p + 1) ** 2 - 1]
        verts = [0, 1, 2] if tri else [0, 1, 2, 3]
        assert np.max(np.abs(pts[corners, :2] - xv[verts, :2])) <= 1e-14
    assert abs(total - 1.0) <= 1e-12


def _solution_nodes(sim, s):
    """Physical coordinates of every volume's solution nodes (P1 map of its vertices)."""
    out = []
    n_vol = sim.n_vol
    xv_all = np.ctypeslib.as_array(s.xyz_ve, shape=(n_vol * 24,)).reshape(n_vol, 8, 3)
    for v in range(n_vol):
        o = s.ops[s.vol_ops[v]]
        r = np.ctypeslib.as_array(o.rst_vs, shape=(o.n_s * 2,)).reshape(o.n_s, 2)
        xv = xv_all[v]
        if o.n_ve == 3:   # barycentric coordinates on (-1,-1/sqrt3), (1,-1/sqrt3), (0,2/sqrt3)
            l2 = (np.sqrt(3.0) * r[:, 1] + 1.0) / 3.0
            l1 = (r[:, 0] + 1.0 - l2) / 2.0
            w = np.stack([1.0 - l1 - l2, l1, l2], axis=1)
        else:
            a, b = (1 - r[:, 0]) / 2, (1 + r[:, 0]) / 2
            c, d = (1 - r[:, 1]) / 2, (1 + r[:, 1]) / 2
            w = np.stack([a * c, b * c, a * d, b * d], axis=1)
        out.append(w @ xv[: w.shape[1], :2])
    return out


def test_euler_primitive_variables_and_errors(tmp_path):
    sim = dg.Simulation(dg.Config(d=2, p=2, n_elem=(2, 2, 1)))
    path = str(tmp_path / "euler.vtu")
    sim.write_vtk(path)
    pieces = _pieces(path)
    assert len(pieces) == 4
    for n_pt, n_cell, a in pieces:
        assert n_pt == 9 and n_cell == 4
        assert a["$\\mathbf{v}$"].shape == (3 * n_pt,)
        assert np.all(a["$\\rho$"] > 0) and np.all(a["$\\mathit{p}$"] > 0)
        for k in ("$|\\rho-\\rho_e|$", "$|\\mathbf{v}-\\mathbf{v}_e|$", "$|p-p_e|$"):
            assert np.max(a[k]) <= 1e-13, k   # the initial state is the interpolated exact solution
    with pytest.raises(dg.DpgError) as e:
        sim.write_vtk("/nonexistent-dir/x.vtu")
    assert e.value.status == dg.api.DPG_ERR_IO
