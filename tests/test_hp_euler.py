"""Mixed orders for the Euler equations (periodic isentropic vortex on jittered boxes, orders drawn per volume from
1..p_max): the oracle's own mixed-order set-up (TRI / TET with the reference's Witherden-Vincent rules of each order)
gives the library's residual on QUAD, HEX, TRI and TET meshes (1e-12), and its positivity limiter runs each volume
with the Bezier operators of its own order."""
import numpy as np
import pytest

import dpgsolver_gb300 as dg
from oracle import Oracle, Problem
from tests_support import wv_rule

CASES = [("tp", 2, (6, 6, 1), 3), ("tri", 2, (6, 6, 1), 4), ("tet", 3, (6, 6, 3), 3), ("tp", 3, (4, 4, 2), 3)]
IDS = ["quad", "tri", "tet", "hex"]


def problem(element, d, n, p_max):
    c = dict(d=d, p=1, p_max=p_max, p_seed=4, n_elem=n, element=element, pde="euler", num_flux="Roe-Pike",
             test_case="isentropic_vortex", lo=(-5, -5, 0), hi=(5, 5, 1 if d == 2 else 2.5), jitter=0.1, seed=3)
    kw = {}
    if element in ("tri", "tet"):
        kw["vol_rules"] = {p: wv_rule(element, 2 * p) for p in range(1, p_max + 1)}
    if element == "tet":
        kw["face_rules"] = {p: wv_rule("tri", 2 * p) for p in range(1, p_max + 1)}
    return c, kw


@pytest.mark.parametrize("element,d,n,p_max", CASES, ids=IDS)
def test_oracle_set_up_gives_the_library_residual(element, d, n, p_max):
    c, kw = problem(element, d, n, p_max)
    sim = dg.Simulation(dg.Config(**c))
    own = Oracle(Problem(**c, **kw))
    u = sim.sol_coef()
    assert np.max(np.abs(own.initial_solution() - u)) <= 1e-13
    _, r1 = own.compute_rhs(u)
    _, r2 = Oracle(data_model=dg.load_library().dpg_sim_view(sim.handle)).compute_rhs(u)
    assert np.max(np.abs(r1 - r2)) <= 1e-12 * np.max(np.abs(r1))
