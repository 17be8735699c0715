"""States and an independent numpy restatement for the positivity tests (enforce_positivity_highorder, solve.c:187-233;
compute_relaxation, solve_implicit.c:821-873)."""
import numpy as np

EPS_PHYS = 1e-13
EPS = 1e-15
GM1 = 0.4


def blocks(sim, u):
    """[n_vol, n_var, n_s] view of a state in the reference layout (per volume [n_s, n_var] column-major)."""
    return u.reshape(sim.n_vol, sim.n_var, sim.n_s)


def cons_to_prim(w, d):
    w = w.copy()
    rho_inv = 1.0 / w[0]
    rho2V2 = np.zeros_like(w[0])
    for a in range(d):
        rho2V2 = rho2V2 + w[1 + a] * w[1 + a]
        w[1 + a] = w[1 + a] * rho_inv
    w[d + 1] = GM1 * (w[d + 1] - 0.5 * rho2V2 * rho_inv)
    return w


def prim_to_cons(w, d):
    w = w.copy()
    V2 = np.zeros_like(w[0])
    for a in range(d):
        V2 = V2 + w[1 + a] * w[1 + a]
        w[1 + a] = w[0] * w[1 + a]
    w[d + 1] = w[d + 1] / GM1 + 0.5 * w[0] * V2
    return w


def limit_volume(ue, SB, BS, d):
    """enforce_positivity_highorder on one volume ue [n_var, n_s]; returns (new ue, ok)."""
    nv = d + 2
    b = cons_to_prim(ue @ SB.T, d)
    for vr in (0, nv - 1):
        avg = b[vr].mean()
        if avg < EPS_PHYS:
            return ue, False
        mn = b[vr].min()
        if mn < EPS_PHYS:
            p_ho = max(0.0, min(1.0, (avg - EPS_PHYS) / (avg - mn)))
            for v in range(nv):
                a = b[v].mean()
                if v in (0, nv - 1) and a < EPS_PHYS:
                    a = EPS_PHYS
                b[v] = p_ho * b[v] + (1 - p_ho) * a
    return prim_to_cons(b, d) @ BS.T, True


def bezier_prim_min(ue, SB, d):
    """Smallest primitive density and pressure Bezier coefficients of one volume."""
    b = cons_to_prim(ue @ SB.T, d)
    return b[0].min(), b[d + 1].min()


def relaxation(ue, due, SB, d):
    nv = d + 2
    relax = 1.0
    while True:
        b = cons_to_prim((ue + relax * due) @ SB.T, d)
        if b[0].mean() >= EPS_PHYS and b[nv - 1].mean() >= EPS_PHYS:
            return relax
        relax /= 2.0
        if relax <= EPS:
            return -1.0


def perturbed_state(sim, every=5, seed=0):
    """The initial state with, in every `every`-th volume, a negative pressure (odd volumes of that set) or density
    (even ones) at solution node 0, a vertex of the element, where the Bezier coefficient equals the nodal value; the
    volume averages stay positive.  Returns (state, indices of the perturbed volumes)."""
    rng = np.random.default_rng(seed)
    u = sim.sol_coef().copy()
    ub = blocks(sim, u)
    d = sim.d
    picked = np.arange(0, sim.n_vol, every)
    for k, e in enumerate(picked):
        rho = ub[e, 0, 0]
        m2 = sum(ub[e, 1 + a, 0] ** 2 for a in range(d))
        if k % 2:   # pressure -0.1 .. -0.3 x kinetic energy / 0.4
            ub[e, d + 1, 0] = 0.5 * m2 / rho * (1.0 - rng.uniform(0.25, 0.75))
        else:       # density slightly negative, momentum and energy kept
            ub[e, 0, 0] = -rng.uniform(0.01, 0.05)
    return u, picked
