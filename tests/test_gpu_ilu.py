"""Block ILU(0) preconditioner of the implicit solve (DPG_PRECOND_BLOCK_ILU), the counterpart of the reference's
default PETSc method GMRES(60) + ILU(1), rtol 1e-4 (external/petsc/options_files/petsc_options_gmres_default.txt).

- On a chain of elements (walls at both ends, one element across a periodic direction) the element-block matrix is
  block tridiagonal and its block ILU(0) in volume order is its exact block LU factorisation: preconditioned GMRES
  solves the Newton system in one iteration.
- On the curved Navier-Stokes annulus (BR2, rotating and adiabatic no-slip walls) Newton-GMRES with the block ILU
  reaches ||F||_inf <= 1e-10 in both element orders, with fewer Krylov iterations than block-Jacobi, at the state
  the block-Jacobi solve reaches; the oracle's residual there is at the same level.
"""
import ctypes as C

import numpy as np
import pytest

import dpgsolver_gb300 as dg
from oracle import Oracle

pytestmark = pytest.mark.gpu

TC = dict(d=2, p=2, n_elem=(3, 12, 1), mesh="annulus", lo=(1.0, 0, 0), hi=(2.0, 0, 0), pde="navier_stokes",
          mu=5e-3, Pr=0.72, omega=0.5, test_case="taylor_couette", bc=("noslip_all_rotating", "noslip_adiabatic"))


def _raw_solve(ctx, **kw):
    """dpg_gpu_newton_solve without raising on DPG_ERR_NOT_CONVERGED: (status, stats)."""
    lib = dg.load_library()
    prm = dg.api.NewtonParams()
    lib.dpg_newton_params_default(C.byref(prm))
    for k, v in kw.items():
        assert hasattr(prm, k), k
        setattr(prm, k, v)
    st = dg.api.NewtonStats()
    rc = lib.dpg_gpu_newton_solve(ctx.handle, C.byref(prm), C.byref(st))
    return rc, st


@pytest.mark.parametrize("d,p,n", [(2, 2, (6, 1, 1)), (2, 3, (5, 1, 1)), (3, 1, (4, 1, 1))])
def test_block_ilu_is_exact_on_a_chain(d, p, n):
    bc = ("slipwall", "slipwall") + ("periodic",) * 4
    cfg = dg.Config(d=d, p=p, n_elem=n, lo=(0, 0, 0), hi=(3, 1, 1), jitter=0.0, test_case="free_stream",
                    vortex=(0, 0, 0, 1.0, 0.5, 0.2, 0.1, 1.0), bc=bc)
    sim = dg.Simulation(cfg)
    ctx = dg.GpuContext(sim)
    u = sim.sol_coef()
    ctx.upload(u * (1.0 + 1e-2 * np.random.default_rng(2).standard_normal(u.shape)))
    rc, st = _raw_solve(ctx, precond=dg.PRECOND_BLOCK_ILU, max_newton=1, gmres_rtol=1e-11, dtau0=1.0,
                        gmres_restart=30, max_gmres=30, tol=1e-300)
    assert rc in (dg.api.DPG_OK, dg.api.DPG_ERR_NOT_CONVERGED)
    assert st.newton_iterations == 1 and st.gmres_iterations == 1, (st.newton_iterations, st.gmres_iterations)
    # block-Jacobi needs more Krylov iterations on the same system
    ctx.upload(u * (1.0 + 1e-2 * np.random.default_rng(2).standard_normal(u.shape)))
    rc, sj = _raw_solve(ctx, precond=dg.PRECOND_BLOCK_JACOBI, max_newton=1, gmres_rtol=1e-11, dtau0=1.0,
                        gmres_restart=30, max_gmres=30, tol=1e-300)
    assert sj.gmres_iterations > 1


@pytest.mark.parametrize("order", [dg.api.ILU_ORDER_VOLUME, dg.api.ILU_ORDER_COLOUR], ids=["volume", "colour"])
def test_block_ilu_newton_on_the_annulus(order):
    sim = dg.Simulation(dg.Config(**TC))
    orc = Oracle(sim)
    ctx = dg.GpuContext(sim)
    u0 = orc.initial_solution()
    kw = dict(tol=1e-10, dtau0=1.0, max_newton=200, gmres_restart=60, max_gmres=600, gmres_rtol=1e-4)
    ctx.upload(u0)
    rc, sj = _raw_solve(ctx, precond=dg.PRECOND_BLOCK_JACOBI, **kw)
    assert rc == dg.api.DPG_OK
    u_bj = ctx.download()
    ctx.upload(u0)
    rc, si = _raw_solve(ctx, precond=dg.PRECOND_BLOCK_ILU, ilu_order=order, **kw)
    assert rc == dg.api.DPG_OK and si.residual_final <= 1e-10
    assert si.gmres_iterations < sj.gmres_iterations, (si.gmres_iterations, sj.gmres_iterations)
    u = ctx.download()
    assert np.max(np.abs(u - u_bj)) <= 1e-7 * np.max(np.abs(u_bj))
    m_ref, _ = orc.compute_rhs(u)
    assert m_ref <= 2e-10, m_ref



@pytest.mark.parametrize("precond", [dg.PRECOND_BLOCK_ILU, dg.PRECOND_BLOCK_JACOBI], ids=["ilu", "block-jacobi"])
def test_local_cfl_ramping_reaches_the_same_steady_state(precond):
    """The reference's pseudo time steps for this case (lhs_terms cfl_ramping, cfl_initial 10 in
    input_files/navier_stokes/steady/taylor_couette/test_case.data): per element dtau_e = cfl min(h_e / lambda_e,
    h_e^2 / mu).  Newton-GMRES converges to ||F||_inf <= 1e-10 at the state of the global-dtau solve."""
    sim = dg.Simulation(dg.Config(**TC))
    ctx = dg.GpuContext(sim)
    u0 = sim.sol_coef()
    kw = dict(tol=1e-10, max_newton=200, gmres_restart=60, max_gmres=600, gmres_rtol=1e-4)
    ctx.upload(u0)
    rc, sg = _raw_solve(ctx, precond=dg.PRECOND_BLOCK_JACOBI, dtau0=1.0, **kw)
    assert rc == dg.api.DPG_OK
    u_ref = ctx.download()
    ctx.upload(u0)
    rc, sl = _raw_solve(ctx, precond=precond, cfl_initial=10.0, **kw)
    assert rc == dg.api.DPG_OK and sl.residual_final <= 1e-10, (rc, sl.newton_iterations)
    assert np.max(np.abs(ctx.download() - u_ref)) <= 1e-7 * np.max(np.abs(u_ref))


@pytest.mark.parametrize("p", [2, 3])
def test_block_ilu_on_subdomains_converges_to_the_same_state(p):
    """ilu_parts > 1: contiguous ranges of the element order factorised independently (the couplings between them
    left out); Newton-GMRES reaches the same steady state.  p = 3 gives element blocks of 64 x 64, whose sweeps
    stage their operands in shared memory."""
    sim = dg.Simulation(dg.Config(**dict(TC, p=p)))
    ctx = dg.GpuContext(sim)
    u0 = sim.sol_coef()
    kw = dict(tol=1e-10, max_newton=200, gmres_restart=60, max_gmres=600, gmres_rtol=1e-4, cfl_initial=10.0)
    ctx.upload(u0)
    rc, s1 = _raw_solve(ctx, precond=dg.PRECOND_BLOCK_ILU, **kw)
    assert rc == dg.api.DPG_OK
    u1 = ctx.download()
    ctx.upload(u0)
    rc, s3 = _raw_solve(ctx, precond=dg.PRECOND_BLOCK_ILU, ilu_parts=3, **kw)
    assert rc == dg.api.DPG_OK and s3.residual_final <= 1e-10
    assert np.max(np.abs(ctx.download() - u1)) <= 1e-7 * np.max(np.abs(u1))
