"""Implicit path on the GPU: matrix-free Newton-GMRES with block-Jacobi, without preconditioner and with the learned
block inverse; MLP gradients against a NumPy restatement.

Steady problem on the periodic box: a uniform free stream u* with velocity (0.6, 0.3) (F(u*) = 0 exactly up to
rounding; F(u*) is still subtracted so that u* is the root to rounding), started from u* plus a seeded perturbation
with zero total mass, momentum and energy (pseudo-transient continuation conserves those totals, which fixes the
solution).  The linearisation about a uniform state has no growing modes; about the isentropic vortex it has
(eigenvalues with real part up to ~1e-2 on a 4x4 p=2 mesh), and restarted GMRES then stagnates once dtau exceeds
their inverse, so the vortex is not used as a steady test here.  Convergence: ||F||_inf <= 1e-10.
"""
import numpy as np
import pytest

import dpgsolver_gb300 as dg
from tests_support import sim_arrays

pytestmark = pytest.mark.gpu


def _problem(n=8, p=2, amp=1e-2):
    sim = dg.Simulation(dg.Config(d=2, p=p, n_elem=(n, n, 1), test_case="free_stream",
                                  vortex=(5.0, 0.0, 0.0, 1.0, 0.6, 0.3, 0.0, 1.0)))
    ctx = dg.GpuContext(sim)
    u_star = sim.sol_coef()
    ctx.upload(u_star)
    ctx.compute_rhs()
    forcing = ctx.rhs()
    a = sim_arrays(sim)
    wt = a["w_vc"] @ a["cv0_vs_vc"]                                   # integral of each basis function (unit J)
    jac = a["jacobian_det_vc"].reshape(sim.n_vol, sim.n_c)[:, 0]
    m = (jac[:, None, None] * wt[None, None, :]) * np.ones((sim.n_vol, sim.n_var, sim.n_s))
    rng = np.random.default_rng(7)
    d = amp * rng.standard_normal(u_star.shape).reshape(sim.n_vol, sim.n_var, sim.n_s)
    d -= (np.sum(m * d, axis=(0, 2)) / np.sum(m, axis=(0, 2)))[None, :, None]   # zero totals (constants are exact)
    return sim, ctx, u_star, forcing, u_star + d.ravel()


def _oracle_residual(sim, u, forcing):
    from oracle import Oracle
    _, F = Oracle(sim).compute_rhs(u)
    return float(np.max(np.abs(F - forcing)))


def test_block_jacobi_newton_converges_and_oracle_agrees():
    sim, ctx, u_star, forcing, u0 = _problem()
    ctx.upload(u0)
    st = ctx.newton_solve(dg.PRECOND_BLOCK_JACOBI, tol=1e-10, forcing=forcing, dtau0=10.0, max_newton=40)
    assert st.residual_final <= 1e-10
    assert st.newton_iterations > 0 and st.gmres_iterations > 0
    # the CPU oracle confirms the converged state (FP64 parity of the residual is ~1e-11 relative)
    assert _oracle_residual(sim, ctx.download(), forcing) <= 1e-9


def test_block_jacobi_beats_no_preconditioner():
    sim, ctx, u_star, forcing, u0 = _problem()
    ctx.upload(u0)
    st_bj = ctx.newton_solve(dg.PRECOND_BLOCK_JACOBI, tol=1e-10, forcing=forcing, dtau0=10.0, max_newton=40)
    ctx.upload(u0)
    with pytest.raises(dg.DpgError) as ei:   # same Newton budget without a preconditioner does not converge
        ctx.newton_solve(dg.PRECOND_NONE, tol=1e-10, forcing=forcing, dtau0=10.0,
                         max_newton=st_bj.newton_iterations, max_gmres=1000)
    assert ei.value.status == dg.api.DPG_ERR_NOT_CONVERGED


def _bf16(a):
    """Round to BF16 (round to nearest even), as each GEMM operand is staged for the tensor cores, back to float64."""
    b = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    b = ((b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return b.view(np.float32).astype(np.float64)


def _numpy_loss_grad(params, dims, x, t):
    """Restatement of the network in mlp.cu: P = I + W3 relu(W2 relu(W1 x + b1) + b2) + b3, loss = mean((P - T)^2);
    every matrix product takes its two operands rounded to BF16 (the tensor-core GEMM), the rest in FP32/FP64."""
    d_in, hid, d_out = dims
    nb = int(round(np.sqrt(d_out)))
    o = 0
    W1 = params[o:o + hid * d_in].reshape(hid, d_in); o += hid * d_in
    b1 = params[o:o + hid].astype(np.float64); o += hid
    W2 = params[o:o + hid * hid].reshape(hid, hid); o += hid * hid
    b2 = params[o:o + hid].astype(np.float64); o += hid
    W3 = params[o:o + d_out * hid].reshape(d_out, hid); o += d_out * hid
    b3 = params[o:o + d_out].astype(np.float64)
    mm = lambda a, b: _bf16(a) @ _bf16(b)
    f32 = lambda a: a.astype(np.float32).astype(np.float64)
    h1 = f32(np.maximum(mm(x, W1.T) + b1, 0))
    h2 = f32(np.maximum(mm(h1, W2.T) + b2, 0))
    y = f32(mm(h2, W3.T) + b3)
    eye = np.eye(nb).ravel()[None, :]
    r = eye + y - t
    loss = np.mean(r * r)
    g = f32(2.0 * r / r.size)
    gW3 = mm(g.T, h2); gb3 = g.sum(0)
    g2 = f32(mm(g, W3) * (h2 > 0))
    gW2 = mm(g2.T, h1); gb2 = g2.sum(0)
    g1 = f32(mm(g2, W2) * (h1 > 0))
    gW1 = mm(g1.T, x); gb1 = g1.sum(0)
    return loss, np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])


@pytest.mark.parametrize("hidden,batch", [(32, 40), (256, 300)])
def test_mlp_gradients_match_numpy(hidden, batch):
    """Forward and backward passes of the tensor-core MLP (tiles of 128 x 128 with ragged edges at these sizes)
    against the numpy restatement with the same BF16 operand rounding."""
    sim = dg.Simulation(dg.Config(d=2, p=1, n_elem=(4, 4, 1)))
    ctx = dg.GpuContext(sim)
    ctx.mlp_enable(hidden=hidden, capacity=64, seed=3)
    dims = ctx.mlp_dims()
    rng = np.random.default_rng(0)
    params = ctx.mlp_params(set_to=(0.2 * rng.standard_normal(ctx.mlp_params().size)).astype(np.float32))
    x = rng.standard_normal((batch, dims[0])).astype(np.float32)
    t = rng.standard_normal((batch, dims[2])).astype(np.float32)
    loss, grad = ctx.mlp_loss_grad(x, t)
    loss_ref, grad_ref = _numpy_loss_grad(params, dims, x, t)
    assert abs(loss - loss_ref) <= 1e-5 * abs(loss_ref)
    assert np.max(np.abs(grad - grad_ref)) <= 1e-4 * np.max(np.abs(grad_ref))


def test_learned_preconditioner_changes_iterations_not_the_answer():
    sim, ctx, u_star, forcing, u0 = _problem()
    ctx.mlp_enable(hidden=128, capacity=16 * sim.n_vol, seed=1)
    ctx.upload(u0)
    st_bj = ctx.newton_solve(dg.PRECOND_BLOCK_JACOBI, tol=1e-10, forcing=forcing, dtau0=10.0, collect_blocks=1,
                             max_newton=40)
    u_bj = ctx.download()
    assert ctx.mlp_samples() > 0
    loss0 = ctx.mlp_train(epochs=1, batch=64, lr=1e-3)
    loss = ctx.mlp_train(epochs=300, batch=64, lr=1e-3)
    assert loss < loss0
    ctx.upload(u0)
    st_mlp = ctx.newton_solve(dg.PRECOND_MLP, tol=1e-10, forcing=forcing, dtau0=10.0, max_newton=40)
    u_mlp = ctx.download()
    print(f"block-Jacobi: {st_bj.newton_iterations} Newton / {st_bj.gmres_iterations} GMRES; learned: "
          f"{st_mlp.newton_iterations} Newton / {st_mlp.gmres_iterations} GMRES, {st_mlp.fallback_steps} fallback steps")
    assert st_mlp.residual_final <= 1e-10
    assert _oracle_residual(sim, u_mlp, forcing) <= 1e-9


def test_gemm_wait_timeout_is_reported_and_the_context_recovers():
    """Failure detection without a GPU fault: with a poll limit of zero the bounded mbarrier waits of the tensor-core
    GEMMs give up while their MMAs are still running.  The kernels then let every issued MMA finish before they free
    their tensor memory, the call returns DPG_ERR_TIMEOUT, and with the default limit restored the same call on the
    same context gives the numpy result again."""
    sim = dg.Simulation(dg.Config(d=2, p=1, n_elem=(4, 4, 1)))
    ctx = dg.GpuContext(sim)
    ctx.mlp_enable(hidden=256, capacity=64, seed=3)
    dims = ctx.mlp_dims()
    rng = np.random.default_rng(1)
    params = ctx.mlp_params(set_to=(0.05 * rng.standard_normal(ctx.mlp_params().size)).astype(np.float32))
    x = rng.standard_normal((300, dims[0])).astype(np.float32)
    t = rng.standard_normal((300, dims[2])).astype(np.float32)
    ctx.mlp_set_wait_limit(0)
    try:
        with pytest.raises(dg.DpgError) as e:
            ctx.mlp_loss_grad(x, t)
    finally:
        ctx.mlp_set_wait_limit(-1)
    assert e.value.status == dg.api.DPG_ERR_TIMEOUT
    loss, grad = ctx.mlp_loss_grad(x, t)
    loss_ref, grad_ref = _numpy_loss_grad(params, dims, x, t)
    assert abs(loss - loss_ref) <= 1e-5 * abs(loss_ref)
    assert np.max(np.abs(grad - grad_ref)) <= 1e-4 * np.max(np.abs(grad_ref))
