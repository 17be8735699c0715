/* Complex-step linearisation of the CPU oracle's residual (TEST INFRASTRUCTURE ONLY; see oracle_dg.h).
 *
 * The oracle's residual (oracle_residual.inc) evaluated on complex states: F(u + i h v) with h = 1e-30 gives
 *   dF/du v = Im F(u + i h v) / h
 * to rounding, with no subtractive cancellation -- the complex-step method of the reference's linearisation test
 * (test_integration_linearization.c: the complex-step Jacobian against the assembled one, 4e-13).  F is the
 * scaled residual m_inv rhs of compute_rhs_dg (dg/solve_dg.c:130-136), serial, face terms subtracted from each
 * volume in increasing (face, side) order as the oracle's face loop does. */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle_dg.h"

#define GAMMA 1.4
#define GM1   0.4

typedef double complex real;
#define RE(x)     creal(x)
#define R_SQRT    csqrt
#define R_POW     cpow
#include "oracle_residual.inc"

double oracle_cs_jvp(oracle_ctx* octx, const double* u, const double* v, double h, double* jv, double* f)
{
	const struct dpg_sim* sim = oracle_ctx_sim(octx);
	struct res_ctx c = { sim, oracle_ctx_m_inv(octx), sim->pde_index == DPG_PDE_NAVIER_STOKES,
	                     (double*)oracle_ctx_grad_operator(octx), NULL, NULL, NULL };
	const int64_t n = sim->vol_dof_off[sim->n_vol];
	size_t stride = 0, blk = 0;
	for (int i = 0; i < sim->n_ops; ++i) {
		if ((size_t)sim->ops[i].n_s*sim->n_eq > stride) stride = (size_t)sim->ops[i].n_s*sim->n_eq;
		if ((size_t)sim->d*sim->ops[i].n_s*sim->n_var > blk) blk = (size_t)sim->d*sim->ops[i].n_s*sim->n_var;
	}
	real* sol = malloc(sizeof(real)*(size_t)n);
	real* rhs = malloc(sizeof(real)*(size_t)n);
	real* fbuf = calloc((size_t)sim->n_face*2*stride,sizeof(real));
	for (int64_t i = 0; i < n; ++i) sol[i] = u[i] + I*(h*v[i]);
	if (c.ns) {
		c.g_v = calloc((size_t)sim->n_vol*blk,sizeof(real));
		c.g_c = calloc((size_t)sim->n_vol*blk,sizeof(real));
		c.g_f = calloc((size_t)sim->n_face*2*blk,sizeof(real));
		for (int e = 0; e < sim->n_vol; ++e) grad_volume(&c,e,sol);
		for (int q = 0; q < sim->n_face; ++q) grad_face(&c,q,sol);
		for (int e = 0; e < sim->n_vol; ++e) grad_gather(&c,e);
	}
	for (int e = 0; e < sim->n_vol; ++e) volume_term(&c,e,sol,rhs);
	for (int q = 0; q < sim->n_face; ++q) face_term(&c,q,sol,&fbuf[(size_t)q*2*stride],&fbuf[((size_t)q*2 + 1)*stride]);
	for (int e = 0; e < sim->n_vol; ++e) {
		const struct dpg_element_ops* ops = &sim->ops[sim->vol_ops[e]];
		int key[DPG_NFL_MAX];
		for (int lf = 0; lf < ops->n_fl; ++lf) key[lf] = 2*sim->vol_face[e*DPG_NFL_MAX + lf] + sim->vol_face_side[e*DPG_NFL_MAX + lf];
		for (int a = 1; a < ops->n_fl; ++a)
			for (int b = a; b > 0 && key[b] < key[b-1]; --b) { const int t = key[b]; key[b] = key[b-1]; key[b-1] = t; }
		real* rv = &rhs[sim->vol_dof_off[e]];
		for (int lf = 0; lf < ops->n_fl; ++lf) {
			const real* src = &fbuf[(size_t)key[lf]*stride];
			for (int k = 0; k < ops->n_s*sim->n_eq; ++k) rv[k] -= src[k];
		}
		scale_m_inv(&c,e,rhs);
	}
	double mx = 0.0;
	for (int64_t i = 0; i < n; ++i) {
		jv[i] = cimag(rhs[i])/h;
		if (f) f[i] = creal(rhs[i]);
		if (fabs(creal(rhs[i])) > mx) mx = fabs(creal(rhs[i]));
	}
	free(sol); free(rhs); free(fbuf); free(c.g_v); free(c.g_c); free(c.g_f);
	return mx;
}
