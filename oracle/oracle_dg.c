/* CPU oracle of the DG residual path (TEST INFRASTRUCTURE ONLY; see oracle_dg.h).
 *
 * Restates, serially and in FP64, the reference's explicit DG residual:
 *   compute_rhs_dg                          dg/solve_dg.c:130-136
 *   ├ initialize_zero_memory_volumes        solve_T.c:159-182           rhs := 0
 *   ├ compute_volume_rlhs_dg                dg/compute_volume_rlhs_dg_T.c:53-72
 *   │   ├ constructor_sol_vc_interp         compute_volume_rlhs_T.c:277-285   s_vc = cv0_vs_vc * sol_coef
 *   │   ├ compute_Flux_T_euler / _advection flux_euler_T.c:71-143,259-298 / flux_advection_T.c:63-118
 *   │   ├ constructor_flux_ref_piece_T      compute_rlhs_T.c:71-110      fr[:,eq,r] = sum_x m[:,x,r] f[:,x,eq]
 *   │   └ compute_rhs_v_dg_like_T           compute_volume_rlhs_T.c:166-177   rhs += sum_r tw1_vt_vc[r] fr[:,:,r]
 *   ├ compute_face_rlhs_dg                  dg/compute_face_rlhs_dg_T.c:88-114
 *   │   ├ constructor_s_fc_interp_T         boundary_T.c:134-145  (left), boundary_T.c:80-92 (right, permuted)
 *   │   ├ numerical flux                    numerical_flux_euler_T.c:60 (LF), :470 (Roe-Pike),
 *   │   │                                   numerical_flux_advection_T.c:39-75 (upwind)
 *   │   ├ scale_by_Jacobian_e_T             compute_face_rlhs_T.c:337-342   nnf *= jacobian_det_fc
 *   │   └ compute_rhs_f_dg_like_T           compute_face_rlhs_T.c:297-310,347-359
 *   │                                       rhs_l -= tw0_vt_fc_l nnf; nnf -> right order, negated; rhs_r -= tw0 nnf
 *   ├ scale_rhs_by_m_inv_std                dg/solve_dg.c:265-272      rhs := m_inv rhs
 *   └ compute_max_rhs_dg_like               compute_rlhs.c:59-71       ||rhs||_inf
 * and time_step_ssp_rk_33 (solve_explicit.c:252-301) with enforce_positivity_highorder after every stage (solve.c:187-233,
 * for the PDEs of test_case_requires_positivity), and the Newton update's compute_relaxation
 * (solve_implicit.c:821-873).  The mass matrix and its inverse are rebuilt here from the
 * operators and the Jacobian determinants (constructor_mass_T, volume_solver_T.c:115-131).
 * The right-to-left face-node reordering is the gather sR_l[i] = sR[nc_fc[i]] of permute_Matrix_T (GSL convention,
 * matrix_math_T.c:96-126); the left-to-right reordering of nnf applies its inverse (identical to the reference's
 * reuse of nc_fc for the identity and reversal orderings that occur on its meshes).
 */
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "oracle_dg.h"

#define GAMMA 1.4
#define GM1   0.4

struct oracle_ctx {
	const struct dpg_sim* sim;
	double** m_inv;   /* per volume [n_s x n_s] */
	int positivity;   /* enforce_positivity_highorder after each RK stage (test_case_requires_positivity) */
	double* ccSB0;    /* per (type, p) [n_s x n_s]: solution -> Bezier coefficients */
	double* ccBS0;    /* per (type, p) [n_s x n_s]: Bezier -> solution coefficients */
	int n_threads;    /* host threads of the residual                                 */
	double* fbuf;     /* face terms of one residual                                   */
	/* Navier-Stokes (BR2): gradient coefficients, [n_s, n_var] column-major blocks per direction */
	int ns;           /* the PDE has second-order (viscous) terms                      */
	double* cv1_vc;   /* [d][n_c x n_s] d/dr of the solution basis at the volume cubature nodes */
	double* g_v;      /* [n_vol][d][n_s n_var]  grad_coef_v                             */
	double* g_f;      /* [n_face][2][d][n_s n_var] grad_coef_f of each side             */
	double* g_c;      /* [n_vol][d][n_s n_var]  grad_coef = grad_coef_v + sum of the faces' grad_coef_f */
};

/* ---------------------------------------------------------------------------------------------------------- */
static int lu_invert(int n, const double* a, double* ainv)
{
	double* lu = malloc(sizeof(double)*(size_t)n*n);
	int* piv = malloc(sizeof(int)*(size_t)n);
	memcpy(lu,a,sizeof(double)*(size_t)n*n);
	for (int k = 0; k < n; ++k) {
		int pr = k; double best = fabs(lu[(size_t)k*n+k]);
		for (int i = k+1; i < n; ++i) if (fabs(lu[(size_t)i*n+k]) > best) { best = fabs(lu[(size_t)i*n+k]); pr = i; }
		piv[k] = pr;
		if (best == 0.0) { free(lu); free(piv); return -1; }
		if (pr != k) for (int j = 0; j < n; ++j) { double t = lu[(size_t)k*n+j]; lu[(size_t)k*n+j] = lu[(size_t)pr*n+j]; lu[(size_t)pr*n+j] = t; }
		for (int i = k+1; i < n; ++i) {
			const double l = lu[(size_t)i*n+k]/lu[(size_t)k*n+k];
			lu[(size_t)i*n+k] = l;
			for (int j = k+1; j < n; ++j) lu[(size_t)i*n+j] -= l*lu[(size_t)k*n+j];
		}
	}
	double* col = malloc(sizeof(double)*(size_t)n);
	for (int jc = 0; jc < n; ++jc) {
		for (int i = 0; i < n; ++i) col[i] = (i == jc);
		for (int k = 0; k < n; ++k) if (piv[k] != k) { double t = col[k]; col[k] = col[piv[k]]; col[piv[k]] = t; }
		for (int i = 0; i < n; ++i) { double s = col[i]; for (int j = 0; j < i; ++j) s -= lu[(size_t)i*n+j]*col[j]; col[i] = s; }
		for (int i = n-1; i >= 0; --i) { double s = col[i]; for (int j = i+1; j < n; ++j) s -= lu[(size_t)i*n+j]*col[j]; col[i] = s/lu[(size_t)i*n+i]; }
		for (int i = 0; i < n; ++i) ainv[(size_t)i*n+jc] = col[i];
	}
	free(col); free(lu); free(piv);
	return 0;
}

/* bernstein_std (bases.c:1013-1019) */
static double bernstein_std(int p, int i, double r)
{
	double c = 1.0;   /* binomial_coef(p, i) */
	for (int k = 1; k <= i; ++k) c = c*(double)(p-i+k)/(double)k;
	return c*pow(0.5*(1.0+r),i)*pow(0.5*(1.0-r),p-i);
}

oracle_ctx* oracle_create(const struct dpg_sim* sim)
{
	oracle_ctx* ctx = calloc(1,sizeof *ctx);
	ctx->sim = sim;
	ctx->m_inv = calloc((size_t)sim->n_vol,sizeof(double*));
	for (int v = 0; v < sim->n_vol; ++v) {
		const struct dpg_element_ops* ops = &sim->ops[sim->vol_ops[v]];
		const int n_s = ops->n_s, n_c = ops->n_c;
		const double* jdet = &sim->jacobian_det_vc[sim->vol_geo_off[v]];
		double* m = malloc(sizeof(double)*(size_t)n_s*n_s);
		for (int i = 0; i < n_s; ++i)
		for (int j = 0; j < n_s; ++j) {
			double s = 0.0;
			for (int c = 0; c < n_c; ++c)
				s += ops->cv0_vs_vc[(size_t)c*n_s+i]*(ops->w_vc[c]*jdet[c])*ops->cv0_vs_vc[(size_t)c*n_s+j];
			m[(size_t)i*n_s+j] = s;
		}
		ctx->m_inv[v] = malloc(sizeof(double)*(size_t)n_s*n_s);
		lu_invert(n_s,m,ctx->m_inv[v]);
		free(m);
	}
	/* test_case_requires_positivity (test_case.c:63-80): Euler and Navier-Stokes */
	ctx->positivity = (sim->pde_index == DPG_PDE_EULER || sim->pde_index == DPG_PDE_NAVIER_STOKES);
	/* BR2 gradients (has_2nd_order): the derivative operator cv1_vs_vc of the solution basis, formed here from the
	 * data model's cubature nodes */
	ctx->ns = (sim->pde_index == DPG_PDE_NAVIER_STOKES);
	if (ctx->ns) {
		const struct dpg_element_ops* o = &sim->ops[0];
		const size_t blk = (size_t)o->n_s*sim->n_var*o->d;
		ctx->cv1_vc = malloc(sizeof(double)*(size_t)o->d*o->n_c*o->n_s);
		oracle_grad_operator(o->d,o->p,o->n_c,o->rst_vc,ctx->cv1_vc);
		ctx->g_v = calloc((size_t)sim->n_vol*blk,sizeof(double));
		ctx->g_c = calloc((size_t)sim->n_vol*blk,sizeof(double));
		ctx->g_f = calloc((size_t)sim->n_face*2*blk,sizeof(double));
	}
	/* Bezier operators of the (single) element type: ccBS0 = tensor-product Bernstein basis at the solution nodes
	 * (constructor_basis_tp_bezier, bases.c:478-511; the Lagrange basis at its own nodes is the identity),
	 * ccSB0 = its inverse by a solve (element_operators.c:270-297) */
	const struct dpg_element_ops* ops = &sim->ops[0];
	const int n_s = ops->n_s, d = ops->d, p = ops->p;
	ctx->ccBS0 = malloc(sizeof(double)*(size_t)n_s*n_s);
	ctx->ccSB0 = malloc(sizeof(double)*(size_t)n_s*n_s);
	for (int s = 0; s < n_s; ++s)
		for (int b = 0; b < n_s; ++b) {
			double v = 1.0;
			for (int a = 0, t = b; a < d; ++a, t /= (p+1)) v *= bernstein_std(p,t % (p+1),ops->rst_vs[(size_t)s*d+a]);
			ctx->ccBS0[(size_t)s*n_s+b] = v;
		}
	lu_invert(n_s,ctx->ccBS0,ctx->ccSB0);
	return ctx;
}

void oracle_destroy(oracle_ctx* ctx)
{
	if (!ctx) return;
	for (int v = 0; v < ctx->sim->n_vol; ++v) free(ctx->m_inv[v]);
	free(ctx->m_inv); free(ctx->ccSB0); free(ctx->ccBS0); free(ctx->fbuf);
	free(ctx->cv1_vc); free(ctx->g_v); free(ctx->g_f); free(ctx->g_c); free(ctx);
}

void oracle_set_positivity(oracle_ctx* ctx, int on) { ctx->positivity = on; }

void oracle_set_threads(oracle_ctx* ctx, int n_threads)
{
	ctx->n_threads = n_threads < 1 ? 1 : (n_threads > 256 ? 256 : n_threads);
}

/* ---------------------------------------------------------------------------------------------------------- */
/* Positivity (Euler): Bezier coefficients of the conservative variables, read as primitive variables        */
/* ---------------------------------------------------------------------------------------------------------- */

/* convert_variables_T 'c' -> 'p' and 'p' -> 'c' (solution_euler_T.c:136-200) on n coefficients, [n, n_var]
 * column-major */
static void cons_to_prim(int d, int n, double* w)
{
	const int nv = d + 2;
	for (int i = 0; i < n; ++i) {
		const double rho_inv = 1.0/w[i];
		double rho2V2 = 0.0;
		for (int a = 0; a < d; ++a) {
			rho2V2 += w[i + (size_t)n*(1+a)]*w[i + (size_t)n*(1+a)];
			w[i + (size_t)n*(1+a)] = w[i + (size_t)n*(1+a)]*rho_inv;
		}
		w[i + (size_t)n*(nv-1)] = GM1*(w[i + (size_t)n*(nv-1)] - 0.5*rho2V2*rho_inv);
	}
}

static void prim_to_cons(int d, int n, double* w)
{
	const int nv = d + 2;
	for (int i = 0; i < n; ++i) {
		double V2 = 0.0;
		for (int a = 0; a < d; ++a) {
			V2 += w[i + (size_t)n*(1+a)]*w[i + (size_t)n*(1+a)];
			w[i + (size_t)n*(1+a)] = w[i]*w[i + (size_t)n*(1+a)];
		}
		w[i + (size_t)n*(nv-1)] = w[i + (size_t)n*(nv-1)]/GM1 + 0.5*w[i]*V2;
	}
}

/* average_T / minimum_T (math_functions_T.c:162-178) */
static double average(const double* x, int n) { double s = 0.0; for (int i = 0; i < n; ++i) s += x[i]; return s/(double)n; }
static double minimum(const double* x, int n) { double m = 1.7976931348623157e308; for (int i = 0; i < n; ++i) if (x[i] < m) m = x[i]; return m; }

/* y = op x for the n_var columns of x ([n, n_var] column-major; op row-major n x n) */
static void apply_op(const double* op, int n, int n_var, const double* x, double* y)
{
	for (int v = 0; v < n_var; ++v)
		for (int i = 0; i < n; ++i) {
			double s = 0.0;
			for (int j = 0; j < n; ++j) s += op[(size_t)i*n+j]*x[j + (size_t)n*v];
			y[i + (size_t)n*v] = s;
		}
}

/* enforce_positivity_highorder (solve.c:187-233) with correct_coef (solve.c:356-374) on one volume's coefficients:
 * Bezier coefficients, converted to primitive variables; for density, then pressure: stop if the average is below
 * EPS_PHYS, else, if the minimum is below, pull every variable's coefficients toward their average by
 * p_ho = clamp((avg - EPS_PHYS) / (avg - min), 0, 1); back to conservative and to solution coefficients.  Returns
 * -1 where the reference stops with "Average density/pressure approaching 0.0". */
static int positivity_volume(const oracle_ctx* ctx, double* u)
{
	const struct dpg_element_ops* ops = &ctx->sim->ops[0];
	const int n = ops->n_s, d = ops->d, nv = d + 2;
	double b[125*5];
	apply_op(ctx->ccSB0,n,nv,u,b);
	cons_to_prim(d,n,b);
	for (int vr = 0; vr < nv; vr += nv-1) {
		const double avg = average(&b[(size_t)vr*n],n);
		if (avg < DPG_EPS_PHYS) return -1;
		const double mn = minimum(&b[(size_t)vr*n],n);
		if (mn < DPG_EPS_PHYS) {
			const double p_ho = fmax(0.0,fmin(1.0,(avg-DPG_EPS_PHYS)/(avg-mn)));
			for (int v = 0; v < nv; ++v) {
				double* x = &b[(size_t)v*n];
				double a = average(x,n);
				if ((v == 0 || v == nv-1) && a < DPG_EPS_PHYS) a = DPG_EPS_PHYS;
				for (int i = 0; i < n; ++i) x[i] = p_ho*x[i] + (1-p_ho)*a;
			}
		}
	}
	prim_to_cons(d,n,b);
	apply_op(ctx->ccBS0,n,nv,b,u);
	return 0;
}

static void parallel_positivity(oracle_ctx* ctx, double* sol_coef, int* flags);

int oracle_enforce_positivity(oracle_ctx* ctx, double* sol_coef)
{
	const struct dpg_sim* sim = ctx->sim;
	if (!ctx->positivity) return 0;
	int* flags = calloc((size_t)sim->n_vol,sizeof(int));
	parallel_positivity(ctx,sol_coef,flags);   /* volumes are independent: any split gives the serial result */
	int rc = 0;
	for (int v = 0; v < sim->n_vol; ++v) if (flags[v]) rc = -1;
	free(flags);
	return rc;
}

/* compute_relaxation (solve_implicit.c:821-873): the largest relax = 2^-k such that the Bezier coefficients of
 * u + relax du, read as primitive variables, have density and pressure averages of at least EPS_PHYS; -1 where relax
 * falls below EPS (the reference's "Under relaxation approaching zero"). */
static double relaxation_volume(const oracle_ctx* ctx, const double* u, const double* du)
{
	const struct dpg_element_ops* ops = &ctx->sim->ops[0];
	const int n = ops->n_s, d = ops->d, nv = d + 2;
	double b[125*5], db[125*5];
	apply_op(ctx->ccSB0,n,nv,u,b);
	apply_op(ctx->ccSB0,n,nv,du,db);
	double relax = 1.0;
	do {
		for (int i = 0; i < n*nv; ++i) b[i] += relax*db[i];
		cons_to_prim(d,n,b);
		if (!(average(b,n) < DPG_EPS_PHYS || average(&b[(size_t)(nv-1)*n],n) < DPG_EPS_PHYS)) break;
		prim_to_cons(d,n,b);
		for (int i = 0; i < n*nv; ++i) b[i] -= relax*db[i];
		relax /= 2.0;
	} while (relax > DPG_EPS);
	return relax < DPG_EPS ? -1.0 : relax;
}

int oracle_positivity_relaxation(oracle_ctx* ctx, const double* u, const double* du, double* relax)
{
	const struct dpg_sim* sim = ctx->sim;
	int rc = 0;
	for (int v = 0; v < sim->n_vol; ++v) {
		relax[v] = ctx->positivity ? relaxation_volume(ctx,&u[sim->vol_dof_off[v]],&du[sim->vol_dof_off[v]]) : 1.0;
		if (relax[v] < 0.0) rc = -1;
	}
	return rc;
}

/* ---- physical fluxes: f[x*n_eq + eq] -------------------------------------------------------------------- */
void oracle_flux_euler(int d, const double* s, double* f)
{
	const int n_eq = d+2;
	const double rho = s[0], rho_inv = 1.0/rho, E = s[d+1];
	double uvw[3] = {0,0,0}, V2 = 0.0;
	for (int a = 0; a < d; ++a) { uvw[a] = rho_inv*s[1+a]; V2 += uvw[a]*uvw[a]; }
	const double p = GM1*(E - 0.5*rho*V2);
	for (int x = 0; x < d; ++x) {
		f[x*n_eq + 0] = s[1+x];
		for (int a = 0; a < d; ++a)
			f[x*n_eq + 1+a] = s[1+a]*uvw[x] + (a == x ? p : 0.0);
		f[x*n_eq + d+1] = (E+p)*uvw[x];
	}
}

/* ---- numerical fluxes ----------------------------------------------------------------------------------- */
static double min_abs_real(double a, double b) { double c = (fabs(a) < fabs(b) ? a : b); return c < 0.0 ? -c : c; }
static double max_abs_real(double a, double b) { double c = (fabs(a) > fabs(b) ? a : b); return c < 0.0 ? -c : c; }

void oracle_numflux_euler_roe_pike(int d, const double* WL, const double* WR, const double* n, double* nF)
{
	double uL[3] = {0,0,0}, uR[3] = {0,0,0};
	const double rhoL = WL[0], rhoR = WR[0], EL = WL[d+1], ER = WR[d+1];
	const double rhoL_inv = 1.0/rhoL, rhoR_inv = 1.0/rhoR;
	double V2L = 0.0, V2R = 0.0, VnL = 0.0, VnR = 0.0;
	for (int a = 0; a < d; ++a) {
		uL[a] = WL[1+a]*rhoL_inv; uR[a] = WR[1+a]*rhoR_inv;
		V2L += uL[a]*uL[a]; V2R += uR[a]*uR[a];
		VnL += n[a]*uL[a];  VnR += n[a]*uR[a];
	}
	const double pL = GM1*(EL-0.5*rhoL*V2L), HL = (EL+pL)*rhoL_inv;
	const double pR = GM1*(ER-0.5*rhoR*V2R), HR = (ER+pR)*rhoR_inv;
	const double r = sqrt(rhoR/rhoL), rP1 = r+1.0, rho = r*rhoL;
	double u[3] = {0,0,0}, Vn = 0.0, V2 = 0.0;
	for (int a = 0; a < d; ++a) { u[a] = (r*uR[a]+uL[a])/rP1; Vn += n[a]*u[a]; V2 += u[a]*u[a]; }
	const double H = (r*HR+HL)/rP1, c2 = GM1*(H-0.5*V2), c = sqrt(c2);
	const double l1 = min_abs_real(VnL-c,Vn-c), l5 = max_abs_real(VnR+c,Vn+c), l234 = (Vn > 0.0 ? Vn : -Vn);
	const double drho = rhoR-rhoL, dE = ER-EL, dp = pR-pL, dVn = VnR-VnL;
	const double lc1 = 0.5*(l5+l1) - l234, lc2 = 0.5*(l5-l1);
	const double disInter1 = lc1*dp/(c*c) + lc2*rho*dVn/c, disInter2 = lc1*rho*dVn + lc2*dp/c;
	const double rhoVnL = rhoL*VnL, rhoVnR = rhoR*VnR, pLR = pL+pR;
	nF[0] = 0.5*((rhoVnL + rhoVnR) - (l234*drho + disInter1));
	for (int a = 0; a < d; ++a) {
		const double drhou = rhoR*uR[a]-rhoL*uL[a];
		nF[1+a] = 0.5*((rhoVnL*uL[a] + rhoVnR*uR[a] + n[a]*pLR) - (l234*drhou + disInter1*u[a] + disInter2*n[a]));
	}
	nF[d+1] = 0.5*((VnL*(EL+pL) + VnR*(ER+pR)) - (l234*dE + disInter1*H + disInter2*Vn));
}

void oracle_numflux_euler_lax_friedrichs(int d, const double* WL, const double* WR, const double* n, double* nF)
{
	const int n_eq = d+2;
	double fl[3*5], fr[3*5];
	double V2L = 0.0, V2R = 0.0;
	for (int a = 0; a < d; ++a) {
		const double ul = WL[1+a]/WL[0], ur = WR[1+a]/WR[0];
		V2L += ul*ul; V2R += ur*ur;
	}
	const double pL = GM1*(WL[d+1]-0.5*WL[0]*V2L), pR = GM1*(WR[d+1]-0.5*WR[0]*V2R);
	const double maxlL = sqrt(V2L) + sqrt(GAMMA*pL/WL[0]), maxlR = sqrt(V2R) + sqrt(GAMMA*pR/WR[0]);
	const double maxV = (maxlL > maxlR ? maxlL : maxlR);
	oracle_flux_euler(d,WL,fl);
	oracle_flux_euler(d,WR,fr);
	for (int eq = 0; eq < n_eq; ++eq) {
		double s = 0.0;
		for (int x = 0; x < d; ++x) s += n[x]*(fl[x*n_eq+eq] + fr[x*n_eq+eq]);
		nF[eq] = 0.5*(s + maxV*(WL[eq]-WR[eq]));
	}
}

double oracle_numflux_advection_upwind(int d, const double* b, double wl, double wr, const double* n)
{
	double bn = 0.0;
	for (int a = 0; a < d; ++a) bn += b[a]*n[a];
	return (bn > 2.220446049250313e-16 ? bn*wl : bn*wr);
}

/* ---- residual ------------------------------------------------------------------------------------------- */
static void numflux(const struct dpg_sim* sim, const double* wl, const double* wr, const double* n, double* nf)
{
	switch (sim->ind_num_flux[0]) {
	case DPG_NUM_FLUX_ROE_PIKE:       oracle_numflux_euler_roe_pike(sim->d,wl,wr,n,nf); break;
	case DPG_NUM_FLUX_LAX_FRIEDRICHS: oracle_numflux_euler_lax_friedrichs(sim->d,wl,wr,n,nf); break;
	default:                          nf[0] = oracle_numflux_advection_upwind(sim->d,sim->b_adv,wl[0],wr[0],n); break;
	}
}

/* ---- boundary values (test_case/boundary/boundary_euler_T.c, boundary_navier_stokes_T.c) ---------------------- */

static void to_prim(int d, const double* u, double* w)
{
	w[0] = u[0];
	double V2 = 0.0;
	for (int a = 0; a < d; ++a) { w[1+a] = u[1+a]/u[0]; V2 += w[1+a]*w[1+a]; }
	w[d+1] = GM1*(u[d+1] - 0.5*u[0]*V2);
}

static void to_cons(int d, const double* w, double* u)
{
	u[0] = w[0];
	double V2 = 0.0;
	for (int a = 0; a < d; ++a) { u[1+a] = w[0]*w[1+a]; V2 += w[1+a]*w[1+a]; }
	u[d+1] = w[d+1]/GM1 + 0.5*w[0]*V2;
}

/* The boundary state s_b of one face node from the interior trace s_l (unit normal n of the interior, position x):
 *   slip wall (constructor_Boundary_Value_T_euler_slipwall, boundary_euler_T.c:494-530): rho, E kept, momentum
 *     mirrored about the face, rhouvw - 2 (n . rhouvw) n;
 *   Riemann invariants (constructor_Boundary_Value_T_euler_riemann, :99-180) against the external state bc_state;
 *   no-slip, all variables (..._navier_stokes_no_slip_all_rotating, boundary_navier_stokes_T.c:198-256):
 *     s_b = 2 s_wall - s_l with the wall's density and total energy and the rotating-wall velocity omega x r;
 *   no-slip, adiabatic flux (..._no_slip_flux_adiabatic, :258-330): rho, E kept, momentum negated (zero wall
 *     velocity). */
static void boundary_state(const struct dpg_sim* sim, int bc, const double* sl, const double* n, const double* x, double* sb)
{
	const int d = sim->d;
	switch (bc) {
	case DPG_BC_SLIPWALL: {
		double rvn = 0.0;
		for (int a = 0; a < d; ++a) rvn += n[a]*sl[1+a];
		sb[0] = sl[0]; sb[d+1] = sl[d+1];
		for (int a = 0; a < d; ++a) sb[1+a] = sl[1+a] - 2.0*rvn*n[a];
		break;
	} case DPG_BC_RIEMANN: {
		double wl[5], wr[5], w[5] = {0,0,0,0,0}, ur[3];
		to_prim(d,sl,wl);
		wr[0] = sim->bc_state[0];
		for (int a = 0; a < d; ++a) wr[1+a] = sim->bc_state[1+a];
		wr[d+1] = sim->bc_state[4];
		const double cl = sqrt(GAMMA*wl[d+1]/wl[0]), cr = sqrt(GAMMA*wr[d+1]/wr[0]);
		double vnl = 0.0, vnr = 0.0;
		for (int a = 0; a < d; ++a) { vnl += n[a]*wl[1+a]; vnr += n[a]*wr[1+a]; ur[a] = wr[1+a]; }
		const double Rl = vnl + 2.0/GM1*cl, Rr = vnr - 2.0/GM1*cr;
		const double vn = 0.5*(Rl + Rr), c = 0.25*GM1*(Rl - Rr);
		if (fabs(vn) >= fabs(c)) {
			const double* src = (vn < 0.0 ? wr : wl);
			for (int k = 0; k < d+2; ++k) w[k] = src[k];
		} else {
			const double* src = (vn < 0.0 ? wr : wl);
			const double vns = (vn < 0.0 ? vnr : vnl);
			const double ent = src[d+1]/pow(src[0],GAMMA);
			w[0] = pow(1.0/GAMMA*c*c/ent,1.0/GM1);
			for (int a = 0; a < d; ++a) w[1+a] = (src[1+a] - vns*n[a]) + vn*n[a];
			w[d+1] = 1.0/GAMMA*c*c*w[0];
		}
		(void)ur;
		to_cons(d,w,sb);
		break;
	} case DPG_BC_NOSLIP_ALL_ROTATING: {
		const double r = sqrt(x[0]*x[0] + x[1]*x[1]), th = atan2(x[1],x[0]), vt = sim->bc_omega*r;
		const double uw[3] = {-sin(th)*vt, cos(th)*vt, 0.0};
		sb[0] = -sl[0] + 2.0*sim->bc_rho;
		for (int a = 0; a < d; ++a) sb[1+a] = -sl[1+a] + 2.0*sim->bc_rho*uw[a];
		sb[d+1] = -sl[d+1] + 2.0*sim->bc_E;
		break;
	} default: {  /* DPG_BC_NOSLIP_ADIABATIC */
		sb[0] = sl[0]; sb[d+1] = sl[d+1];
		for (int a = 0; a < d; ++a) sb[1+a] = -sl[1+a];
		break;
	} }
}

/* Second-order (viscous) flux of compute_Flux_T_navier_stokes (flux_navier_stokes_T.c:170-245, 1000-1040), with the
 * reference's sign (it is subtracted from the inviscid flux): f[x][eq], constant viscosity mu, Prandtl number Pr;
 * g[x][var] the gradient of the conservative variables. */
static void flux_viscous(int d, double mu, double Pr, const double* s, const double (*g)[5], double f[3][5])
{
	const double rho = s[0], rho_inv = 1.0/rho, E = s[d+1];
	double uvw[3] = {0,0,0}, du[3][3] = {{0}}, tau[3][3] = {{0}}, dTs[3];
	for (int a = 0; a < d; ++a) uvw[a] = s[1+a]*rho_inv;
	for (int i = 0; i < d; ++i)
		for (int x = 0; x < d; ++x) du[i][x] = rho_inv*(g[x][1+i] - g[x][0]*uvw[i]);
	double divV = 0.0;
	for (int a = 0; a < d; ++a) divV += du[a][a];
	for (int i = 0; i < d; ++i)
		for (int j = 0; j < d; ++j)
			tau[i][j] = (i == j) ? mu*2.0*(du[i][i] - divV/3.0) : mu*(du[j][i] + du[i][j]);
	for (int x = 0; x < d; ++x) {
		double dV2 = 0.0;
		for (int a = 0; a < d; ++a) dV2 += uvw[a]*du[a][x];
		dTs[x] = rho_inv*rho_inv*(g[x][d+1]*rho - E*g[x][0]) - 0.5*(2.0*dV2);
	}
	for (int x = 0; x < d; ++x) {
		f[x][0] = -0.0;
		for (int i = 0; i < d; ++i) f[x][1+i] = -tau[i][x];
		double w = 0.0;
		for (int j = 0; j < d; ++j) w += uvw[j]*tau[x][j];
		f[x][d+1] = -(GAMMA/Pr*mu*dTs[x] + w);
	}
}

/* Volume term of volume v into rhs_v (compute_volume_rlhs_dg); with viscous terms the flux is the inviscid one
 * plus the second-order one at the interpolated full gradient cv0_vs_vc grad_coef (constructor_grad_vc_interp,
 * compute_volume_rlhs_T.c:287-295). */
static void volume_term(const oracle_ctx* ctx, int v, const double* sol_coef, double* rhs)
{
	const struct dpg_sim* sim = ctx->sim;
	const int d = sim->d, n_var = sim->n_var, n_eq = sim->n_eq;
	const struct dpg_element_ops* ops = &sim->ops[sim->vol_ops[v]];
	const int n_s = ops->n_s, n_c = ops->n_c;
	const double* sc = &sol_coef[sim->vol_dof_off[v]];
	double* rv = &rhs[sim->vol_dof_off[v]];
	const double* met = &sim->metrics_vc[(size_t)sim->vol_geo_off[v]*d*d];
	double* s_vc = malloc(sizeof(double)*(size_t)n_c*n_var);
	double* fr   = malloc(sizeof(double)*(size_t)n_c*n_eq*d);
	double* g_vc = ctx->ns ? malloc(sizeof(double)*(size_t)d*n_c*n_var) : NULL;
	for (int var = 0; var < n_var; ++var)
		for (int c = 0; c < n_c; ++c) {
			double s = 0.0;
			for (int i = 0; i < n_s; ++i) s += ops->cv0_vs_vc[(size_t)c*n_s+i]*sc[i + (size_t)n_s*var];
			s_vc[c + (size_t)n_c*var] = s;
		}
	if (ctx->ns) {
		const double* gc = &ctx->g_c[(size_t)v*d*n_s*n_var];
		for (int x = 0; x < d; ++x)
			for (int var = 0; var < n_var; ++var)
				for (int c = 0; c < n_c; ++c) {
					double s = 0.0;
					for (int i = 0; i < n_s; ++i)
						s += ops->cv0_vs_vc[(size_t)c*n_s+i]*gc[(size_t)x*n_s*n_var + i + (size_t)n_s*var];
					g_vc[((size_t)x*n_var + var)*n_c + c] = s;
				}
	}
	for (int c = 0; c < n_c; ++c) {
		double s[5], f[3*5];
		for (int var = 0; var < n_var; ++var) s[var] = s_vc[c + (size_t)n_c*var];
		if (sim->n_var == d + 2) oracle_flux_euler(d,s,f);
		else for (int x = 0; x < d; ++x) f[x] = sim->b_adv[x]*s[0];
		if (ctx->ns) {
			double g[3][5], fv[3][5];
			for (int x = 0; x < d; ++x)
				for (int var = 0; var < n_var; ++var) g[x][var] = g_vc[((size_t)x*n_var + var)*n_c + c];
			flux_viscous(d,sim->mu,sim->Pr,s,(const double (*)[5])g,fv);
			for (int x = 0; x < d; ++x)
				for (int eq = 0; eq < n_eq; ++eq) f[x*n_eq + eq] += fv[x][eq];
		}
		for (int eq = 0; eq < n_eq; ++eq)
		for (int r = 0; r < d; ++r) {
			double acc = 0.0;
			for (int x = 0; x < d; ++x) acc += met[c + (size_t)n_c*(x + d*r)]*f[x*n_eq+eq];
			fr[c + (size_t)n_c*(eq + (size_t)n_eq*r)] = acc;
		}
	}
	for (int k = 0; k < n_s*n_eq; ++k) rv[k] = 0.0;
	for (int r = 0; r < d; ++r) {
		const double* tw1 = &ops->tw1_vt_vc[(size_t)r*n_s*n_c];
		for (int eq = 0; eq < n_eq; ++eq)
			for (int i = 0; i < n_s; ++i) {
				double acc = 0.0;
				for (int c = 0; c < n_c; ++c) acc += tw1[(size_t)i*n_c+c]*fr[c + (size_t)n_c*(eq + (size_t)n_eq*r)];
				rv[i + (size_t)n_s*eq] += acc;
			}
	}
	free(s_vc); free(fr); free(g_vc);
}

/* ---- BR2 gradient coefficients (compute_grad_coef_dg_T, dg/compute_grad_coef_dg_T.c) --------------------------- */

/* grad_coef_v[x] = m_inv tw0_vt_vc (detJ d/dx_x) sol_coef, detJ d/dx_x = sum_r m_{x r} d/dr_r at the volume cubature
 * nodes (constructor_grad_xyz_p, :360-380; compute_grad_coef_volumes, :170-212). */
static void grad_volume(const oracle_ctx* ctx, int v, const double* sol_coef)
{
	const struct dpg_sim* sim = ctx->sim;
	const struct dpg_element_ops* ops = &sim->ops[sim->vol_ops[v]];
	const int d = sim->d, n_var = sim->n_var, n_s = ops->n_s, n_c = ops->n_c;
	const double* sc = &sol_coef[sim->vol_dof_off[v]];
	const double* met = &sim->metrics_vc[(size_t)sim->vol_geo_off[v]*d*d];
	double* gv = &ctx->g_v[(size_t)v*d*n_s*n_var];
	double dr[3][64*5], tmp[125*5];
	for (int r = 0; r < d; ++r)
		for (int var = 0; var < n_var; ++var)
			for (int c = 0; c < n_c; ++c) {
				double s = 0.0;
				for (int i = 0; i < n_s; ++i) s += ctx->cv1_vc[((size_t)r*n_c + c)*n_s + i]*sc[i + (size_t)n_s*var];
				dr[r][c + n_c*var] = s;
			}
	for (int x = 0; x < d; ++x) {
		for (int var = 0; var < n_var; ++var)
			for (int i = 0; i < n_s; ++i) {
				double acc = 0.0;
				for (int c = 0; c < n_c; ++c) {
					double gx = 0.0;
					for (int r = 0; r < d; ++r) gx += met[c + (size_t)n_c*(x + d*r)]*dr[r][c + n_c*var];
					acc += ops->cv0_vs_vc[(size_t)c*n_s + i]*ops->w_vc[c]*gx;
				}
				tmp[i + (size_t)n_s*var] = acc;
			}
		for (int var = 0; var < n_var; ++var)
			for (int i = 0; i < n_s; ++i) {
				double acc = 0.0;
				for (int j = 0; j < n_s; ++j) acc += ctx->m_inv[v][(size_t)i*n_s + j]*tmp[j + (size_t)n_s*var];
				gv[(size_t)x*n_s*n_var + i + (size_t)n_s*var] = acc;
			}
	}
}

/* Traces of face f: s_l and s_r at the face nodes in side 0's node order (boundary faces: the boundary state). */
static void face_traces(const struct dpg_sim* sim, int f, const double* sol_coef, double* sl, double* sr)
{
	const int d = sim->d, n_var = sim->n_var;
	const int vl = sim->face_vol[2*f], vr = sim->face_vol[2*f+1];
	const int lfl = sim->face_lf[2*f], lfr = sim->face_lf[2*f+1];
	const struct dpg_element_ops* opl = &sim->ops[sim->vol_ops[vl]];
	const int n_fc = sim->face_nfc[f];
	const int64_t go = sim->face_geo_off[f];
	const int* nc = &sim->nc_fc[go];
	const double* scl = &sol_coef[sim->vol_dof_off[vl]];
	for (int var = 0; var < n_var; ++var)
		for (int q = 0; q < n_fc; ++q) {
			double a = 0.0;
			const double* cl = &opl->cv0_vs_fc[((size_t)lfl*n_fc + q)*opl->n_s];
			for (int i = 0; i < opl->n_s; ++i) a += cl[i]*scl[i + (size_t)opl->n_s*var];
			sl[q + n_fc*var] = a;
		}
	if (vr >= 0) {
		const struct dpg_element_ops* opr = &sim->ops[sim->vol_ops[vr]];
		const double* scr = &sol_coef[sim->vol_dof_off[vr]];
		for (int var = 0; var < n_var; ++var)
			for (int q = 0; q < n_fc; ++q) {
				double b = 0.0;
				const double* cr = &opr->cv0_vs_fc[((size_t)lfr*n_fc + nc[q])*opr->n_s];
				for (int i = 0; i < opr->n_s; ++i) b += cr[i]*scr[i + (size_t)opr->n_s*var];
				sr[q + n_fc*var] = b;
			}
		return;
	}
	for (int q = 0; q < n_fc; ++q) {
		double w[5], b[5], x[3] = {0,0,0};
		for (int var = 0; var < n_var; ++var) w[var] = sl[q + n_fc*var];
		for (int a = 0; a < d; ++a) x[a] = sim->xyz_fc[(size_t)go*d + q + (size_t)n_fc*a];
		boundary_state(sim,sim->face_bc[f],w,&sim->normals_fc[(size_t)(go + q)*d],x,b);
		for (int var = 0; var < n_var; ++var) sr[q + n_fc*var] = b[var];
	}
}

/* grad_coef_f of the two sides of face f: m_inv tw0_vt_fc (jacobian_det_fc n_x (s_num - s_side)), s_num the central
 * numerical solution (u_l + u_r)/2 (get_sol_scale, :690-700; compute_g_coef_f_i and the right side's permuted reuse
 * of the same product, :230-260; boundary faces: s_r the boundary state, compute_g_coef_related_boundary). */
static void grad_face(const oracle_ctx* ctx, int f, const double* sol_coef)
{
	const struct dpg_sim* sim = ctx->sim;
	const int d = sim->d, n_var = sim->n_var;
	const int n_fc = sim->face_nfc[f];
	const int64_t go = sim->face_geo_off[f];
	const int* nc = &sim->nc_fc[go];
	double sl[64*5], sr[64*5], jnd[3][64*5], jnd_r[64*5], tmp[125*5];
	face_traces(sim,f,sol_coef,sl,sr);
	for (int x = 0; x < d; ++x)
		for (int var = 0; var < n_var; ++var)
			for (int q = 0; q < n_fc; ++q) {
				const double diff = -0.5*sl[q + n_fc*var] + 0.5*sr[q + n_fc*var];
				jnd[x][q + n_fc*var] = sim->jacobian_det_fc[go + q]*sim->normals_fc[(size_t)(go + q)*d + x]*diff;
			}
	for (int side = 0; side < 2; ++side) {
		const int v = sim->face_vol[2*f + side], lf = sim->face_lf[2*f + side];
		if (v < 0) continue;
		const struct dpg_element_ops* ops = &sim->ops[sim->vol_ops[v]];
		const int n_s = ops->n_s;
		double* gf = &ctx->g_f[((size_t)f*2 + side)*d*n_s*n_var];
		for (int x = 0; x < d; ++x) {
			const double* src = jnd[x];
			if (side == 1) {   /* into the right side's node order (the normal and s_num - s_r change sign together) */
				for (int var = 0; var < n_var; ++var)
					for (int q = 0; q < n_fc; ++q) jnd_r[nc[q] + n_fc*var] = jnd[x][q + n_fc*var];
				src = jnd_r;
			}
			for (int var = 0; var < n_var; ++var)
				for (int i = 0; i < n_s; ++i) {
					double acc = 0.0;
					const double* tw0 = &ops->tw0_vt_fc[((size_t)lf*n_s + i)*n_fc];
					for (int q = 0; q < n_fc; ++q) acc += tw0[q]*src[q + n_fc*var];
					tmp[i + (size_t)n_s*var] = acc;
				}
			for (int var = 0; var < n_var; ++var)
				for (int i = 0; i < n_s; ++i) {
					double acc = 0.0;
					for (int j = 0; j < n_s; ++j) acc += ctx->m_inv[v][(size_t)i*n_s + j]*tmp[j + (size_t)n_s*var];
					gf[(size_t)x*n_s*n_var + i + (size_t)n_s*var] = acc;
				}
		}
	}
}

/* grad_coef = grad_coef_v + the faces' grad_coef_f, added in face order (add_face_grad_coef_f_to_volumes). */
static void grad_gather(const oracle_ctx* ctx, int v)
{
	const struct dpg_sim* sim = ctx->sim;
	const struct dpg_element_ops* ops = &sim->ops[sim->vol_ops[v]];
	const size_t blk = (size_t)sim->d*ops->n_s*sim->n_var;
	int key[DPG_NFL_MAX];
	for (int lf = 0; lf < ops->n_fl; ++lf) key[lf] = 2*sim->vol_face[v*DPG_NFL_MAX + lf] + sim->vol_face_side[v*DPG_NFL_MAX + lf];
	for (int a = 1; a < ops->n_fl; ++a)
		for (int b = a; b > 0 && key[b] < key[b-1]; --b) { const int t = key[b]; key[b] = key[b-1]; key[b-1] = t; }
	double* gc = &ctx->g_c[(size_t)v*blk];
	memcpy(gc,&ctx->g_v[(size_t)v*blk],sizeof(double)*blk);
	for (int lf = 0; lf < ops->n_fl; ++lf) {
		const double* gf = &ctx->g_f[(size_t)key[lf]*blk];
		for (size_t k = 0; k < blk; ++k) gc[k] += gf[k];
	}
}

/* Face term of face f (compute_face_rlhs_dg): out_l = tw0_vt_fc_l nnf and out_r = tw0_vt_fc_r (-nnf in the right
 * node order), each [n_s, n_eq] column-major; the caller subtracts them from the two volumes' rhs.  Boundary faces
 * use the boundary state as the right state (constructor_Boundary_Value_fcl) and have no out_r.  With viscous terms
 * the numerical flux adds the central flux of the second-order fluxes at the two sides' partially corrected
 * gradients cv0_vs_fc (grad_coef_v + 1.01 NFMAX grad_coef_f) (constructor_partial_grad_fc_interp,
 * compute_face_rlhs_dg_T.c:245-296; compute_Numerical_Flux_T_central, numerical_flux_central_T.c:75-100; the
 * boundary's gradient is the interior one, constructor_Boundary_Value_T_grad_from_internal); on an adiabatic no-slip
 * wall the energy component of the numerical flux is the prescribed normal flux, zero (set_provided_Numerical_Flux
 * _members). */
static void face_term(const oracle_ctx* ctx, int f, const double* sol_coef, double* out_l, double* out_r)
{
	const struct dpg_sim* sim = ctx->sim;
	const int d = sim->d, n_var = sim->n_var, n_eq = sim->n_eq;
	const int vl = sim->face_vol[2*f], vr = sim->face_vol[2*f+1];
	const int lfl = sim->face_lf[2*f], lfr = sim->face_lf[2*f+1];
	const struct dpg_element_ops* opl = &sim->ops[sim->vol_ops[vl]];
	const int n_fc = sim->face_nfc[f];
	const int64_t go = sim->face_geo_off[f];
	const int* nc = &sim->nc_fc[go];
	const double* nrm = &sim->normals_fc[(size_t)go*d];
	const double* jf = &sim->jacobian_det_fc[go];
	double sl[64*5], sr[64*5], nnf[64*5], nnf_r[64*5];
	double gl[3][64*5], gr[3][64*5];
	face_traces(sim,f,sol_coef,sl,sr);
	if (ctx->ns) {
		const double scale = 1.01*(2*d);   /* PENALTY_SCALING * NFMAX (compute_scaling_weak_gradient) */
		for (int side = 0; side < 2; ++side) {
			const int v = sim->face_vol[2*f + side], lf = sim->face_lf[2*f + side];
			if (v < 0) {   /* boundary: the interior gradient */
				for (int x = 0; x < d; ++x) memcpy(gr[x],gl[x],sizeof(double)*(size_t)n_fc*n_var);
				continue;
			}
			const struct dpg_element_ops* ops = &sim->ops[sim->vol_ops[v]];
			const int n_s = ops->n_s;
			const double* gv = &ctx->g_v[(size_t)v*d*n_s*n_var];
			const double* gf = &ctx->g_f[((size_t)f*2 + side)*d*n_s*n_var];
			for (int x = 0; x < d; ++x)
				for (int var = 0; var < n_var; ++var)
					for (int q = 0; q < n_fc; ++q) {
						double acc = 0.0;
						const double* cf = &ops->cv0_vs_fc[((size_t)lf*n_fc + (side ? nc[q] : q))*n_s];
						for (int i = 0; i < n_s; ++i) {
							const size_t k = (size_t)x*n_s*n_var + i + (size_t)n_s*var;
							acc += cf[i]*(gv[k] + scale*gf[k]);
						}
						(side ? gr : gl)[x][q + n_fc*var] = acc;
					}
		}
	}
	const int adiabatic = (vr < 0 && sim->face_bc[f] == DPG_BC_NOSLIP_ADIABATIC);
	for (int q = 0; q < n_fc; ++q) {
		double wl[5], wr[5], nf[5];
		for (int var = 0; var < n_var; ++var) { wl[var] = sl[q + n_fc*var]; wr[var] = sr[q + n_fc*var]; }
		const double* n = &nrm[(size_t)q*d];
		numflux(sim,wl,wr,n,nf);
		if (ctx->ns) {
			double a[3][5], b[3][5], fl[3][5], fr[3][5];
			for (int x = 0; x < d; ++x)
				for (int var = 0; var < n_var; ++var) { a[x][var] = gl[x][q + n_fc*var]; b[x][var] = gr[x][q + n_fc*var]; }
			flux_viscous(d,sim->mu,sim->Pr,wl,(const double (*)[5])a,fl);
			flux_viscous(d,sim->mu,sim->Pr,wr,(const double (*)[5])b,fr);
			for (int x = 0; x < d; ++x)
				for (int eq = 0; eq < n_eq; ++eq) nf[eq] += n[x]*(0.5*fl[x][eq] + 0.5*fr[x][eq]);
			if (adiabatic) nf[d+1] = 0.0;
		}
		for (int eq = 0; eq < n_eq; ++eq) nnf[q + n_fc*eq] = nf[eq]*jf[q];
	}
	/* left: tw0_vt_fc * nnf */
	for (int eq = 0; eq < n_eq; ++eq)
		for (int i = 0; i < opl->n_s; ++i) {
			double acc = 0.0;
			const double* tw0 = &opl->tw0_vt_fc[((size_t)lfl*opl->n_s + i)*n_fc];
			for (int q = 0; q < n_fc; ++q) acc += tw0[q]*nnf[q + n_fc*eq];
			out_l[i + (size_t)opl->n_s*eq] = acc;
		}
	if (vr < 0) return;
	const struct dpg_element_ops* opr = &sim->ops[sim->vol_ops[vr]];
	/* right: nnf into right node order, negated */
	for (int eq = 0; eq < n_eq; ++eq)
		for (int q = 0; q < n_fc; ++q) nnf_r[nc[q] + n_fc*eq] = -nnf[q + n_fc*eq];
	for (int eq = 0; eq < n_eq; ++eq)
		for (int i = 0; i < opr->n_s; ++i) {
			double acc = 0.0;
			const double* tw0 = &opr->tw0_vt_fc[((size_t)lfr*opr->n_s + i)*n_fc];
			for (int q = 0; q < n_fc; ++q) acc += tw0[q]*nnf_r[q + n_fc*eq];
			out_r[i + (size_t)opr->n_s*eq] = acc;
		}
}

/* scale_rhs_by_m_inv_std (dg/solve_dg.c:265-272) on volume v */
static void scale_m_inv(const oracle_ctx* ctx, int v, double* rhs)
{
	const struct dpg_sim* sim = ctx->sim;
	const int n_var = sim->n_var, n_s = sim->ops[sim->vol_ops[v]].n_s;
	double* rv = &rhs[sim->vol_dof_off[v]];
	double tmp[125*5];
	for (int var = 0; var < n_var; ++var)
		for (int i = 0; i < n_s; ++i) {
			double acc = 0.0;
			for (int j = 0; j < n_s; ++j) acc += ctx->m_inv[v][(size_t)i*n_s+j]*rv[j + (size_t)n_s*var];
			tmp[i + (size_t)n_s*var] = acc;
		}
	for (int k = 0; k < n_s*n_var; ++k) rv[k] = tmp[k];
}

/* ---- host threads: a static split of [0, n) per phase ---- */
struct rhs_job {
	const struct dpg_sim* sim;
	const double* sol;
	double* rhs;
	double* fbuf;       /* [n_face][2][stride] face terms */
	size_t stride;
	int phase, t, nt;
	const oracle_ctx* ctx;
	int* flags;         /* positivity: per-volume status */
};

static void run_range(struct rhs_job* job)
{
	const struct dpg_sim* sim = job->sim;
	const int n = (job->phase == 1 || job->phase == 6 ? sim->n_face : sim->n_vol);
	const int lo = (int)((int64_t)n*job->t/job->nt), hi = (int)((int64_t)n*(job->t+1)/job->nt);
	for (int i = lo; i < hi; ++i) {
		if (job->phase == 4) job->flags[i] = positivity_volume(job->ctx,&job->rhs[sim->vol_dof_off[i]]) ? 1 : 0;
		else if (job->phase == 3) scale_m_inv(job->ctx,i,job->rhs);
		else if (job->phase == 5) grad_volume(job->ctx,i,job->sol);
		else if (job->phase == 6) grad_face(job->ctx,i,job->sol);
		else if (job->phase == 7) grad_gather(job->ctx,i);
		else if (job->phase == 0) volume_term(job->ctx,i,job->sol,job->rhs);
		else if (job->phase == 1) face_term(job->ctx,i,job->sol,&job->fbuf[(size_t)i*2*job->stride],
		                                    &job->fbuf[((size_t)i*2 + 1)*job->stride]);
		else {
			/* the volume's (face, side) pairs in increasing order: the serial face loop's order of subtraction */
			const struct dpg_element_ops* ops = &sim->ops[sim->vol_ops[i]];
			int key[DPG_NFL_MAX];
			for (int lf = 0; lf < ops->n_fl; ++lf) key[lf] = 2*sim->vol_face[i*DPG_NFL_MAX + lf] + sim->vol_face_side[i*DPG_NFL_MAX + lf];
			for (int a = 1; a < ops->n_fl; ++a)
				for (int b = a; b > 0 && key[b] < key[b-1]; --b) { const int t = key[b]; key[b] = key[b-1]; key[b-1] = t; }
			double* rv = &job->rhs[sim->vol_dof_off[i]];
			const int n = ops->n_s*sim->n_eq;
			for (int lf = 0; lf < ops->n_fl; ++lf) {
				const double* c = &job->fbuf[(size_t)key[lf]*job->stride];
				for (int k = 0; k < n; ++k) rv[k] -= c[k];
			}
		}
	}
}

static void* run_thread(void* arg) { run_range((struct rhs_job*)arg); return NULL; }

static void parallel_phase(oracle_ctx* ctx, struct rhs_job* base, int phase)
{
	const int nt = ctx->n_threads > 1 ? ctx->n_threads : 1;
	struct rhs_job jobs[256];
	pthread_t th[256];
	for (int t = 0; t < nt; ++t) { jobs[t] = *base; jobs[t].phase = phase; jobs[t].t = t; jobs[t].nt = nt; }
	for (int t = 1; t < nt; ++t) pthread_create(&th[t],NULL,run_thread,&jobs[t]);
	run_range(&jobs[0]);
	for (int t = 1; t < nt; ++t) pthread_join(th[t],NULL);
}

static void parallel_positivity(oracle_ctx* ctx, double* sol_coef, int* flags)
{
	struct rhs_job job = { ctx->sim, NULL, sol_coef, NULL, 0, 0, 0, 1, ctx, flags };
	parallel_phase(ctx,&job,4);
}

double oracle_compute_rhs_unscaled(oracle_ctx* ctx, const double* sol_coef, double* rhs)
{
	const struct dpg_sim* sim = ctx->sim;
	size_t stride = 0;
	for (int i = 0; i < sim->n_ops; ++i)
		if ((size_t)sim->ops[i].n_s*sim->n_eq > stride) stride = (size_t)sim->ops[i].n_s*sim->n_eq;
	if (!ctx->fbuf) ctx->fbuf = malloc(sizeof(double)*(size_t)sim->n_face*2*stride);
	struct rhs_job job = { sim, sol_coef, rhs, ctx->fbuf, stride, 0, 0, 1, ctx, NULL };
	if (ctx->ns) {
		parallel_phase(ctx,&job,5);   /* grad_coef_v                          */
		parallel_phase(ctx,&job,6);   /* grad_coef_f of both sides of each face */
		parallel_phase(ctx,&job,7);   /* grad_coef                            */
	}
	parallel_phase(ctx,&job,0);   /* volume terms (rhs := volume term)        */
	parallel_phase(ctx,&job,1);   /* face terms per face                       */
	parallel_phase(ctx,&job,2);   /* subtracted per volume in face order       */
	double mx = 0.0;
	for (int64_t i = 0; i < sim->vol_dof_off[sim->n_vol]; ++i) if (fabs(rhs[i]) > mx) mx = fabs(rhs[i]);
	return mx;
}

double oracle_compute_rhs(oracle_ctx* ctx, const double* sol_coef, double* rhs)
{
	const struct dpg_sim* sim = ctx->sim;
	oracle_compute_rhs_unscaled(ctx,sol_coef,rhs);
	struct rhs_job job = { sim, sol_coef, rhs, NULL, 0, 0, 0, 1, ctx, NULL };
	parallel_phase(ctx,&job,3);
	double mx = 0.0;
	for (int64_t i = 0; i < sim->vol_dof_off[sim->n_vol]; ++i) if (fabs(rhs[i]) > mx) mx = fabs(rhs[i]);
	return mx;
}

double oracle_rk_step(oracle_ctx* ctx, double* sol_coef, double dt, int n_steps)
{
	const struct dpg_sim* sim = ctx->sim;
	const int64_t n = sim->vol_dof_off[sim->n_vol];
	double* sp = malloc(sizeof(double)*(size_t)n);
	double* rhs = malloc(sizeof(double)*(size_t)n);
	double mx = 0.0;
	for (int step = 0; step < n_steps; ++step) {
		for (int rk = 0; rk < 3; ++rk) {
			mx = oracle_compute_rhs(ctx,sol_coef,rhs);
			switch (rk) {
			case 0: for (int64_t i = 0; i < n; ++i) { sp[i] = sol_coef[i]; sol_coef[i] += dt*rhs[i]; } break;
			case 1: for (int64_t i = 0; i < n; ++i) sol_coef[i] = (1.0/4.0)*(3.0*sp[i] + sol_coef[i] + dt*rhs[i]); break;
			case 2: for (int64_t i = 0; i < n; ++i) sol_coef[i] = (1.0/3.0)*(sp[i] + 2.0*sol_coef[i] + 2.0*dt*rhs[i]); break;
			}
			if (oracle_enforce_positivity(ctx,sol_coef)) { free(sp); free(rhs); return NAN; }
		}
	}
	free(sp); free(rhs);
	return mx;
}
