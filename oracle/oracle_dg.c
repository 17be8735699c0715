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

typedef double real;
#define RE(x)     (x)
#define R_SQRT    sqrt
#define R_POW     pow
#include "oracle_residual.inc"

struct oracle_ctx {
	struct res_ctx r; /* the data model, mass inverses and BR2 scratch of the residual (oracle_residual.inc) */
	int positivity;   /* enforce_positivity_highorder after each RK stage (test_case_requires_positivity) */
	double* ccSB0;    /* per (type, p) [n_s x n_s]: solution -> Bezier coefficients */
	double* ccBS0;    /* per (type, p) [n_s x n_s]: Bezier -> solution coefficients */
	double* ccSB0k[9];   /* by operator set (order) of mixed-order meshes; [0] = ccSB0 */
	double* ccBS0k[9];
	int n_ops;
	int n_threads;    /* host threads of the residual                                 */
	double* fbuf;     /* face terms of one residual                                   */
	int n_vol;        /* volumes of the data model (kept: the data model may be freed before the context) */
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

/* barycentric coordinates l[d+1] of x in the reference simplex (TRI: element.c:453-466, TET: nodes.c:508-515 of
 * the reference), by Cramer's rule */
static void simplex_bary(int d, const double* x, double* l)
{
	const double s3 = sqrt(3.0), s6 = sqrt(6.0);
	const double V2[3][2] = {{-1.0, -1.0/s3}, {1.0, -1.0/s3}, {0.0, 2.0/s3}};
	const double V3[4][3] = {{-1.0, -1.0/s3, -1.0/s6}, {1.0, -1.0/s3, -1.0/s6}, {0.0, 2.0/s3, -1.0/s6},
	                         {0.0, 0.0, 3.0/s6}};
	if (d == 2) {
		const double a = V2[1][0]-V2[0][0], b = V2[2][0]-V2[0][0], c = V2[1][1]-V2[0][1], e = V2[2][1]-V2[0][1];
		const double rx = x[0]-V2[0][0], ry = x[1]-V2[0][1], det = a*e - b*c;
		l[1] = (rx*e - b*ry)/det;
		l[2] = (a*ry - c*rx)/det;
		l[0] = 1.0 - l[1] - l[2];
		return;
	}
	double M[3][3], r[3];
	for (int i = 0; i < 3; ++i) {
		for (int k = 0; k < 3; ++k) M[i][k] = V3[k+1][i] - V3[0][i];
		r[i] = x[i] - V3[0][i];
	}
#define DET3(A) ((A)[0][0]*((A)[1][1]*(A)[2][2]-(A)[1][2]*(A)[2][1]) - (A)[0][1]*((A)[1][0]*(A)[2][2]-(A)[1][2]*(A)[2][0]) \
                + (A)[0][2]*((A)[1][0]*(A)[2][1]-(A)[1][1]*(A)[2][0]))
	const double det = DET3(M);
	l[0] = 1.0;
	for (int k = 0; k < 3; ++k) {
		double A[3][3];
		memcpy(A,M,sizeof A);
		for (int i = 0; i < 3; ++i) A[i][k] = r[i];
		l[k+1] = DET3(A)/det;
		l[0] -= l[k+1];
	}
#undef DET3
}

/* Bernstein polynomial (a0, .., ad) of degree p on a simplex at barycentric l as the reference's product of 1D
 * Bernstein polynomials of collapsed coordinates (constructor_basis_si_bezier, bases.c:572-608):
 * B(l) = B^{a0+a1}_{a1}(l1/(l0+l1)) B^{a0+a1+a2}_{a2}(l2/(l0+l1+l2)) [B^{p}_{a3}(l3)] */
static double simplex_bernstein(int d, const int* a, const double* l)
{
	double v = 1.0, s = l[0];
	int n = a[0];
	for (int k = 1; k <= d; ++k) {
		n += a[k];
		s += l[k];
		const double t = (s > 0.0 ? l[k]/s : 0.5);   /* collapsed coordinate in [0, 1]; any value where s = 0 */
		v *= bernstein_std(n,a[k],2.0*t - 1.0);
	}
	return v;
}

oracle_ctx* oracle_create(const struct dpg_sim* sim)
{
	oracle_ctx* ctx = calloc(1,sizeof *ctx);
	ctx->r.sim = sim;
	ctx->n_vol = sim->n_vol;
	ctx->r.m_inv = calloc((size_t)sim->n_vol,sizeof(double*));
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
		ctx->r.m_inv[v] = malloc(sizeof(double)*(size_t)n_s*n_s);
		lu_invert(n_s,m,ctx->r.m_inv[v]);
		free(m);
	}
	/* test_case_requires_positivity (test_case.c:63-80): Euler and Navier-Stokes */
	ctx->positivity = (sim->pde_index == DPG_PDE_EULER || sim->pde_index == DPG_PDE_NAVIER_STOKES);
	/* BR2 gradients (has_2nd_order): the derivative operator cv1_vs_vc of the solution basis, formed here from the
	 * data model's cubature nodes */
	ctx->r.ns = (sim->pde_index == DPG_PDE_NAVIER_STOKES);
	if (ctx->r.ns) {
		const struct dpg_element_ops* o = &sim->ops[0];
		const size_t blk = (size_t)o->n_s*sim->n_var*o->d;
		ctx->r.cv1_vc = malloc(sizeof(double)*(size_t)o->d*o->n_c*o->n_s);
		oracle_grad_operator(o->d,o->p,o->n_c,o->rst_vc,ctx->r.cv1_vc);
		ctx->r.g_v = calloc((size_t)sim->n_vol*blk,sizeof(double));
		ctx->r.g_c = calloc((size_t)sim->n_vol*blk,sizeof(double));
		ctx->r.g_f = calloc((size_t)sim->n_face*2*blk,sizeof(double));
	}
	/* Bezier operators of each operator set (order): ccBS0 = Bernstein basis at the solution nodes, tensor-product
	 * (constructor_basis_tp_bezier, bases.c:478-511) or simplex (constructor_basis_si_bezier, bases.c:572-608; the
	 * Lagrange basis at its own nodes is the identity),
	 * ccSB0 = its inverse by a solve (element_operators.c:270-297) */
	ctx->n_ops = (sim->n_ops < 9 ? sim->n_ops : 9);
	for (int ko = 0; ko < ctx->n_ops; ++ko) {
	const struct dpg_element_ops* ops = &sim->ops[ko];
	const int n_s = ops->n_s, d = ops->d, p = ops->p;
	ctx->ccBS0 = malloc(sizeof(double)*(size_t)n_s*n_s);
	ctx->ccSB0 = malloc(sizeof(double)*(size_t)n_s*n_s);
	if (ops->e_type == DPG_TRI || ops->e_type == DPG_TET) {
		for (int s = 0; s < n_s; ++s) {
			double l[4];
			simplex_bary(d,&ops->rst_vs[(size_t)s*d],l);
			int b = 0;
			for (int i = 0; i <= p; ++i)
			for (int j = 0; j <= p-i; ++j)
			for (int k = 0; k <= p-i-j; ++k)
			for (int m = 0; m <= (d-2)*(p-i-j-k); ++m) {
				if (i+j+k+m != p) continue;
				const int a[4] = {i, j, k, m};
				ctx->ccBS0[(size_t)s*n_s + b++] = simplex_bernstein(d,a,l);
			}
		}
	} else {
		for (int s = 0; s < n_s; ++s)
			for (int b = 0; b < n_s; ++b) {
				double v = 1.0;
				for (int a = 0, t = b; a < d; ++a, t /= (p+1)) v *= bernstein_std(p,t % (p+1),ops->rst_vs[(size_t)s*d+a]);
				ctx->ccBS0[(size_t)s*n_s+b] = v;
			}
	}
	lu_invert(n_s,ctx->ccBS0,ctx->ccSB0);
	ctx->ccBS0k[ko] = ctx->ccBS0; ctx->ccSB0k[ko] = ctx->ccSB0;
	}
	ctx->ccBS0 = ctx->ccBS0k[0]; ctx->ccSB0 = ctx->ccSB0k[0];
	return ctx;
}

void oracle_destroy(oracle_ctx* ctx)
{
	if (!ctx) return;
	for (int v = 0; v < ctx->n_vol; ++v) free(ctx->r.m_inv[v]);
	free(ctx->r.m_inv); free(ctx->fbuf);
	for (int k = 0; k < ctx->n_ops; ++k) { free(ctx->ccSB0k[k]); free(ctx->ccBS0k[k]); }
	free(ctx->r.cv1_vc); free(ctx->r.g_v); free(ctx->r.g_f); free(ctx->r.g_c); free(ctx);
}

void oracle_set_positivity(oracle_ctx* ctx, int on) { ctx->positivity = on; }
const struct dpg_sim* oracle_ctx_sim(const oracle_ctx* ctx) { return ctx->r.sim; }
double** oracle_ctx_m_inv(const oracle_ctx* ctx) { return ctx->r.m_inv; }
const double* oracle_ctx_grad_operator(const oracle_ctx* ctx) { return ctx->r.cv1_vc; }

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
static int positivity_volume(const oracle_ctx* ctx, int k, double* u)
{
	const struct dpg_element_ops* ops = &ctx->r.sim->ops[k];
	const int n = ops->n_s, d = ops->d, nv = d + 2;
	double b[125*5];
	apply_op(ctx->ccSB0k[k],n,nv,u,b);
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
	apply_op(ctx->ccBS0k[k],n,nv,b,u);
	return 0;
}

static void parallel_positivity(oracle_ctx* ctx, double* sol_coef, int* flags);

int oracle_enforce_positivity(oracle_ctx* ctx, double* sol_coef)
{
	const struct dpg_sim* sim = ctx->r.sim;
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
	const struct dpg_element_ops* ops = &ctx->r.sim->ops[0];
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
	const struct dpg_sim* sim = ctx->r.sim;
	int rc = 0;
	for (int v = 0; v < sim->n_vol; ++v) {
		relax[v] = ctx->positivity ? relaxation_volume(ctx,&u[sim->vol_dof_off[v]],&du[sim->vol_dof_off[v]]) : 1.0;
		if (relax[v] < 0.0) rc = -1;
	}
	return rc;
}

/* the pointwise pieces, exported for unit tests */
void oracle_flux_euler(int d, const double* s, double* f) { flux_euler_r(d,s,f); }
void oracle_numflux_euler_roe_pike(int d, const double* WL, const double* WR, const double* n, double* nF)
{ numflux_roe_pike_r(d,WL,WR,n,nF); }
void oracle_numflux_euler_lax_friedrichs(int d, const double* WL, const double* WR, const double* n, double* nF)
{ numflux_lax_friedrichs_r(d,WL,WR,n,nF); }
double oracle_numflux_advection_upwind(int d, const double* b, double wl, double wr, const double* n)
{ return numflux_upwind_r(d,b,wl,wr,n); }

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
		if (job->phase == 4) job->flags[i] = positivity_volume(job->ctx,sim->vol_ops[i],&job->rhs[sim->vol_dof_off[i]]) ? 1 : 0;
		else if (job->phase == 3) scale_m_inv(&job->ctx->r,i,job->rhs);
		else if (job->phase == 5) grad_volume(&job->ctx->r,i,job->sol);
		else if (job->phase == 6) grad_face(&job->ctx->r,i,job->sol);
		else if (job->phase == 7) grad_gather(&job->ctx->r,i);
		else if (job->phase == 0) volume_term(&job->ctx->r,i,job->sol,job->rhs);
		else if (job->phase == 1) face_term(&job->ctx->r,i,job->sol,&job->fbuf[(size_t)i*2*job->stride],
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
	struct rhs_job job = { ctx->r.sim, NULL, sol_coef, NULL, 0, 0, 0, 1, ctx, flags };
	parallel_phase(ctx,&job,4);
}

double oracle_compute_rhs_unscaled(oracle_ctx* ctx, const double* sol_coef, double* rhs)
{
	const struct dpg_sim* sim = ctx->r.sim;
	size_t stride = 0;
	for (int i = 0; i < sim->n_ops; ++i)
		if ((size_t)sim->ops[i].n_s*sim->n_eq > stride) stride = (size_t)sim->ops[i].n_s*sim->n_eq;
	if (!ctx->fbuf) ctx->fbuf = malloc(sizeof(double)*(size_t)sim->n_face*2*stride);
	struct rhs_job job = { sim, sol_coef, rhs, ctx->fbuf, stride, 0, 0, 1, ctx, NULL };
	if (ctx->r.ns) {
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
	const struct dpg_sim* sim = ctx->r.sim;
	oracle_compute_rhs_unscaled(ctx,sol_coef,rhs);
	struct rhs_job job = { sim, sol_coef, rhs, NULL, 0, 0, 0, 1, ctx, NULL };
	parallel_phase(ctx,&job,3);
	double mx = 0.0;
	for (int64_t i = 0; i < sim->vol_dof_off[sim->n_vol]; ++i) if (fabs(rhs[i]) > mx) mx = fabs(rhs[i]);
	return mx;
}

double oracle_rk_step(oracle_ctx* ctx, double* sol_coef, double dt, int n_steps)
{
	const struct dpg_sim* sim = ctx->r.sim;
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
