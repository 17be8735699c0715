/* Initial and exact solutions of the test cases on this path.
 *
 * The reference sets sol_coef by evaluating the solution at the solution nodes and converting to coefficients
 * (set_sol_* in test_case/solution/; for the Lagrange basis the conversion is the identity).
 *
 *  - DPG_TC_ISENTROPIC_VORTEX: Shu's isentropic vortex of strength beta centred at (xc, yc) on the free stream
 *    (rho, u, v, w, p); the 3D form has its axis along z.  The exact solution at time t is the initial field
 *    advected with the free-stream velocity on the periodic box (nearest periodic image).
 *  - DPG_TC_ADVECTION_SINE: u0 = sin(2 pi x) sin(2 pi y) advected with constant b_adv on the periodic box
 *    (compute_b_adv constant form, solution_advection_T.c:188-215).
 *  - DPG_TC_FREE_STREAM: the constant free-stream state (used for free-stream preservation checks).
 *  - DPG_TC_PERIODIC_VORTEX: the reference's Gaussian periodic vortex (constructor_sol_periodic_vortex_T,
 *    solution_periodic_vortex_T.c:97-148, set_xy_c and set_data_periodic_vortex, :175-240): rho = p_inf/(Rg t_inf),
 *    (u, v) = V_inf (cos theta, sin theta) + con (-(y-y_c), x-x_c) / r_v^2 exp(-r^2/2),
 *    p = p_inf - rho con^2 / (2 r_v^2) exp(-r^2), r^2 = |x - x_c|^2 / r_v^2, con = V_inf / 10, the centre moving along
 *    theta with period 2 (theta a multiple of pi/2) or 2 sqrt(2).
 *  - DPG_TC_TAYLOR_COUETTE: the flow between the cylinders r_i < r < r_o, the inner one rotating at omega, of
 *    constructor_sol_taylor_couette (solution_taylor_couette_T.c): V_theta = c (1/r - r/r_o^2),
 *    c = omega / (1/r_i^2 - 1/r_o^2), uniform pressure p_i, temperature
 *    T = T_i - 2 c^2 / r_o^2 (mu/kappa) log(r/r_i) - c^2 (mu/kappa) (1/r^2 - 1/r_i^2) (zero heat flux at r_o),
 *    kappa = mu c_p / Pr, c_p = gamma r_s / (gamma - 1), rho = p / (r_s T).
 */
#include <math.h>
#include <string.h>

#include "dpg_host.h"

static double wrap(double x, double lo, double hi)
{
	const double L = hi - lo;
	if (L <= 0.0) return x;
	double y = fmod(x - lo, L);
	if (y < 0.0) y += L;
	return lo + y;
}

void dpg_exact_solution(const struct dpg_sim* sim, double t, const double* xyz, double* u)
{
	const int d = sim->d;
	if (sim->test_case == DPG_TC_ADVECTION_SINE) {
		double x = xyz[0] - sim->b_adv[0]*t, y = (d > 1 ? xyz[1] - sim->b_adv[1]*t : 0.0);
		u[0] = sin(2.0*M_PI*x)*(d > 1 ? sin(2.0*M_PI*y) : 1.0);
		return;
	}
	if (sim->test_case == DPG_TC_PERIODIC_VORTEX) {
		const double r_v = sim->vortex[0], th = sim->vortex[1], V = sim->vortex[2], p_inf = sim->vortex[3];
		const double rho = p_inf/(sim->vortex[5]*sim->vortex[4]);
		const double L = (fmod(th,M_PI/2.0) < DPG_EPS) ? 2.0 : 2.0*sqrt(2.0);
		double u_inf = V*cos(th), v_inf = V*sin(th);
		if (fabs(u_inf) < 1e-1*DPG_EPS) u_inf = 1e-1*DPG_EPS;
		if (fabs(v_inf) < 1e-1*DPG_EPS) v_inf = 1e-1*DPG_EPS;
		const double con = 0.1*V;
		const double frac = fmod(t*V + 0.5*L,L)/L;
		const double xc = (frac - 0.5)*L*cos(th), yc = (frac - 0.5)*L*sin(th);
		const double r2 = ((xyz[0]-xc)*(xyz[0]-xc) + (xyz[1]-yc)*(xyz[1]-yc))/(r_v*r_v);
		const double uu = u_inf - con*(xyz[1]-yc)/(r_v*r_v)*exp(-0.5*r2);
		const double vv = v_inf + con*(xyz[0]-xc)/(r_v*r_v)*exp(-0.5*r2);
		const double pp = p_inf - rho*(con*con)/(2.0*r_v*r_v)*exp(-r2);
		u[0] = rho; u[1] = rho*uu; u[2] = rho*vv;
		if (d == 3) u[3] = 0.0;
		u[d+1] = pp/(DPG_GAMMA - 1.0) + 0.5*rho*(uu*uu + vv*vv);
		return;
	}
	if (sim->test_case == DPG_TC_TAYLOR_COUETTE) {
		const double r_i = sim->tc_data[0], r_o = sim->tc_data[1], p_i = sim->tc_data[2], T_i = sim->tc_data[3];
		const double r = sqrt(xyz[0]*xyz[0] + xyz[1]*xyz[1]), th = atan2(xyz[1],xyz[0]);
		const double c = sim->bc_omega/(1.0/(r_i*r_i) - 1.0/(r_o*r_o));
		const double cp = DPG_GAMMA*sim->r_s/(DPG_GAMMA - 1.0), mu_k = sim->mu/(sim->mu*cp/sim->Pr);
		const double Vt = c*(1.0/r - r/(r_o*r_o));
		const double T = T_i - 2.0*c*c/(r_o*r_o)*mu_k*log(r/r_i) - c*c*mu_k*(1.0/(r*r) - 1.0/(r_i*r_i));
		const double rho = p_i/(sim->r_s*T), uu = -sin(th)*Vt, vv = cos(th)*Vt;
		u[0] = rho; u[1] = rho*uu; u[2] = rho*vv;
		u[3] = p_i/(DPG_GAMMA - 1.0) + 0.5*rho*(uu*uu + vv*vv);
		return;
	}
	const double beta = sim->vortex[0], xc = sim->vortex[1], yc = sim->vortex[2];
	const double rho_inf = sim->vortex[3], u_inf = sim->vortex[4], v_inf = sim->vortex[5],
	             w_inf = sim->vortex[6], p_inf = sim->vortex[7];
	double rho = rho_inf, uu = u_inf, vv = v_inf, ww = w_inf, p = p_inf;
	if (sim->test_case == DPG_TC_ISENTROPIC_VORTEX) {
		/* position relative to the advected centre, taken on the nearest periodic image */
		const double cx = wrap(xc + u_inf*t, sim->domain_lo[0], sim->domain_hi[0]);
		const double cy = wrap(yc + v_inf*t, sim->domain_lo[1], sim->domain_hi[1]);
		double dx = xyz[0] - cx, dy = xyz[1] - cy;
		const double Lx = sim->domain_hi[0] - sim->domain_lo[0], Ly = sim->domain_hi[1] - sim->domain_lo[1];
		if (Lx > 0.0) dx -= Lx*nearbyint(dx/Lx);   /* nearest periodic image (periodic directions only) */
		if (Ly > 0.0) dy -= Ly*nearbyint(dy/Ly);
		const double r2 = dx*dx + dy*dy;
		const double e  = exp(0.5*(1.0 - r2));
		const double T_inf = p_inf/rho_inf;
		const double dT = -(DPG_GAMMA-1.0)*beta*beta/(8.0*DPG_GAMMA*M_PI*M_PI)*e*e;
		const double T  = T_inf + dT;
		rho = rho_inf*pow(T/T_inf,1.0/(DPG_GAMMA-1.0));
		p   = rho*T;
		uu  = u_inf - beta/(2.0*M_PI)*dy*e;
		vv  = v_inf + beta/(2.0*M_PI)*dx*e;
	}
	u[0] = rho;
	u[1] = rho*uu;
	if (d > 1) u[2] = rho*vv;
	if (d > 2) u[3] = rho*ww;
	double V2 = uu*uu + (d > 1 ? vv*vv : 0.0) + (d > 2 ? ww*ww : 0.0);
	u[d+1] = p/(DPG_GAMMA-1.0) + 0.5*rho*V2;
}

void dpg_set_initial_solution(struct dpg_sim* sim)
{
	const int d = sim->d, n_var = sim->n_var;
	for (int v = 0; v < sim->n_vol; ++v) {
		const struct dpg_element_ops* ops = &sim->ops[sim->vol_ops[v]];
		const int n_s = ops->n_s, n_ve = ops->n_ve;
		const double* xyz_ve = &sim->xyz_ve[(size_t)v*DPG_NVE_MAX*3];
		double* sc = &sim->sol_coef[sim->vol_dof_off[v]];
		for (int s = 0; s < n_s; ++s) {
			/* P1 map of the solution node (curved volumes: the parametric map of its (r, theta), the geometry node) */
			double val[DPG_NVE_MAX];
			const double* r = &ops->rst_vs[(size_t)s*d];
			if (ops->e_type == DPG_TRI) {
				dpg_tri_p1_at(r,val,NULL);
			} else if (ops->e_type == DPG_TET) {
				dpg_tet_p1_at(r,val,NULL);
			} else {
				for (int k = 0; k < n_ve; ++k) {
					double t = 1.0;
					for (int a = 0; a < d; ++a) {
						const int b = (k >> a) & 1;
						t *= b ? 0.5*(1.0+r[a]) : 0.5*(1.0-r[a]);
					}
					val[k] = t;
				}
			}
			double x[3] = {0,0,0};
			for (int i = 0; i < d; ++i)
				for (int k = 0; k < n_ve; ++k) x[i] += val[k]*xyz_ve[k*3+i];
			if (sim->geom == DPG_GEOM_CYLINDER) {
				const double rr = x[0], th = x[1];
				x[0] = rr*cos(th); x[1] = rr*sin(th);
			}
			double u[DPG_NVAR_MAX];
			dpg_exact_solution(sim,sim->time,x,u);
			for (int var = 0; var < n_var; ++var) sc[s + (size_t)n_s*var] = u[var];
		}
	}
}
