/* CPU oracle of the DG residual path (TEST INFRASTRUCTURE ONLY).
 *
 * A plain-C restatement, in FP64 and serial, of the reference's compute_rhs_dg, time_step_ssp_rk_33, positivity
 * limiter and Newton under-relaxation on the host data model of include/dpg_simulation.h.  Only the tests, the smoke
 * check and the CPU-baseline leg of the benchmark load it; the library's residual path never calls it.
 */
#ifndef DPG_ORACLE_DG_H
#define DPG_ORACLE_DG_H

#include <stdint.h>

#include "dpg_simulation.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_ctx oracle_ctx;

/* ---- the oracle's own set-up (oracle_setup.c): the data model filled from the problem parameters alone ---- */
struct oracle_params {
	int d, p;              /* 2 (QUAD) or 3 (HEX); uniform order                          */
	int n_elem[3];         /* structured periodic box                                      */
	double lo[3], hi[3];
	double jitter;         /* vertex jitter as a fraction of h (seeded splitmix64)          */
	uint64_t seed;
	int pde_index;         /* DPG_PDE_EULER or DPG_PDE_ADVECTION                           */
	int num_flux;          /* DPG_NUM_FLUX_ROE_PIKE / _LAX_FRIEDRICHS / _UPWIND            */
	int test_case;         /* DPG_TC_*                                                     */
	double vortex[8];      /* beta, xc, yc, rho, u, v, w, p                                */
	double b_adv[3];
	/* boundaries, viscosity and curved geometry */
	int bc_side[6];        /* box sides x-, x+, y-, y+, z-, z+ (0: periodic); annulus: inner, outer wall  */
	int mesh_kind;         /* 0 box, 1 annulus (n_elem[0] radial x n_elem[1] azimuthal, r in lo[0]..hi[0]) */
	double mu, Pr, omega;  /* Navier-Stokes viscosity, Prandtl number, rotating-wall angular velocity     */
	double bc_state[5];    /* Riemann external primitive state                                           */
	double wall_p, wall_T; /* rotating wall (BC_NOSLIP_ALL_ROTATING) pressure and temperature, r_s = 1     */
	int e_type;            /* 0 or DPG_QUAD / DPG_HEX: tensor-product; DPG_TRI: a 2D box of cells split into  */
	                       /* two triangles each; DPG_TET: a 3D box of cells split into six tetrahedra       */
	int p_max;             /* mixed orders: p_max > p draws each volume's order from p .. p_max             */
	uint64_t p_seed;       /* (splitmix64 from p_seed, in volume order); faces take the larger order       */
	/* TRI / TET volume cubature of order p given by the caller (vrule_n[p] > 0): vrule[p][n][d+2], barycentric
	 * coordinates and a weight (weights summing to 1); otherwise Stroud's rule with p + 2 Gauss points per direction */
	int vrule_n[9];
	const double* vrule[9];
	/* TET face cubature of order p given by the caller (frule_n[p] > 0): frule[p][n][4], barycentric coordinates on
	 * the face and a weight (summing to 1), a rule invariant under the face's vertex permutations; otherwise the
	 * symmetrised collapsed rule */
	int frule_n[9];
	const double* frule[9];
};
/* Structured periodic box, or a gmsh 2.2 mesh (periodic in every direction of its bounding box); 0 or < 0. */
int  oracle_sim_structured(const struct oracle_params* prm, struct dpg_sim** out);
int  oracle_sim_gmsh(const struct oracle_params* prm, const char* path, struct dpg_sim** out);
void oracle_sim_free(struct dpg_sim* sim);
void oracle_initial_solution(const struct dpg_sim* sim, double* sol);
void oracle_exact_solution(const struct dpg_sim* sim, double t, const double* xyz, double* u);
/* L2 errors of rho, u, v, (w), p (Euler) or u (SUMMATION_L2_VOL, compute_error.c:545-555) of sol at time t. */
int  oracle_l2_error(const struct dpg_sim* sim, const double* sol, double t, double* err);
void oracle_nodes_gl(int n, double* x, double* w);
void oracle_nodes_gll(int n, double* x, double* w);
int  oracle_gj_invert(int n, const double* a, double* inv);
/* d/dr_a of the order-p GLL Lagrange basis at n_pt reference points r[n_pt][d]: out[d][n_pt][n_s] */
void oracle_grad_operator(int d, int p, int n_pt, const double* r, double* out);

/* ---- the residual restatement (oracle_dg.c) on a data model ----
 * Builds the per-volume mass-matrix inverses (constructor_derived_DG_Solver_Volume_T, dg/volume_solver_dg_T.c:49-78).
 * The tests run it on the data model of oracle_sim_* (and, to check the library's set-up through the residual, on
 * the library's). */
oracle_ctx* oracle_create(const struct dpg_sim* sim);
/* Host threads of the residual (default 1).  Volumes and faces are split among the threads and each volume
 * subtracts its face terms in increasing face order, so every thread count gives the serial result bit for bit. */
void oracle_set_threads(oracle_ctx* ctx, int n_threads);
void        oracle_destroy(oracle_ctx* ctx);

/* compute_rhs_dg (dg/solve_dg.c:130-136): returns ||rhs||_inf; rhs has the layout of sol_coef. */
double oracle_compute_rhs(oracle_ctx* ctx, const double* sol_coef, double* rhs);
/* Same but without the m_inv scaling (the raw volume + face residual of compute_rlhs_common_dg, :182-189). */
double oracle_compute_rhs_unscaled(oracle_ctx* ctx, const double* sol_coef, double* rhs);
/* n_steps of time_step_ssp_rk_33 (solve_explicit.c:252-301) on sol_coef in place; returns the last max_rhs. */
double oracle_rk_step(oracle_ctx* ctx, double* sol_coef, double dt, int n_steps);

/* enforce_positivity_highorder (solve.c:187-233) on every volume, in place; on by default for Euler (as
 * test_case_requires_positivity, test_case.c:63-80) and applied after every stage of oracle_rk_step.  Returns 0, or
 * -1 if some volume's average density or pressure is below EPS_PHYS (the reference stops there; that volume is
 * left unchanged and oracle_rk_step returns NaN). */
int  oracle_enforce_positivity(oracle_ctx* ctx, double* sol_coef);
void oracle_set_positivity(oracle_ctx* ctx, int on);
/* compute_relaxation (solve_implicit.c:821-873) per volume for the Newton update du at u: relax[n_vol]; returns -1
 * if some volume's relaxation fell below EPS (relax -1 there). */
int  oracle_positivity_relaxation(oracle_ctx* ctx, const double* u, const double* du, double* relax);

/* Complex-step Jacobian-vector product of the scaled residual F = m_inv rhs (oracle_cs.c): jv = dF/du(u) v from
 * Im F(u + i h v) / h (h = 1e-30 for exact-to-rounding products); f (may be NULL) receives Re F = F(u).  Serial.
 * Returns ||F(u)||_inf. */
double oracle_cs_jvp(oracle_ctx* ctx, const double* u, const double* v, double h, double* jv, double* f);
/* The data model, per-volume mass inverses and BR2 derivative operator the oracle context holds. */
const struct dpg_sim* oracle_ctx_sim(const oracle_ctx* ctx);
double** oracle_ctx_m_inv(const oracle_ctx* ctx);
const double* oracle_ctx_grad_operator(const oracle_ctx* ctx);

/* Pointwise pieces, exposed for unit tests. */
void oracle_flux_euler(int d, const double* s, double* f /* [d][n_eq] */);
void oracle_numflux_euler_roe_pike(int d, const double* wl, const double* wr, const double* n, double* nf);
void oracle_numflux_euler_lax_friedrichs(int d, const double* wl, const double* wr, const double* n, double* nf);
double oracle_numflux_advection_upwind(int d, const double* b, double wl, double wr, const double* n);

#ifdef __cplusplus
}
#endif
#endif
