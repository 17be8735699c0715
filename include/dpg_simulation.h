/* Host-side data model of the DG residual path.
 *
 * This mirrors the members of the reference's `struct Simulation`, `Solver_Volume_T`, `DG_Solver_Volume_T`,
 * `Solver_Face_T` and `Solver_Element` that the DG residual reads, flattened into structure-of-arrays form so that
 * they can be handed to the GPU in a few contiguous copies:
 *
 *   reference member (file:line)                                        here
 *   Simulation::d / pde_index / n_var / n_eq (simulation.h:31-204,
 *     test_case_T.h:50-178)                                              dpg_sim.d, pde_index, n_var, n_eq
 *   Test_Case_T::ind_num_flux[2] (test_case_T.h:116)                     dpg_sim.ind_num_flux[2]
 *   Test_Case_T::solver_proc / solver_type_e / dt / time_final           dpg_sim.solver_proc ...
 *   Solver_Element::cv0_vs_vc, tw1_vt_vc, cv0_vs_fc, tw0_vt_fc, w_vc
 *     (element_solver.h:31-74)                                           dpg_element_ops
 *   Solver_Volume_T::sol_coef, rhs ([n_s, n_var] column-major,
 *     volume_solver_T.h:31-104)                                          dpg_sim.sol_coef / rhs at vol_dof_off[v]
 *   Solver_Volume_T::metrics_vc ([n_c, d, d] column-major),
 *     jacobian_det_vc ([n_c])                                            dpg_sim.metrics_vc / jacobian_det_vc
 *   DG_Solver_Volume_T::sol_coef_p, m_inv (dg/volume_solver_dg_T.h:30-43) dpg_sim.sol_coef_p / m_inv
 *   Face::neigh_info[2].{volume, ind_lf, ind_ord} (face.h:47-97)         dpg_sim.face_vol / face_lf / face_nc
 *   Solver_Face_T::normals_fc ([n_fc, d] row-major), jacobian_det_fc     dpg_sim.normals_fc / jacobian_det_fc
 *
 * All arrays are owned by the dpg_sim and freed by dpg_sim_destroy().
 */
#ifndef DPG_SIMULATION_H
#define DPG_SIMULATION_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Element types, PDE indices, numerical flux and solver codes keep the reference's integer values
 * (definitions_elements.h:33-39, definitions_test_case.h:23-62, definitions_numerical_flux.h:23-31) so that control
 * and test-case files translate one to one. */
enum { DPG_LINE = 1, DPG_TRI = 2, DPG_QUAD = 3, DPG_TET = 4, DPG_HEX = 5, DPG_WEDGE = 6, DPG_PYR = 7 };
enum { DPG_PDE_ADVECTION = 1, DPG_PDE_DIFFUSION = 2, DPG_PDE_EULER = 3, DPG_PDE_NAVIER_STOKES = 4 };
enum { DPG_NUM_FLUX_INVALID = 0, DPG_NUM_FLUX_UPWIND = 11, DPG_NUM_FLUX_BR2_STABLE = 21,
       DPG_NUM_FLUX_ROE_PIKE = 31, DPG_NUM_FLUX_LAX_FRIEDRICHS = 32 };
enum { DPG_SOLVER_E = 100, DPG_SOLVER_I = 200, DPG_SOLVER_EI = 300 };
enum { DPG_SOLVER_E_EULER = 101, DPG_SOLVER_E_SSP_RK_33 = 102, DPG_SOLVER_E_LS_RK_54 = 103 };
enum { DPG_SOLVER_I_DIRECT = 201, DPG_SOLVER_I_ITERATIVE = 202 };

/* Test cases provided by this library (initial + exact solutions). */
enum { DPG_TC_ISENTROPIC_VORTEX = 1,  /* Shu isentropic vortex on a periodic box (2D; 3D: axis along z) */
       DPG_TC_ADVECTION_SINE    = 2,  /* u0 = sin(2 pi x) sin(2 pi y), constant b_adv                      */
       DPG_TC_FREE_STREAM       = 3,  /* constant state: DG must preserve it exactly                         */
       DPG_TC_TAYLOR_COUETTE    = 4,  /* flow between concentric cylinders, inner one rotating (2D NS;
                                       * solution_taylor_couette_T.c: exact velocity and temperature)       */
       DPG_TC_PERIODIC_VORTEX   = 5 };/* the reference's euler/periodic/periodic_vortex: a Gaussian vortex
                                       * advected across [-1,1]^2 (solution_periodic_vortex_T.c:97-240);
                                       * vortex[] = r_v, theta, V_inf, p_inf, t_inf, Rg                     */

/* Boundary conditions: the reference's codes (test_case/boundary/definitions_bc.h:59-69).  0 = interior or
 * periodic face. */
enum { DPG_BC_RIEMANN = 101, DPG_BC_SLIPWALL = 102,
       DPG_BC_NOSLIP_ADIABATIC = 111, DPG_BC_NOSLIP_ALL_ROTATING = 113 };

/* Geometry of the volumes: straight (P1 map of the vertices) or the parametric annulus (curved, geometry order p;
 * the reference's constructor_xyz_cylinder_parametric_T, geometry_parametric_T.c:128-171). */
enum { DPG_GEOM_STRAIGHT = 0, DPG_GEOM_CYLINDER = 1 };

#define DPG_GAMMA 1.4 /* definitions_physics.h:23 */
#define DPG_GM1   0.4 /* definitions_physics.h:24 */
#define DPG_EPS_PHYS 1.0e-13 /* positivity threshold of density and pressure, definitions_physics.h:30 */
#define DPG_EPS      1.0e-15 /* definitions_tol.h:23 */

#define DPG_DIM_MAX   3
#define DPG_NVAR_MAX  5
#define DPG_NFL_MAX   6   /* local faces per element (HEX)   */
#define DPG_NVE_MAX   8   /* vertices per element (HEX)      */
#define DPG_P_MAX     8   /* highest element order           */

/* Dense reference-element operators of one (element type, order p).  All matrices are row-major, exactly the
 * reference's `op_std` (operator.h:40-44) content for the straight (index 0) variants. */
struct dpg_element_ops {
	int e_type, d, p;
	int n_s;      /* solution nodes / basis functions                     */
	int n_c;      /* volume cubature nodes                                */
	int n_fl;     /* local faces                                          */
	int n_fc;     /* cubature nodes per face (uniform for one (type,p))   */
	int n_ve;     /* vertices                                             */

	double* rst_vs;      /* [n_s  x d]  solution nodes (reference coordinates)           */
	double* rst_vc;      /* [n_c  x d]  volume cubature nodes                            */
	double* w_vc;        /* [n_c]       volume cubature weights                          */
	double* rst_fc;      /* [n_fl][n_fc x d] face cubature nodes in volume coordinates   */
	double* w_fc;        /* [n_fc]      face cubature weights (reference face measure)   */
	double* normals_ref; /* [n_fl x d]  outward reference normals                        */

	double* cv0_vs_vc;   /* [n_c x n_s]             */
	double* tw1_vt_vc;   /* [d][n_s x n_c]          (d/dr_d phi)^T * diag(w_vc)            */
	double* cv0_vs_fc;   /* [n_fl][n_fc x n_s]      */
	double* tw0_vt_fc;   /* [n_fl][n_s x n_fc]      phi^T * diag(w_fc)                      */
	double* cv0_vv_vc;   /* [n_c x n_ve]  P1 geometry basis values at cubature nodes          */
	double* cv1_vv_vc;   /* [d][n_c x n_ve] P1 geometry basis derivatives at cubature nodes  */
	double* cv0_vv_fc;   /* [n_fl][n_fc x n_ve]                                              */
	double* cv1_vv_fc;   /* [n_fl][d][n_fc x n_ve]                                           */
	double* m_inv_ref;   /* [n_s x n_s] inverse of cv0^T diag(w) cv0 (unit Jacobian)          */
	/* Bezier (Bernstein) coefficients of the solution, for the positivity limiter (solve.c:187-233):
	 * ccBS0 = Bezier basis at the solution nodes (Bezier -> solution coefficients), ccSB0 = its inverse
	 * (element_operators.c:270-297, get_basis_types:1098-1110); the tensor-product factors in 1D. */
	double* ccBS0_vs_vs; /* [n_s x n_s] row-major; column b = i + n1 (j + n1 k), Bernstein i, j, k   */
	double* ccSB0_vs_vs; /* [n_s x n_s] row-major                                                      */
	double* bez1;        /* [n1 x n1] Bernstein polynomial i at GLL node n: bez1[n n1 + i]            */
	double* bez1_inv;    /* [n1 x n1] inverse of bez1                                                */
	/* Mixed orders: a face takes the larger order p_f of its two volumes (compute_face_reference_order,
	 * face_solver.c:123-132) and its cubature is that of order p_f; the volume basis of order p is interpolated
	 * to it by the reference's cv0_vs_fc[ind_lf][ind_href][0][p_f][p] (get_operator__cv0_vs_fc_T,
	 * compute_face_rlhs_T.c:67-80).  For p < p_f <= DPG_P_MAX: [n_fl][n_fc(p_f) x n_s] and [n_fl][n_s x n_fc(p_f)]
	 * (phi^T diag(w_fc(p_f))), or NULL when no face of order p_f meets a volume of order p.  Order p itself is
	 * cv0_vs_fc / tw0_vt_fc (dpg_face_cv0 / dpg_face_tw0 below pick the right one). */
	double* cv0_vs_fcp[DPG_P_MAX + 1];
	double* tw0_vt_fcp[DPG_P_MAX + 1];
};

struct dpg_sim {
	/* ---- Simulation / Test_Case ---- */
	int d;
	int pde_index;
	int n_var, n_eq;
	int ind_num_flux[2];
	int solver_proc, solver_type_e, solver_type_i;
	int test_case;
	double dt, time, time_final;
	double b_adv[DPG_DIM_MAX];         /* advection velocity (solution_advection_T.c:188-215)          */
	double vortex[8];                  /* isentropic vortex: beta, xc, yc, rho_inf, u_inf, v_inf, w_inf, p_inf */
	double domain_lo[DPG_DIM_MAX], domain_hi[DPG_DIM_MAX];

	/* ---- element operators, one entry per (type, p) present ---- */
	int n_ops;
	struct dpg_element_ops* ops;

	/* ---- volumes ---- */
	int n_vol;
	int* vol_ops;           /* [n_vol] index into ops                                     */
	int* vol_p;             /* [n_vol] p_ref                                              */
	int* vol_affine;        /* [n_vol] 1 if the geometry map is affine (constant metrics)  */
	int64_t* vol_dof_off;   /* [n_vol+1] offset (in doubles) of sol_coef/rhs              */
	int64_t* vol_geo_off;   /* [n_vol+1] offset (in cubature nodes) of the metric arrays  */
	int64_t* vol_minv_off;  /* [n_vol+1] offset (in doubles) of m_inv                      */
	double* xyz_ve;         /* [n_vol][DPG_NVE_MAX][3] vertex coordinates                  */
	double* sol_coef;       /* [vol_dof_off[n_vol]]                                        */
	double* sol_coef_p;     /* RK stage storage                                           */
	double* rhs;            /* [vol_dof_off[n_vol]]                                        */
	double* metrics_vc;     /* per volume [n_c, d, d] column-major: m_ij at c + n_c*(i+d*j) */
	double* jacobian_det_vc;/* per volume [n_c]                                            */
	double* xyz_vc;         /* per volume [n_c, d] column-major                            */
	double* m_inv;          /* per volume [n_s x n_s] row-major                            */
	int* vol_face;          /* [n_vol][DPG_NFL_MAX] face index of each local face          */
	int* vol_face_side;     /* [n_vol][DPG_NFL_MAX] 0 = left (neigh_info[0]), 1 = right    */

	/* ---- faces ---- */
	int n_face;
	int* face_vol;          /* [n_face][2] volume on side 0 / side 1 (-1 if boundary)      */
	int* face_lf;           /* [n_face][2] local face index ind_lf on each side             */
	int* face_nfc;          /* [n_face]    cubature nodes of the face                       */
	int* face_bc;           /* [n_face]    0 interior or periodic                           */
	int64_t* face_geo_off;  /* [n_face+1]  offset (in face nodes)                           */
	int* nc_fc;             /* per face [n_fc]: right-side node index for each left node     */
	double* normals_fc;     /* per face [n_fc, d] row-major, unit outward of side 0          */
	double* jacobian_det_fc;/* per face [n_fc]                                              */
	double* xyz_fc;         /* per face [n_fc, d] column-major                              */

	/* ---- boundary conditions, viscosity and curved geometry ----
	 * A boundary face has face_vol[2f+1] = -1 and its reference BC code in face_bc[f]. */
	int geom;               /* DPG_GEOM_*; DPG_GEOM_CYLINDER: xyz_ve hold (r, theta) of the vertices  */
	double mu, Pr, r_s;     /* constant viscosity, Prandtl number, gas constant (Navier-Stokes)       */
	double bc_omega;        /* angular velocity of the BC_NOSLIP_ALL_ROTATING walls                   */
	double bc_rho, bc_E;    /* density and total energy imposed by BC_NOSLIP_ALL_ROTATING             */
	double bc_state[5];     /* external primitive state (rho, u, v, w, p) of BC_RIEMANN               */
	double tc_data[4];      /* Taylor-Couette: r_i, r_o, p_i (inner pressure), T_i (inner temperature) */

	/* ---- mixed orders ----
	 * ops[k] has order p_min + k (n_ops orders); vol_p / vol_ops give each volume's.  face_nfc[f] and the face
	 * arrays are those of the face's cubature of order face_p[f]. */
	int* face_p;            /* [n_face] face reference order: max(p_l, p_r); a boundary face, p of side 0 */
};

/* Face operators of a volume basis (ops) at the cubature of face order p_f >= ops->p. */
static inline const double* dpg_face_cv0(const struct dpg_element_ops* ops, int p_f)
{
	return p_f == ops->p ? ops->cv0_vs_fc : ops->cv0_vs_fcp[p_f];
}
static inline const double* dpg_face_tw0(const struct dpg_element_ops* ops, int p_f)
{
	return p_f == ops->p ? ops->tw0_vt_fc : ops->tw0_vt_fcp[p_f];
}
/* Order of face f (the volume order when face_p is absent). */
static inline int dpg_face_order(const struct dpg_sim* sim, int f)
{
	return sim->face_p ? sim->face_p[f] : sim->vol_p[sim->face_vol[2*f]];
}

#ifdef __cplusplus
}
#endif

#endif /* DPG_SIMULATION_H */
