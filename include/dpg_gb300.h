/* C ABI of the GB300 DG residual engine.
 *
 * Two halves:
 *   1. dpg_sim_*  : host set-up of the simulation (mesh, reference-element operators, geometry, initial solution),
 *                   the part of the reference that runs before the residual (constructor_Simulation,
 *                   constructor_derived_Elements / constructor_derived_computational_elements, set_up_solver_geometry,
 *                   set_initial_solution).  Pure host code; usable without a GPU.
 *   2. dpg_gpu_*  : the residual hot path on one GB300.  These are the calls a reference-side binding replaces
 *                   compute_rhs / time_step_ssp_rk_33 / solve_explicit / solve_implicit with.
 *
 * Conventions: plain pointers and sizes; every call returns an int status (DPG_OK == 0) and never aborts; a context
 * owns one CUDA stream and is not thread-safe; host arrays are the reference's per-volume column-major [n_s, n_var]
 * sol_coef / rhs blocks concatenated in volume order (volume v starts at v * n_s * n_var).
 */
#ifndef DPG_GB300_H
#define DPG_GB300_H

#include <stdint.h>

#include "dpg_simulation.h"   /* element / PDE / numerical-flux / solver / test-case codes, the host data model */

#ifdef __cplusplus
extern "C" {
#endif

struct dpg_sim;
typedef struct dpg_gpu_ctx dpg_gpu_ctx;

/* ---- status codes ---- */
enum {
	DPG_OK                = 0,
	DPG_ERR_INVALID       = 1,  /* bad argument or inconsistent input                          */
	DPG_ERR_UNSUPPORTED   = 2,  /* PDE / flux / element combination not provided (reference: EXIT_UNSUPPORTED) */
	DPG_ERR_CUDA          = 3,  /* a CUDA runtime call failed                                  */
	DPG_ERR_NONFINITE     = 4,  /* the residual or state contains NaN/Inf                       */
	DPG_ERR_TIMEOUT       = 5,  /* a bounded device-side wait gave up                          */
	DPG_ERR_NOT_CONVERGED = 6,  /* Newton/GMRES did not reach the tolerance                    */
	DPG_ERR_NO_DEVICE     = 7,  /* no CUDA device visible                                       */
	DPG_ERR_IO            = 8,  /* control file could not be read                               */
	DPG_ERR_TOO_LARGE     = 9   /* problem exceeds the fixed scratch of dpg_gpu_compute_rhs_noalloc */
};
const char* dpg_status_string(int status);

/* ---- precision of the operator contractions (geometry, fluxes, RK and norms stay FP64) ---- */
enum {
	DPG_PREC_FP64        = 0,  /* FP64 FMA contractions (the FP64-on-GPU form)                         */
	DPG_PREC_BF16X3      = 1,  /* hi/lo BF16 split, 3 tcgen05 products, FP32 accumulate                 */
	DPG_PREC_TF32X3      = 2,  /* hi/lo TF32 split, 3 tcgen05 products, FP32 accumulate                 */
	DPG_PREC_BF16_SLICED = 3   /* exponent-aligned 8-bit BF16 slices, exact FP32 level sums, FP64 combine */
};

/* =====================================================================================================
 * Host set-up
 * ===================================================================================================== */
struct dpg_sim_params {
	int d;                 /* 2 or 3                                                    */
	int e_type;            /* DPG_QUAD or DPG_HEX                                       */
	int p;                 /* order (uniform)                                           */
	int n_elem[3];         /* structured periodic mesh size per direction               */
	double lo[3], hi[3];   /* box                                                       */
	double jitter;         /* vertex jitter as a fraction of h (periodic-consistent)    */
	uint64_t seed;         /* seed of the jitter                                        */
	int pde_index;         /* DPG_PDE_EULER or DPG_PDE_ADVECTION                        */
	int num_flux;          /* DPG_NUM_FLUX_ROE_PIKE / _LAX_FRIEDRICHS / _UPWIND         */
	int test_case;         /* DPG_TC_*                                                  */
	double vortex[8];      /* beta, xc, yc, rho, u, v, w, p                             */
	double b_adv[3];       /* advection velocity                                        */
	int solver_proc, solver_type_e;
	double dt, time_final;
	/* boundaries, viscosity and curved geometry (appended: the fields above keep their offsets) */
	int bc_side[6];        /* box sides x-, x+, y-, y+, z-, z+: 0 periodic, else a DPG_BC_* code          */
	int mesh_kind;         /* DPG_MESH_BOX (structured box) or DPG_MESH_ANNULUS (n_elem[0] radial x        */
	                       /* n_elem[1] azimuthal curved QUADs between radii lo[0] and hi[0], periodic in theta; */
	                       /* bc_side[0] the inner wall, bc_side[1] the outer wall)                          */
	int num_flux_2nd;      /* DPG_NUM_FLUX_BR2_STABLE for Navier-Stokes                                    */
	double mu, Pr;         /* constant viscosity and Prandtl number (Navier-Stokes)                       */
	double omega;          /* angular velocity of BC_NOSLIP_ALL_ROTATING walls                            */
	double bc_state[5];    /* BC_RIEMANN external primitive state rho, u, v, w, p                         */
	double wall_p, wall_T; /* pressure and temperature imposed by BC_NOSLIP_ALL_ROTATING (r_s = 1)        */
	/* mixed orders (appended): p_max > p draws each volume's order uniformly from p .. p_max, in volume order,  */
	/* as p + splitmix64(state) mod (p_max - p + 1) with state starting at p_seed (the reference's p_ref range  */
	/* [p_ref[0], p_ref[1]], simulation.h; faces take the larger order of their volumes).  Linear advection on   */
	/* periodic straight-sided meshes; p_max <= p: uniform order p.                                             */
	int p_max;
	uint64_t p_seed;
};
enum { DPG_MESH_BOX = 0, DPG_MESH_ANNULUS = 1 };
void dpg_sim_params_default(struct dpg_sim_params* prm);

/* Build mesh, operators, geometry and the initial solution.  Replaces constructor_Simulation (simulation.c:128-144)
 * + constructor_derived_computational_elements(IL_SOLVER_DG) + set_up_solver_geometry (geometry_T.c:165-185) +
 * set_initial_solution for the structured periodic meshes of this path. */
int  dpg_sim_create(const struct dpg_sim_params* prm, struct dpg_sim** sim_out);
/* Same on a gmsh 2.2 ASCII mesh (the reference's mesh input, mesh_readers.c) of prm->e_type: 4-node
 * quadrilaterals or 3-node triangles (d = 2), 8-node hexahedra or 4-node tetrahedra (d = 3); boundaries periodic
 * through the file's $Periodic node correspondences or, for QUAD/HEX, tagged with a boundary condition of this path
 * by their boundary elements' physical tags; the structured-mesh fields of prm (n_elem, lo, hi, jitter) are not
 * used.  DPG_ERR_IO for an unreadable file, DPG_ERR_UNSUPPORTED for other element types or conditions, a boundary
 * face without a periodic image or condition, or a binary / non-2.x file. */
int  dpg_sim_create_from_gmsh(const struct dpg_sim_params* prm, const char* msh_path, struct dpg_sim** sim_out);

/* The reference's volume and face lists, as a binding reads them from its struct Simulation (sim->volumes,
 * sim->faces): replaces constructor_Volumes / constructor_Faces (volume.c, face.c) and the geometry set-up
 * (set_up_solver_geometry_T, geometry_T.c:165-185) for straight-sided QUAD / HEX volumes.  Faces keep the
 * reference's sides; operators, metrics, normals and face node correspondences are formed by this library.  The
 * nodes of a periodic face pair are matched modulo the extents of prm->lo .. prm->hi in each direction where
 * hi > lo (the periodic lengths; else the vertices' bounding box); the rest of prm is the problem. */
struct dpg_ref_volume {
	const double* xyz_ve;     /* Volume::xyz_ve: [2^d][d], vertices in the reference's tensor-product order       */
	const double* sol_coef;   /* Solver_Volume_T::sol_coef: [n_s(p_ref), n_var] column-major, or NULL (the test   */
	                          /* case's initial state)                                                            */
	int p_ref;                /* Solver_Volume_T::p_ref (an adapted mesh's per-volume order), or 0: prm->p; mixed */
	                          /* orders as for p_max (linear advection on periodic meshes)                        */
};
struct dpg_ref_face {
	int volume[2];            /* neigh_info[side].volume->index (0-based); volume[1] = -1 on a boundary face      */
	int ind_lf[2];            /* neigh_info[side].ind_lf                                                         */
	int bc;                   /* Face::bc of a boundary face (a BC_* code, modulo BC_STEP_SC = 10000); else ignored */
};
int  dpg_sim_create_from_lists(const struct dpg_sim_params* prm, int n_vol, const struct dpg_ref_volume* vols,
                               int n_face, const struct dpg_ref_face* faces, struct dpg_sim** sim_out);
/* Same from a control file in the reference's key-value format (set_simulation_core, simulation.c:371-431; the
 * test_case.data / solution.data keys of test_case_T.c:258-302 may appear in the same file).  With mesh_path
 * (and mesh_format gmsh) the mesh is read from that file, relative to the control file's directory or else to the
 * working directory; without it, the structured box of mesh_elements / domain_lo / domain_hi. */
int  dpg_sim_create_from_ctrl(const char* ctrl_path, struct dpg_sim** sim_out);
void dpg_sim_destroy(struct dpg_sim* sim);

/* sizes: [d, n_var, n_vol, n_face, n_dof_doubles, n_s(group 0), n_c, n_fc, p, e_type] */
int  dpg_sim_info(const struct dpg_sim* sim, int64_t* info10);
int  dpg_sim_get_sol_coef(const struct dpg_sim* sim, double* out);
int  dpg_sim_set_sol_coef(struct dpg_sim* sim, const double* in);
int  dpg_sim_get_rhs(const struct dpg_sim* sim, double* out);
int  dpg_sim_set_time(struct dpg_sim* sim, double t);
/* L2 errors (SUMMATION_L2_VOL, compute_error.c:545-555) of rho,u,v,(w),p (Euler) or u (advection) at time t. */
int  dpg_sim_l2_error(const struct dpg_sim* sim, double t, double* err_out, int n_err_max);
/* max over solution nodes of |V| + c (Euler) or |b| (advection); used for the CFL time step. */
double dpg_sim_max_wave_speed(const struct dpg_sim* sim);
/* Restart files in the reference's format (output_restart_gmsh, restart_writers.c:126-145): a gmsh 2.2 mesh of the
 * volumes and the Bezier coefficients of sol_coef per volume ($SolutionCoefficients).  The reader sets sol_coef of
 * `sim` (any periodic QUAD/HEX mesh of the same domain, any order) by evaluating the file's expansion at the solution
 * nodes (set_sol_restart_T, restart_T.c:62-87).  A GPU state is written after dpg_gpu_download_sol_coef +
 * dpg_sim_set_sol_coef and read back with dpg_sim_get_sol_coef + dpg_gpu_upload_sol_coef. */
int  dpg_sim_write_restart(const struct dpg_sim* sim, const char* path);
/* The solution for visualisation, as the reference's output_visualization (visualization.c:73, the serial .vtu of
 * output_visualization_vtk_sol): a VTK XML UnstructuredGrid with one piece per volume -- equally spaced points of
 * the volume's order, linear sub-cells, point data index, p_ref and the solution (u; Euler / Navier-Stokes: rho,
 * velocity, pressure, and for Euler the absolute errors against the exact solution).  DPG_ERR_IO if the file cannot
 * be written.  A GPU state is written after dpg_gpu_download_sol_coef + dpg_sim_set_sol_coef. */
int  dpg_sim_write_vtk(const struct dpg_sim* sim, const char* path);
int  dpg_sim_read_restart(struct dpg_sim* sim, const char* path);
/* Pointer to the host data model (include/dpg_simulation.h) for the oracle and tests. */
const struct dpg_sim* dpg_sim_view(const struct dpg_sim* sim);

/* =====================================================================================================
 * GPU residual path
 * ===================================================================================================== */

/* Upload volumes, faces, operators and the current sol_coef of `sim` to device 0 and build the device tables.
 * Replaces the device-free reference sequence constructor_derived_Elements(IL_ELEMENT_SOLVER_DG) +
 * constructor_derived_computational_elements(IL_SOLVER_DG) (solve_explicit.c:88-89) as the point after which the
 * residual can be evaluated.  The context keeps no pointer into `sim`. */
int  dpg_gpu_create(const struct dpg_sim* sim, dpg_gpu_ctx** ctx_out);
void dpg_gpu_destroy(dpg_gpu_ctx* ctx);

/* Precision of the contractions: DPG_PREC_*; n_slices is used by DPG_PREC_BF16_SLICED (2..7). */
int  dpg_gpu_set_precision(dpg_gpu_ctx* ctx, int mode, int n_slices);

/* Positivity of density and pressure (Euler; on by default, as the reference's test_case_requires_positivity,
 * test_case.c:63-80): enforce_positivity_highorder (solve.c:187-233) after every RK stage and after each Newton update,
 * and the Newton update's per-volume under-relaxation compute_relaxation (solve_implicit.c:821-873).  Where the
 * reference stops (average density or pressure below EPS_PHYS, relaxation below EPS), the RK calls return
 * DPG_ERR_NONFINITE and the Newton solve undoes the step and halves the pseudo time step.  on = 1 for a PDE without
 * density and pressure: DPG_ERR_UNSUPPORTED. */
int  dpg_gpu_set_positivity(dpg_gpu_ctx* ctx, int on);
/* enforce_positivity_highorder on every volume of the context's state (what each RK stage runs); DPG_ERR_NONFINITE
 * where an average density or pressure is below EPS_PHYS (those volumes are left unchanged). */
int  dpg_gpu_enforce_positivity(dpg_gpu_ctx* ctx);
/* The Newton update of update_coef_s_v (solve_implicit.c:724-731): u += relax_v du per volume with compute_relaxation,
 * then the limiter; du is a host vector of n_dof.  DPG_ERR_NONFINITE where the relaxation falls below EPS (volume not
 * updated) or an average is below EPS_PHYS.  Positivity off: u += du. */
int  dpg_gpu_positivity_update(dpg_gpu_ctx* ctx, const double* du);

/* sol_coef host <-> device (all volumes, reference layout). */
int  dpg_gpu_upload_sol_coef  (dpg_gpu_ctx* ctx, const double* sol_coef);
int  dpg_gpu_download_sol_coef(dpg_gpu_ctx* ctx, double* sol_coef);
int  dpg_gpu_download_rhs     (dpg_gpu_ctx* ctx, double* rhs);

/* One DG residual with the semantics of compute_rhs_dg (dg/solve_dg.c:130-136): rhs := 0, volume term, face term,
 * source, rhs := m_inv * rhs; *max_rhs = ||rhs||_inf (compute_max_rhs_dg_like, compute_rlhs.c:59-71). */
int  dpg_gpu_compute_rhs(dpg_gpu_ctx* ctx, double* max_rhs);

/* n_steps SSP-RK3 steps of size dt with the stage formulas of time_step_ssp_rk_33 (solve_explicit.c:252-301).
 * *max_rhs receives the norm of the last stage's residual.  The stages are replayed from a CUDA graph. */
int  dpg_gpu_rk_step(dpg_gpu_ctx* ctx, double dt, int n_steps, double* max_rhs);

/* Whole explicit solve from the context's time to time_final (solve_explicit, solve_explicit.c:78-118), with the
 * final step shortened as in the reference.  Returns the number of steps taken in *n_steps_out. */
int  dpg_gpu_solve_explicit(dpg_gpu_ctx* ctx, double t0, double time_final, double dt, int* n_steps_out,
                            double* max_rhs);

/* ---- implicit path ---------------------------------------------------------------------------------------
 * Newton with pseudo-transient continuation for F(u) = m_inv * rhs(u) = 0, the linear systems
 * (I/dtau - dF/du) du = F solved by matrix-free GMRES(m).  Jacobian-vector products and element blocks come from
 * the analytic linearisation (forward-mode tangents of the FP64 residual formulas: the products of the reference's
 * df_ds / dnnf_ds Jacobians, compute_volume_rlhs_T.c:179-220, compute_face_rlhs_T.c:163-220) or, on request, from
 * finite differences of the residual kernels.  Replaces solve_implicit / implicit_step (solve_implicit.c:95-110, 232-256), whose PETSc
 * system is the same one left-scaled by the mass matrix (compute_CFL_ramping, dg/solve_dg.c:223-248); the exit
 * rule is the reference's ||F||_inf < tol (exit_tol_i). */
enum { DPG_PRECOND_NONE = 0, DPG_PRECOND_BLOCK_JACOBI = 1, DPG_PRECOND_MLP = 2, DPG_PRECOND_BLOCK_ILU = 3 };
/* Element order of the block ILU's factorisation: volume order (the reference's PETSc matrix rows follow the
 * volumes) or colour order (the elements of a face colouring one colour after another: as many levels as colours). */
enum { DPG_ILU_ORDER_VOLUME = 0, DPG_ILU_ORDER_COLOUR = 1 };
enum { DPG_JACOBIAN_TANGENT = 0, DPG_JACOBIAN_FD = 1 };
struct dpg_newton_params {
	double tol;            /* ||F||_inf target (1e-10)                                              */
	int max_newton;        /* Newton steps                                                          */
	int gmres_restart;     /* m of GMRES(m) (default 200: GMRES(30) stagnates on the periodic Euler systems) */
	int max_gmres;         /* Krylov iterations per Newton step                                     */
	double gmres_rtol;     /* relative Krylov tolerance                                             */
	double dtau0;          /* initial pseudo time step (grows as dtau0 * ||F_0|| / ||F_k||)          */
	double dtau_max;
	int precond;           /* DPG_PRECOND_*                                                         */
	int collect_blocks;    /* store (state, block inverse) samples for the learned preconditioner   */
	int verbose;
	const double* forcing; /* host [n_dof] or NULL: solve F(u) = forcing (with forcing = F(u*) the known  */
	                       /* state u* is the steady solution -- a manufactured steady problem)          */
	int jacobian;          /* DPG_JACOBIAN_TANGENT (default) or DPG_JACOBIAN_FD                       */
	int ilu_order;         /* DPG_ILU_ORDER_* of DPG_PRECOND_BLOCK_ILU (default volume order)         */
	int ilu_parts;         /* 0 or 1: one factorisation of the whole mesh; P > 1: P contiguous ranges of */
	                       /* the element order factorised independently (fewer, wider levels)          */
	double cfl_initial;    /* > 0: local pseudo time steps of the reference's CFL ramping (lhs_terms     */
	                       /* cfl_ramping, compute_dt_cfl_constrained, dg/solve_dg.c:284-318): per      */
	                       /* element dtau_e = cfl min(h_e / lambda_e, h_e^2 / mu), cfl = cfl_initial   */
	                       /* max(1, ||F_0|| / ||F_k||), h_e its shortest edge, lambda_e the largest    */
	                       /* |V| + c of its Bezier coefficients; 0 (default): one dtau for all, dtau0   */
	                       /* ||F_0|| / ||F_k|| (at most dtau_max)                                        */
};
struct dpg_newton_stats {
	int newton_iterations, gmres_iterations;
	double residual_initial, residual_final;
	double seconds, assembly_seconds;
	int rejected_steps;    /* Newton steps undone because they produced a non-finite state              */
	int fallback_steps;    /* learned-preconditioner steps redone with exact block-Jacobi                */
};
void dpg_newton_params_default(struct dpg_newton_params* prm);
/* jv = dF/du . v at the context's state u (F = m_inv * rhs; host vectors of n_dof): the analytic linearisation,
 * in FP64 whatever the residual's precision mode (test_integration_linearization checks the reference's Jacobians
 * against complex-step derivatives). */
int  dpg_gpu_jacobian_apply(dpg_gpu_ctx* ctx, const double* v, double* jv);
int  dpg_gpu_newton_solve(dpg_gpu_ctx* ctx, const struct dpg_newton_params* prm, struct dpg_newton_stats* stats);

/* Learned element-block preconditioner (no counterpart in the reference): an MLP maps an element's state and the
 * pseudo time step to an approximation of dtau^-1 (I/dtau - dF/du)_ee^-1.  It is trained on the blocks the
 * block-Jacobi solve assembles (collect_blocks = 1) with the library's own forward/backward kernels; GMRES still
 * decides convergence, so the network changes the iteration count, not the converged state. */
int  dpg_gpu_mlp_enable(dpg_gpu_ctx* ctx, int hidden, int capacity_samples, uint64_t seed);
/* A Newton step whose GMRES solve with the learned inverse misses 10x the Krylov tolerance is redone with exact
 * block-Jacobi (counted in dpg_newton_stats::fallback_steps). */
int  dpg_gpu_mlp_train(dpg_gpu_ctx* ctx, int epochs, int batch, double lr, double* loss_out);
int  dpg_gpu_mlp_samples(dpg_gpu_ctx* ctx);
/* Test hooks: parameter vector (get and/or set, n_params in *n) and loss + gradient of one batch given on host. */
int  dpg_gpu_mlp_params(dpg_gpu_ctx* ctx, float* get, const float* set, int64_t* n);
int  dpg_gpu_mlp_loss_grad(dpg_gpu_ctx* ctx, int batch, const float* x, const float* target, double* loss,
                           float* grad);
int  dpg_gpu_mlp_dims(dpg_gpu_ctx* ctx, int* d_in, int* hidden, int* d_out);
/* Test hook of the failure detection: the poll limit of the bounded mbarrier waits in the network's tensor-core GEMMs
 * (negative: the default, ~4 million polls).  With a tiny limit a wait gives up while its MMAs are still running; the
 * kernel then lets the issued MMAs finish before it frees its tensor memory, and the training / inference call returns
 * DPG_ERR_TIMEOUT with the context still usable.  Applies to every context of the process. */
int  dpg_gpu_mlp_set_wait_limit(dpg_gpu_ctx* ctx, long long polls);

/* Host-buffer convenience for a binding that does not keep device state between calls: copies sol_coef in,
 * runs n_steps RK steps and copies sol_coef out (all timed copies included). */
int  dpg_gpu_rk_step_host(dpg_gpu_ctx* ctx, double* sol_coef_inout, double dt, int n_steps, double* max_rhs);

/* Timing helper: average device time (ms) of each kernel of the last compute_rhs, measured with CUDA events on the
 * context stream.  names_out receives up to n_max entries "name" (static strings; NULL after the last).  With the
 * positivity limiter on, a fourth entry "positivity" times it on the current state -- which it corrects where
 * needed, as an RK stage would; the rhs is overwritten. */
int  dpg_gpu_kernel_times(dpg_gpu_ctx* ctx, int n_rep, double* ms_out, const char** names_out, int n_max);

/* Device time (ms, CUDA events on the context stream) of n_steps SSP-RK3 steps enqueued as by dpg_gpu_rk_step.
 * Measurement helper without a counterpart in the reference (which has no timing code). */
int  dpg_gpu_time_rk_steps(dpg_gpu_ctx* ctx, double dt, int n_steps, double* ms_out);

/* Number of kernels launched by one compute_rhs. */
int  dpg_gpu_launches_per_rhs(dpg_gpu_ctx* ctx);

/* ---- tile shapes of the split-precision kernels --------------------------------------------------------------
 * No counterpart in the reference (its contractions are per-element BLAS calls).  The block configuration of the
 * split-precision residual, valid while a split mode is set (dpg_gpu_set_precision resets it to the wave rule):
 *   elems_per_block     elements per block of the interpolation and lift kernels: the data rows of one tensor-core
 *                       tile are elems_per_block * n_var of its 128; one block per SM (default: the fewest whole
 *                       waves over the SMs, elements spread evenly);
 *   fp64_share_eighths  share of the interpolation kernel's volume-flux work items evaluated in FP64 on the FP64
 *                       pipe, in eighths, 0..8 (the rest in double-float arithmetic on the FP32 pipe; default 2);
 *   face_block_warps    warps per block of the face kernel: 1, 2, 4 or 8 (default 8).
 * Every configuration computes the same residual to within the rounding of the two flux arithmetics (which items
 * take which one depends on the elements per block and the share). */
struct dpg_tile_config {
	int elems_per_block;
	int fp64_share_eighths;
	int face_block_warps;
};
int  dpg_gpu_get_tiles(dpg_gpu_ctx* ctx, struct dpg_tile_config* out);
/* DPG_ERR_INVALID for a configuration outside the ranges above or with no split mode set. */
int  dpg_gpu_set_tiles(dpg_gpu_ctx* ctx, const struct dpg_tile_config* cfg);
/* Tile autotuner: times residual evaluations of the context's current state (CUDA events on the context stream,
 * the best of three batches of n_rep) over candidate configurations -- the elements per block of the wave rule with
 * 0, 1 and 2 extra waves and the largest that fits, then the FP64 share 0..4 eighths, then the face kernel's warps
 * per block 2, 4 and 8, each stage at the best of the previous ones; a candidate replaces the running best only
 * when it is faster by more than 1 % -- and keeps the fastest.  The result is cached for the process by (device,
 * element shape, variables, mesh size, precision mode); force = 1 measures again.  best (may be NULL) receives the
 * chosen configuration, best_ms (may be NULL) its time per residual.  Overwrites the rhs; the state is unchanged.
 * DPG_ERR_UNSUPPORTED in the FP64 form (no tunable tiles). */
int  dpg_gpu_autotune(dpg_gpu_ctx* ctx, int n_rep, int force, struct dpg_tile_config* best, double* best_ms);

/* ---- allocation-free residual ------------------------------------------------------------------------------
 * No counterpart in the reference.  For callers that may not allocate device memory at the time of the call --
 * code running under a memory manager that owns every device allocation, real-time loops where cudaMalloc's
 * implicit device synchronisation is not acceptable, or embedded solvers that provision all memory up front --
 * this entry point evaluates the FP64 residual (semantics of dpg_gpu_compute_rhs) with every input and output
 * supplied by the caller as device pointers, and keeps its intermediate face traces and face fluxes in a
 * fixed scratch array that the library declares statically: it calls no cudaMalloc, cudaFree or allocating
 * library routine.
 *   - Limit: 2 * n_face * n_var * n_fc + n_face * n_var * n_fc doubles must fit into DPG_NOALLOC_SCRATCH_DOUBLES
 *     (2,097,152 doubles = 16 MiB, held by every GPU that loads the library until process exit); larger problems
 *     return DPG_ERR_TOO_LARGE.
 *   - The first call on a device looks up the scratch address (cudaGetSymbolAddress): make that first call before
 *     any stream capture.  Every call sets the kernels' shared-memory limits for its sizes (no allocation).
 *   - All calls share the one scratch array: calls whose work overlaps on the GPU (different streams, or
 *     different threads without ordering) race.  Serialise them on one stream.
 *   - max_rhs (host pointer, may be NULL) receives ||rhs||_inf; when it is non-NULL the call synchronises the
 *     stream.  Operators and geometry have the layout dpg_gpu_create uploads (documented in the fields below). */
#define DPG_NOALLOC_SCRATCH_DOUBLES (1 << 21)
struct dpg_noalloc_mesh {
	int d, n_var, num_flux;                  /* 2|3; 4|5 (Euler) or 1 (advection); DPG_NUM_FLUX_*        */
	int n_vol, n_face, n_s, n_c, n_fl, n_fc;
	const double* cv0_vs_vc;                 /* [n_c x n_s] row-major                                      */
	const double* cv0_vs_fc;                 /* [n_fl*n_fc x n_s] local faces stacked                      */
	const double* lift;                      /* [n_s x (d*n_c + n_fl*n_fc)]: [tw1_vt_vc[0..d) | -tw0_vt_fc],  */
	                                         /* pre-multiplied by the reference m_inv when minv == NULL   */
	const double* metrics;                   /* minv == NULL: [n_vol][d*d] (m_ij at i + d*j); else [n_vol][d*d][n_c] */
	const double* jinv;                      /* [n_vol] 1/detJ (affine volumes; used when minv == NULL)     */
	const double* minv;                      /* [n_vol][n_s x n_s] or NULL                                 */
	const int* vol_face;                     /* [n_vol][n_fl] = (face << 1) | side                         */
	const int* nc_fc;                        /* [n_face][n_fc] right-side node of each left node            */
	const int* nc_fc_inv;                    /* [n_face][n_fc] inverse permutation                         */
	const double* normals_fc;                /* [n_face][n_fc][d] unit normals of side 0                   */
	const double* jacobian_det_fc;           /* [n_face][n_fc]                                             */
	double b_adv[3];                         /* advection velocity                                         */
};
int  dpg_gpu_compute_rhs_noalloc(const struct dpg_noalloc_mesh* mesh, const double* sol_coef, double* rhs,
                                 double* max_rhs, void* cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* DPG_GB300_H */
