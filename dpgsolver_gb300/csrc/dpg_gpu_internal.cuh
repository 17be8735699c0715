// Device context and kernel launch declarations shared by the CUDA translation units.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "dpg_gb300.h"
#include "dpg_simulation.h"

namespace dpg {

constexpr int kMaxStages = 3;

// Per-group device tables (one group = one (element type, order); the structured meshes of this path have one).
struct GroupDev {
	int n_vol, n_s, n_c, n_fl, n_fc, K;    // K = d*n_c + n_fl*n_fc (lift contraction length)
	const double* Cv;      // [n_c  x n_s]        cv0_vs_vc
	const double* Cf;      // [n_fl*n_fc x n_s]   cv0_vs_fc stacked over local faces
	const double* L;       // [n_s  x K]          [tw1_vt_vc[0..d) | -tw0_vt_fc[0..n_fl)], pre-multiplied by
	                       //                     m_inv_ref when every volume is affine
	const double* met;     // affine: [n_vol][d*d] (m_ij at i + d*j); else [n_vol][d*d][n_c]
	const double* jinv;    // [n_vol] 1/detJ (affine)
	const double* minv;    // [n_vol][n_s*n_s] (non-affine) or nullptr
	const int* vol_face;   // [n_vol][n_fl]  (face << 1) | side
	const int* nc_inv;     // [n_face][n_fc] inverse of nc_fc
	int affine;
};

struct FaceDev {
	int n_face, n_fc;
	const double* nrm;     // [n_face][n_fc][d]
	const double* jf;      // [n_face][n_fc]
	const int* nc;         // [n_face][n_fc]
};

} // namespace dpg

struct dpg_gpu_ctx {
	int dev = 0;
	cudaStream_t stream = nullptr;
	int d = 0, n_var = 0, n_eq = 0, pde = 0, num_flux = 0;
	int e_type = 0;             // element type of the (single) group (DPG_QUAD, DPG_HEX, DPG_TRI)
	double b_adv[3] = {0, 0, 0};
	int64_t n_dof = 0;

	dpg::GroupDev g{};
	dpg::FaceDev fc{};

	// state
	double* sol = nullptr;
	double* solp = nullptr;
	double* rhs = nullptr;
	double* trace = nullptr;    // [n_face][2][n_var][n_fc], each side in its own node order
	double* nnf = nullptr;      // [n_face][n_eq][n_fc], left node order, scaled by jacobian_det_fc
	unsigned long long* dmax = nullptr;   // [kMaxStages+1] max |rhs| bit patterns
	double* ddt = nullptr;      // device copy of dt (graph parameter)

	// owned device allocations (freed at destroy)
	void* allocs[32] = {};
	int n_allocs = 0;

	// precision
	int prec_mode = DPG_PREC_FP64;
	int n_slices = 0;
	void* split = nullptr;      // split-precision state (split_ops.cu)

	// CUDA graph of one SSP-RK3 step
	cudaGraphExec_t step_graph = nullptr;
	int step_graph_mode = -1;

	int vol_block_elems = 1;
	int trace_block_elems = 1;
	int tan_block_elems = 1;     // elements per block of the linearisation's volume kernel
	double* trace_t = nullptr;   // tangent of the traces (allocated on the first Jacobian-vector product)
	double* nnf_t = nullptr;     // tangent of the face fluxes

	// positivity of density and pressure (Euler): limiter after every RK stage and Newton update (positivity.cu)
	int positivity = 0;          // on by default for Euler, as the reference's test_case_requires_positivity
	int pos_n1 = 0;              // solution points per direction
	double* bez1 = nullptr;      // [n1 x n1] Bernstein polynomials at the GLL nodes (Bezier -> solution coefficients)
	double* bez1_inv = nullptr;  // [n1 x n1] its inverse
	int pos_dense = 0;           // simplices: dense Bezier operators (no 1D factors), n_s solution nodes
	double* bez_bs = nullptr;    // [n_s x n_s] Bezier -> solution coefficients (ccBS0_vs_vs), dense limiter
	float* bez_sb32 = nullptr;   // [n_s x n_s] ccSB0_vs_vs in FP32 (the dense limiter's screen)
	// mixed orders (Euler): the dense limiter per order group -- its volumes, operators and screen bound
	struct PosGroup { int n_vol = 0, ns = 0; const int* vols = nullptr; const float* sb32 = nullptr;
	                  const double* sb64 = nullptr; const double* bs64 = nullptr; float amp = 0.f; };
	PosGroup pos_grp[DPG_P_MAX];
	int n_pos_grp = 0;
	const int64_t* pos_dof_off = nullptr;   // [n_vol + 1]
	// local pseudo time steps of the implicit solve (the reference's CFL ramping)
	double* h_min = nullptr;     // [n_vol] shortest edge of each volume (chord between its end vertices)
	double* bez_full = nullptr;  // [n_s x n_s] solution -> Bezier coefficients (ccSB0_vs_vs), Euler-like PDEs
	double visc_mu = 0.0;        // constant viscosity (Navier-Stokes), 0 without second-order terms
	double adv_speed = 0.0;      // |b_adv| (advection)
	double bez1_host[50] = {};   // host copies: bez1 at [0, n1^2), bez1_inv at [25, 25 + n1^2) (kernel parameters)
	float pos_amp = 0.f;         // FP32 screen: bound of the coefficient error per unit of |A^-1| |u|
	int* pos_err = nullptr;      // bit 0: an average density / pressure below EPS_PHYS; bit 1: relaxation underflow
	double* du_buf = nullptr;    // [n_dof] device copy of a host Newton update (dpg_gpu_positivity_update)

	void* general = nullptr;    // boundary faces / Navier-Stokes: the general FP64 chain (kernels_ns.cu)
	void* hp = nullptr;         // mixed orders: volumes grouped by order (kernels_hp.cu)
	void* implicit = nullptr;   // Newton-GMRES work space (implicit.cu)
	void* mlp = nullptr;        // learned preconditioner (mlp.cu)
};

namespace dpg {
int launch_trace (dpg_gpu_ctx* c);
int launch_face  (dpg_gpu_ctx* c);
int launch_volume(dpg_gpu_ctx* c, int stage, bool write_rhs, unsigned long long* max_slot);
// J v = d(m_inv rhs)/du . v at u (FP64 formulas, forward-mode tangents); trace_t, nnf_t: work buffers of the sizes
// of the traces and face fluxes.
int jvp_fp64(dpg_gpu_ctx* c, const double* u, const double* v, double* out, double* trace_t, double* nnf_t);
int ensure_tangent_buffers(dpg_gpu_ctx* c);

// general FP64 chain (kernels_ns.cu): boundary faces and the BR2 Navier-Stokes terms, residual and exact
// Jacobian-vector products (forward-mode tangents through the same templated kernels)
int  gen_prepare(dpg_gpu_ctx* c, const struct dpg_sim* sim);
int  gen_residual(dpg_gpu_ctx* c, int stage, bool write_rhs, unsigned long long* max_slot);
int  gen_jvp(dpg_gpu_ctx* c, const double* u, const double* v, double* out);
int  gen_launches_per_rhs(dpg_gpu_ctx* c);
void gen_free(dpg_gpu_ctx* c);

// mixed orders (kernels_hp.cu): FP64 residual over volume groups of each order; which = 0 traces, 1 face fluxes,
// 2 volume terms (with the RK stage)
int  hp_prepare(dpg_gpu_ctx* c, const struct dpg_sim* sim);
int  hp_residual(dpg_gpu_ctx* c, int stage, bool write_rhs, unsigned long long* max_slot);
int  hp_launch_part(dpg_gpu_ctx* c, int which, int stage, bool write_rhs, unsigned long long* max_slot);
void hp_free(dpg_gpu_ctx* c);

// split-precision path (split_ops.cu)
int  split_prepare(dpg_gpu_ctx* c);
void split_free(dpg_gpu_ctx* c);
int  split_launch_trace (dpg_gpu_ctx* c);   // interpolation kernel (traces + volume fluxes)
int  split_launch_face  (dpg_gpu_ctx* c);
int  split_launch_volume(dpg_gpu_ctx* c, int stage, bool write_rhs, unsigned long long* max_slot);
int  split_error(dpg_gpu_ctx* c);   // non-zero when a bounded device wait gave up
using TileConfig = dpg_tile_config;
int  split_get_tiles(dpg_gpu_ctx* c, TileConfig* t);
int  split_set_tiles(dpg_gpu_ctx* c, const TileConfig& t);   // validated; the caller drops the captured step graph
// elements per block of the wave rule: the fewest whole waves of blocks over n_sm SMs (plus extra_waves), elements
// spread evenly, at most 128 / NV data rows
int  wave_rule_eb(int n_vol, int NV, int n_sm, int extra_waves);
void invalidate_step_graph(dpg_gpu_ctx* c);

// residual of the context's precision mode from c->sol into c->rhs (no synchronisation)
int  enqueue_residual_raw(dpg_gpu_ctx* c, unsigned long long* max_slot);

// positivity (positivity.cu): the limiter on a state (no-op when c->positivity is 0) and the Newton update
// u += relax du with the per-volume under-relaxation (positivity on only); errors in c->pos_err
int  launch_positivity(dpg_gpu_ctx* c, double* sol);
int  launch_relaxed_update(dpg_gpu_ctx* c, double* u, const double* du);
int  positivity_error(dpg_gpu_ctx* c);   // reads and clears c->pos_err
int  launch_axpy(dpg_gpu_ctx* c, int64_t n, double a, const double* x, double* y);   // y += a x

// implicit path (implicit.cu) and learned preconditioner (mlp.cu)
int  implicit_solve(dpg_gpu_ctx* c, const dpg_newton_params* prm, dpg_newton_stats* st);
void implicit_free(dpg_gpu_ctx* c);
int  mlp_collect(dpg_gpu_ctx* c, const double* u, const double* lu, const int* piv, const double* shift, double rho);
double mlp_rho(dpg_gpu_ctx* c);
int  mlp_predict(dpg_gpu_ctx* c, const double* u, const double* shift, float** P);
void mlp_free(dpg_gpu_ctx* c);
} // namespace dpg
