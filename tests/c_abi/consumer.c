/* A plain C99 caller of the library through include/dpg_gb300.h only, as the reference's C code would bind it:
 * host set-up, L2 error, restart round trip, a mixed-order triangle mesh with its visualisation output, and -- where
 * a CUDA device is present, or required by a second argument -- one residual evaluation and one SSP-RK3 step, and
 * the mixed-order residual.  Prints "ok" and exits 0 when every call behaves as documented. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "dpg_gb300.h"

#define CHECK(cond, what) do { if (!(cond)) { printf("FAIL %s\n", what); return 1; } } while (0)

int main(int argc, char** argv)
{
	CHECK(argc == 2 || argc == 3, "usage: consumer <restart path> [device]");
	const int need_device = (argc == 3);
	struct dpg_sim_params prm;
	dpg_sim_params_default(&prm);
	prm.d = 2; prm.e_type = DPG_QUAD; prm.p = 2;
	prm.n_elem[0] = 4; prm.n_elem[1] = 4; prm.n_elem[2] = 1;
	struct dpg_sim* sim = NULL;
	CHECK(dpg_sim_create(&prm, &sim) == DPG_OK && sim, "dpg_sim_create");

	int64_t info[10];
	CHECK(dpg_sim_info(sim, info) == DPG_OK, "dpg_sim_info");
	CHECK(info[0] == 2 && info[1] == 4 && info[2] == 16 && info[5] == 9, "sizes");
	const int64_t n_dof = info[4];

	double err[5];
	CHECK(dpg_sim_l2_error(sim, 0.0, err, 5) == DPG_OK, "dpg_sim_l2_error");
	CHECK(err[0] >= 0.0 && err[0] < 0.1, "initial interpolation error");

	double* u = malloc(sizeof(double) * (size_t)n_dof);
	double* v = malloc(sizeof(double) * (size_t)n_dof);
	CHECK(u && v, "malloc");
	CHECK(dpg_sim_get_sol_coef(sim, u) == DPG_OK, "dpg_sim_get_sol_coef");
	CHECK(dpg_sim_write_restart(sim, argv[1]) == DPG_OK, "dpg_sim_write_restart");
	CHECK(dpg_sim_read_restart(sim, argv[1]) == DPG_OK, "dpg_sim_read_restart");
	CHECK(dpg_sim_get_sol_coef(sim, v) == DPG_OK, "dpg_sim_get_sol_coef");
	for (int64_t i = 0; i < n_dof; ++i) CHECK(fabs(u[i] - v[i]) <= 1e-13 * (1.0 + fabs(u[i])), "restart round trip");

	dpg_gpu_ctx* ctx = NULL;
	const int rc = dpg_gpu_create(dpg_sim_view(sim), &ctx);
	if (rc == DPG_OK) {
		double max_rhs = 0.0;
		CHECK(dpg_gpu_compute_rhs(ctx, &max_rhs) == DPG_OK && max_rhs > 0.0, "dpg_gpu_compute_rhs");
		CHECK(dpg_gpu_rk_step(ctx, 1e-3, 1, &max_rhs) == DPG_OK, "dpg_gpu_rk_step");
		CHECK(dpg_gpu_download_sol_coef(ctx, v) == DPG_OK, "dpg_gpu_download_sol_coef");
		dpg_gpu_destroy(ctx);
	} else {
		CHECK(!need_device && rc == DPG_ERR_NO_DEVICE, "dpg_gpu_create without a device");
	}
	CHECK(dpg_status_string(DPG_ERR_UNSUPPORTED) != NULL, "dpg_status_string");
	free(u); free(v);
	dpg_sim_destroy(sim);

	/* a triangle mesh of mixed orders 1..4 (linear advection): set-up, visualisation output, residual */
	dpg_sim_params_default(&prm);
	prm.d = 2; prm.e_type = DPG_TRI; prm.p = 1; prm.p_max = 4; prm.p_seed = 5;
	prm.n_elem[0] = 5; prm.n_elem[1] = 4; prm.n_elem[2] = 1;
	prm.lo[0] = prm.lo[1] = 0.0; prm.hi[0] = prm.hi[1] = 1.0;
	prm.pde_index = DPG_PDE_ADVECTION; prm.num_flux = DPG_NUM_FLUX_UPWIND; prm.test_case = DPG_TC_ADVECTION_SINE;
	CHECK(dpg_sim_create(&prm, &sim) == DPG_OK && sim, "dpg_sim_create (mixed orders)");
	const struct dpg_sim* view = dpg_sim_view(sim);
	CHECK(view->n_vol == 40 && view->n_ops == 4 && view->face_p != NULL, "mixed-order data model");
	for (int f = 0; f < view->n_face; ++f) {
		const int pl = view->vol_p[view->face_vol[2*f]], pr = view->vol_p[view->face_vol[2*f+1]];
		CHECK(dpg_face_order(view, f) == (pl > pr ? pl : pr), "face order");
	}
	CHECK(dpg_sim_write_vtk(sim, argv[1]) == DPG_OK, "dpg_sim_write_vtk");
	const int rc2 = dpg_gpu_create(view, &ctx);
	if (rc2 == DPG_OK) {
		double max_rhs = 0.0;
		CHECK(dpg_gpu_compute_rhs(ctx, &max_rhs) == DPG_OK && max_rhs > 0.0, "dpg_gpu_compute_rhs (mixed orders)");
		CHECK(dpg_gpu_set_precision(ctx, DPG_PREC_BF16_SLICED, 7) == DPG_ERR_UNSUPPORTED, "split on mixed orders");
		dpg_gpu_destroy(ctx);
	} else {
		CHECK(!need_device && rc2 == DPG_ERR_NO_DEVICE, "dpg_gpu_create without a device (mixed orders)");
	}
	dpg_sim_destroy(sim);
	printf("ok\n");
	return 0;
}
