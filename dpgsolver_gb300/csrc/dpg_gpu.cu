// C ABI of the GPU residual path (declared in include/dpg_gb300.h).
//
// dpg_gpu_create uploads one simulation: state in the reference's per-volume [n_s, n_var] column-major layout
// (volumes contiguous, so a residual streams element blocks linearly), FP64 operators, per-element metric terms
// (one d x d block per affine element), per-face normals / surface Jacobians / node correspondence, and the
// element -> face table used by the deterministic gather.  Every call returns a status and never aborts.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "dpg_gpu_internal.cuh"

namespace dpg {
int fp64_configure(dpg_gpu_ctx* c);
}

#define CK(call)                                                                                            \
	do {                                                                                                    \
		cudaError_t err_ = (call);                                                                          \
		if (err_ != cudaSuccess) {                                                                          \
			fprintf(stderr, "dpg_gb300: %s failed: %s (%s:%d)\n", #call, cudaGetErrorString(err_), __FILE__, \
			        __LINE__);                                                                              \
			return DPG_ERR_CUDA;                                                                            \
		}                                                                                                   \
	} while (0)

template <typename T>
static int dalloc(dpg_gpu_ctx* c, T** p, size_t n)
{
	if (c->n_allocs >= (int)(sizeof c->allocs / sizeof c->allocs[0])) return DPG_ERR_INVALID;
	void* q = nullptr;
	CK(cudaMalloc(&q, (n ? n : 1) * sizeof(T)));
	c->allocs[c->n_allocs++] = q;
	*p = (T*)q;
	return DPG_OK;
}

template <typename T>
static int dupload(dpg_gpu_ctx* c, T** p, const T* host, size_t n)
{
	int rc = dalloc(c, p, n);
	if (rc) return rc;
	if (n) CK(cudaMemcpy(*p, host, n * sizeof(T), cudaMemcpyHostToDevice));
	return DPG_OK;
}

// Mixed orders: state, the per-order volume groups and the face tables of kernels_hp.cu (periodic meshes, FP64
// residual and explicit steps).
static int create_mixed_orders(const struct dpg_sim* sim, dpg_gpu_ctx** ctx_out)
{
	const int d = sim->d, nv = sim->n_var;
	if (!((d == 2 && nv == 4) || (d == 3 && nv == 5) || nv == 1)) return DPG_ERR_UNSUPPORTED;
	for (int f = 0; f < sim->n_face; ++f)
		if (sim->face_vol[2 * f + 1] < 0) return DPG_ERR_UNSUPPORTED;
	if (sim->pde_index == DPG_PDE_NAVIER_STOKES || sim->geom != DPG_GEOM_STRAIGHT) return DPG_ERR_UNSUPPORTED;
	dpg_gpu_ctx* c = new dpg_gpu_ctx();
	int rc = DPG_OK;
	auto fail = [&](int code) { dpg_gpu_destroy(c); return code; };
	if (cudaSetDevice(0) != cudaSuccess) return fail(DPG_ERR_CUDA);
	if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(DPG_ERR_CUDA);
	c->d = d; c->n_var = nv; c->n_eq = sim->n_eq; c->pde = sim->pde_index; c->num_flux = sim->ind_num_flux[0];
	c->e_type = sim->ops[0].e_type;
	for (int a = 0; a < 3; ++a) c->b_adv[a] = sim->b_adv[a];
	c->n_dof = sim->vol_dof_off[sim->n_vol];
	if ((rc = dupload(c, &c->sol, sim->sol_coef, (size_t)c->n_dof))) return fail(rc);
	if ((rc = dalloc(c, &c->solp, (size_t)c->n_dof))) return fail(rc);
	if ((rc = dalloc(c, &c->rhs, (size_t)c->n_dof))) return fail(rc);
	if ((rc = dalloc(c, &c->dmax, dpg::kMaxStages + 1))) return fail(rc);
	if ((rc = dalloc(c, &c->ddt, 1))) return fail(rc);
	if (cudaMemset(c->rhs, 0, sizeof(double) * c->n_dof) != cudaSuccess) return fail(DPG_ERR_CUDA);
	if ((rc = dpg::hp_prepare(c, sim))) return fail(rc);
	// Euler: the dense positivity limiter per order group (Bezier operators of each order, n_s <= 64)
	if (sim->pde_index == DPG_PDE_EULER && nv == d + 2) {
		std::vector<std::vector<int>> members(sim->n_ops);
		for (int v = 0; v < sim->n_vol; ++v) members[sim->vol_ops[v]].push_back(v);
		for (int k = 0; k < sim->n_ops; ++k) {
			const dpg_element_ops& o = sim->ops[k];
			if (members[k].empty()) continue;
			if (o.n_s > 64 || !o.ccSB0_vs_vs || !o.ccBS0_vs_vs || c->n_pos_grp >= DPG_P_MAX) return fail(DPG_ERR_UNSUPPORTED);
			dpg_gpu_ctx::PosGroup& g = c->pos_grp[c->n_pos_grp++];
			g.n_vol = (int)members[k].size();
			g.ns = o.n_s;
			g.amp = (float)(4.0 * (o.n_s + 5) * std::ldexp(1.0, -24));
			std::vector<float> sb32((size_t)o.n_s * o.n_s);
			for (size_t i = 0; i < sb32.size(); ++i) sb32[i] = (float)o.ccSB0_vs_vs[i];
			int* dv; float* d32; double* d64; double* dbs;
			if ((rc = dupload(c, &dv, members[k].data(), members[k].size()))) return fail(rc);
			if ((rc = dupload(c, &d32, sb32.data(), sb32.size()))) return fail(rc);
			if ((rc = dupload(c, &d64, o.ccSB0_vs_vs, sb32.size()))) return fail(rc);
			if ((rc = dupload(c, &dbs, o.ccBS0_vs_vs, sb32.size()))) return fail(rc);
			g.vols = dv; g.sb32 = d32; g.sb64 = d64; g.bs64 = dbs;
		}
		int64_t* doff;
		if ((rc = dupload(c, &doff, sim->vol_dof_off, (size_t)sim->n_vol + 1))) return fail(rc);
		c->pos_dof_off = doff;
		if ((rc = dalloc(c, &c->pos_err, 1))) return fail(rc);
		if (cudaMemset(c->pos_err, 0, sizeof(int)) != cudaSuccess) return fail(DPG_ERR_CUDA);
		c->pos_dense = 1;
		c->positivity = 1;
	}
	if (cudaDeviceSynchronize() != cudaSuccess) return fail(DPG_ERR_CUDA);
	*ctx_out = c;
	return DPG_OK;
}

extern "C" int dpg_gpu_create(const struct dpg_sim* sim, dpg_gpu_ctx** ctx_out)
{
	if (!sim || !ctx_out) return DPG_ERR_INVALID;
	*ctx_out = nullptr;
	int n_dev = 0;
	if (cudaGetDeviceCount(&n_dev) != cudaSuccess || n_dev < 1) return DPG_ERR_NO_DEVICE;
	if (sim->n_ops != 1) return create_mixed_orders(sim, ctx_out);
	const dpg_element_ops& ops = sim->ops[0];
	const int d = sim->d, nv = sim->n_var, n_s = ops.n_s, n_c = ops.n_c, n_fl = ops.n_fl, n_fc = ops.n_fc;
	if (!((d == 2 && nv == 4) || (d == 3 && nv == 5) || nv == 1)) return DPG_ERR_UNSUPPORTED;

	dpg_gpu_ctx* c = new dpg_gpu_ctx();
	int rc = DPG_OK;
	auto fail = [&](int code) { dpg_gpu_destroy(c); return code; };
	if (cudaSetDevice(0) != cudaSuccess) return fail(DPG_ERR_CUDA);
	if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(DPG_ERR_CUDA);
	c->d = d; c->n_var = nv; c->n_eq = sim->n_eq; c->pde = sim->pde_index; c->num_flux = sim->ind_num_flux[0];
	c->e_type = ops.e_type;
	for (int a = 0; a < 3; ++a) c->b_adv[a] = sim->b_adv[a];
	const int n_vol = sim->n_vol, n_face = sim->n_face;
	c->n_dof = sim->vol_dof_off[n_vol];

	int affine_all = 1;
	for (int v = 0; v < n_vol; ++v) affine_all &= sim->vol_affine[v];

	dpg::GroupDev& g = c->g;
	g.n_vol = n_vol; g.n_s = n_s; g.n_c = n_c; g.n_fl = n_fl; g.n_fc = n_fc; g.K = d * n_c + n_fl * n_fc;
	g.affine = affine_all;
	const int K = g.K;

	// operators: Cv, Cf, L = [tw1 | -tw0] (times m_inv_ref when every volume is affine)
	std::vector<double> L((size_t)n_s * K), Lm((size_t)n_s * K);
	for (int i = 0; i < n_s; ++i) {
		for (int r = 0; r < d; ++r)
			for (int cc = 0; cc < n_c; ++cc)
				L[(size_t)i * K + r * n_c + cc] = ops.tw1_vt_vc[((size_t)r * n_s + i) * n_c + cc];
		for (int lf = 0; lf < n_fl; ++lf)
			for (int q = 0; q < n_fc; ++q)
				L[(size_t)i * K + d * n_c + lf * n_fc + q] = -ops.tw0_vt_fc[((size_t)lf * n_s + i) * n_fc + q];
	}
	if (affine_all) {
		for (int i = 0; i < n_s; ++i)
			for (int k = 0; k < K; ++k) {
				double s = 0.0;
				for (int j = 0; j < n_s; ++j) s += ops.m_inv_ref[(size_t)i * n_s + j] * L[(size_t)j * K + k];
				Lm[(size_t)i * K + k] = s;
			}
	} else {
		Lm = L;
	}
	if ((rc = dupload(c, (double**)&g.Cv, ops.cv0_vs_vc, (size_t)n_c * n_s))) return fail(rc);
	if ((rc = dupload(c, (double**)&g.Cf, ops.cv0_vs_fc, (size_t)n_fl * n_fc * n_s))) return fail(rc);
	if ((rc = dupload(c, (double**)&g.L, Lm.data(), Lm.size()))) return fail(rc);

	// geometry
	if (affine_all) {
		std::vector<double> met((size_t)n_vol * d * d), jinv(n_vol);
		for (int v = 0; v < n_vol; ++v) {
			const double* m = &sim->metrics_vc[(size_t)sim->vol_geo_off[v] * d * d];
			for (int k = 0; k < d * d; ++k) met[(size_t)v * d * d + k] = m[(size_t)n_c * k];
			jinv[v] = 1.0 / sim->jacobian_det_vc[sim->vol_geo_off[v]];
		}
		if ((rc = dupload(c, (double**)&g.met, met.data(), met.size()))) return fail(rc);
		if ((rc = dupload(c, (double**)&g.jinv, jinv.data(), jinv.size()))) return fail(rc);
		g.minv = nullptr;
	} else {
		// per node metrics [v][k][c] (the host layout is already c fastest within k)
		if ((rc = dupload(c, (double**)&g.met, sim->metrics_vc, (size_t)n_vol * n_c * d * d))) return fail(rc);
		std::vector<double> minv((size_t)n_vol * n_s * n_s);
		for (int v = 0; v < n_vol; ++v) {
			double* dst = &minv[(size_t)v * n_s * n_s];
			if (sim->vol_minv_off[v + 1] > sim->vol_minv_off[v]) {
				memcpy(dst, &sim->m_inv[sim->vol_minv_off[v]], sizeof(double) * n_s * n_s);
			} else {
				const double jd = sim->jacobian_det_vc[sim->vol_geo_off[v]];
				for (int k = 0; k < n_s * n_s; ++k) dst[k] = ops.m_inv_ref[k] / jd;
			}
		}
		if ((rc = dupload(c, (double**)&g.minv, minv.data(), minv.size()))) return fail(rc);
		g.jinv = nullptr;
	}
	std::vector<int> vf((size_t)n_vol * n_fl);
	for (int v = 0; v < n_vol; ++v)
		for (int lf = 0; lf < n_fl; ++lf)
			vf[(size_t)v * n_fl + lf] = (sim->vol_face[v * DPG_NFL_MAX + lf] << 1) | sim->vol_face_side[v * DPG_NFL_MAX + lf];
	if ((rc = dupload(c, (int**)&g.vol_face, vf.data(), vf.size()))) return fail(rc);
	std::vector<int> ncinv((size_t)n_face * n_fc);
	for (int f = 0; f < n_face; ++f)
		for (int q = 0; q < n_fc; ++q) ncinv[(size_t)f * n_fc + sim->nc_fc[(size_t)f * n_fc + q]] = q;
	if ((rc = dupload(c, (int**)&g.nc_inv, ncinv.data(), ncinv.size()))) return fail(rc);

	dpg::FaceDev& fd = c->fc;
	fd.n_face = n_face; fd.n_fc = n_fc;
	if ((rc = dupload(c, (double**)&fd.nrm, sim->normals_fc, (size_t)n_face * n_fc * d))) return fail(rc);
	if ((rc = dupload(c, (double**)&fd.jf, sim->jacobian_det_fc, (size_t)n_face * n_fc))) return fail(rc);
	if ((rc = dupload(c, (int**)&fd.nc, sim->nc_fc, (size_t)n_face * n_fc))) return fail(rc);

	// state
	if ((rc = dupload(c, &c->sol, sim->sol_coef, (size_t)c->n_dof))) return fail(rc);
	if ((rc = dalloc(c, &c->solp, (size_t)c->n_dof))) return fail(rc);
	if ((rc = dalloc(c, &c->rhs, (size_t)c->n_dof))) return fail(rc);
	if ((rc = dalloc(c, &c->trace, (size_t)n_face * 2 * nv * n_fc))) return fail(rc);
	if ((rc = dalloc(c, &c->nnf, (size_t)n_face * nv * n_fc))) return fail(rc);
	if ((rc = dalloc(c, &c->dmax, dpg::kMaxStages + 1))) return fail(rc);
	if ((rc = dalloc(c, &c->ddt, 1))) return fail(rc);
	if (cudaMemset(c->rhs, 0, sizeof(double) * c->n_dof) != cudaSuccess) return fail(DPG_ERR_CUDA);
	// positivity limiter (Euler): 1D Bezier operators and the FP32 screen's error bound per unit of |A^-1| |u|,
	// 4 (D (n1 + 2) + 2) 2^-24 (input truncation, operator rounding and n1-term sums in each of the D passes)
	const bool simplex_e = (ops.e_type == DPG_TRI || ops.e_type == DPG_TET);
	if ((sim->pde_index == DPG_PDE_EULER || sim->pde_index == DPG_PDE_NAVIER_STOKES) && nv == d + 2 && simplex_e) {
		// simplices: dense operators; the FP32 screen's bound (n_s + 5) 2^-24 per unit of |ccSB0| |u| (truncation of u,
		// rounding of the operator, n_s-term sums), with a factor 4 of margin
		if (n_s > 64) return fail(DPG_ERR_UNSUPPORTED);
		c->pos_dense = 1;
		c->pos_amp = (float)(4.0 * (n_s + 5) * std::ldexp(1.0, -24));
		std::vector<float> sb32((size_t)n_s * n_s);
		for (size_t i = 0; i < sb32.size(); ++i) sb32[i] = (float)ops.ccSB0_vs_vs[i];
		if ((rc = dupload(c, &c->bez_bs, ops.ccBS0_vs_vs, (size_t)n_s * n_s))) return fail(rc);
		if ((rc = dalloc(c, &c->bez_sb32, (size_t)n_s * n_s))) return fail(rc);
		if (cudaMemcpy(c->bez_sb32, sb32.data(), sizeof(float) * sb32.size(), cudaMemcpyHostToDevice) != cudaSuccess)
			return fail(DPG_ERR_CUDA);
		if ((rc = dalloc(c, &c->pos_err, 1))) return fail(rc);
		if (cudaMemset(c->pos_err, 0, sizeof(int)) != cudaSuccess) return fail(DPG_ERR_CUDA);
		c->positivity = 1;
	} else if ((sim->pde_index == DPG_PDE_EULER || sim->pde_index == DPG_PDE_NAVIER_STOKES) && nv == d + 2) {
		const int n1 = ops.p + 1;
		c->pos_n1 = n1;
		c->pos_amp = (float)(4.0 * (d * (n1 + 2) + 2) * std::ldexp(1.0, -24));
		for (int i = 0; i < n1 * n1; ++i) { c->bez1_host[i] = ops.bez1[i]; c->bez1_host[25 + i] = ops.bez1_inv[i]; }
		if ((rc = dupload(c, &c->bez1, ops.bez1, (size_t)n1 * n1))) return fail(rc);
		if ((rc = dupload(c, &c->bez1_inv, ops.bez1_inv, (size_t)n1 * n1))) return fail(rc);
		if ((rc = dalloc(c, &c->pos_err, 1))) return fail(rc);
		if (cudaMemset(c->pos_err, 0, sizeof(int)) != cudaSuccess) return fail(DPG_ERR_CUDA);
		c->positivity = 1;
	}
	// shortest edge per volume (compute_min_length_measure, dg/solve_dg.c:322-366: the chord between the two end
	// vertices of each edge), the Bezier operator and the viscosity of the local pseudo time steps
	{
		const int n_ve = ops.n_ve;
		const bool simplex = (ops.e_type == DPG_TRI || ops.e_type == DPG_TET);   // every vertex pair is an edge
		std::vector<double> h(n_vol);
		for (int v = 0; v < n_vol; ++v) {
			double x[8][3];
			for (int k = 0; k < n_ve; ++k) {
				const double* xv = &sim->xyz_ve[((size_t)v * DPG_NVE_MAX + k) * 3];
				if (sim->geom == DPG_GEOM_CYLINDER) { x[k][0] = xv[0] * std::cos(xv[1]); x[k][1] = xv[0] * std::sin(xv[1]); x[k][2] = 0.0; }
				else { x[k][0] = xv[0]; x[k][1] = xv[1]; x[k][2] = xv[2]; }
			}
			double hm = 1e300;
			for (int k = 0; k < n_ve; ++k)
				for (int o = k + 1; o < n_ve; ++o) {
					// tensor-product volumes: the vertices that differ in one reference coordinate bit
					if (!simplex && __builtin_popcount((unsigned)(k ^ o)) != 1) continue;
					double l2 = 0.0;
					for (int i = 0; i < d; ++i) l2 += (x[o][i] - x[k][i]) * (x[o][i] - x[k][i]);
					hm = std::min(hm, std::sqrt(l2));
				}
			h[v] = hm;
		}
		if ((rc = dupload(c, &c->h_min, h.data(), h.size()))) return fail(rc);
		if (nv == d + 2 && ops.ccSB0_vs_vs)
			if ((rc = dupload(c, &c->bez_full, ops.ccSB0_vs_vs, (size_t)n_s * n_s))) return fail(rc);
		c->visc_mu = (sim->pde_index == DPG_PDE_NAVIER_STOKES ? sim->mu : 0.0);
		c->adv_speed = std::sqrt(sim->b_adv[0] * sim->b_adv[0] + sim->b_adv[1] * sim->b_adv[1] + sim->b_adv[2] * sim->b_adv[2]);
	}
	if ((rc = dpg::fp64_configure(c))) return fail(rc);
	// boundary faces or viscous terms: the general chain (the periodic Euler / advection kernels have neither)
	{
		int has_bc = 0;
		for (int f = 0; f < n_face; ++f) has_bc |= (sim->face_vol[2 * f + 1] < 0);
		if (has_bc || sim->pde_index == DPG_PDE_NAVIER_STOKES)
			if ((rc = dpg::gen_prepare(c, sim))) return fail(rc);
	}
	if (cudaDeviceSynchronize() != cudaSuccess) return fail(DPG_ERR_CUDA);
	*ctx_out = c;
	return DPG_OK;
}

extern "C" void dpg_gpu_destroy(dpg_gpu_ctx* c)
{
	if (!c) return;
	if (c->stream) cudaStreamSynchronize(c->stream);
	dpg::split_free(c);
	dpg::gen_free(c);
	dpg::hp_free(c);
	dpg::implicit_free(c);
	dpg::mlp_free(c);
	if (c->step_graph) cudaGraphExecDestroy(c->step_graph);
	for (int i = 0; i < c->n_allocs; ++i) cudaFree(c->allocs[i]);
	if (c->stream) cudaStreamDestroy(c->stream);
	delete c;
}

static void invalidate_graph(dpg_gpu_ctx* c)
{
	if (c->step_graph) { cudaGraphExecDestroy(c->step_graph); c->step_graph = nullptr; }
	c->step_graph_mode = -1;
}

void dpg::invalidate_step_graph(dpg_gpu_ctx* c) { invalidate_graph(c); }

extern "C" int dpg_gpu_set_precision(dpg_gpu_ctx* c, int mode, int n_slices)
{
	if (!c) return DPG_ERR_INVALID;
	if (mode != DPG_PREC_FP64 && mode != DPG_PREC_BF16X3 && mode != DPG_PREC_TF32X3 && mode != DPG_PREC_BF16_SLICED)
		return DPG_ERR_INVALID;
	if (mode == DPG_PREC_BF16_SLICED && (n_slices < 2 || n_slices > 7)) return DPG_ERR_INVALID;
	// the split kernels cover periodic meshes of one order without viscous terms (affine elements: checked when
	// the operators are prepared)
	if (mode != DPG_PREC_FP64 && (c->general || c->hp)) return DPG_ERR_UNSUPPORTED;
	c->prec_mode = mode;
	c->n_slices = n_slices;
	invalidate_graph(c);
	if (mode != DPG_PREC_FP64) {
		const int rc = dpg::split_prepare(c);
		if (rc != DPG_OK) { c->prec_mode = DPG_PREC_FP64; c->n_slices = 0; }
		return rc;
	}
	dpg::split_free(c);
	return DPG_OK;
}

extern "C" int dpg_gpu_set_positivity(dpg_gpu_ctx* c, int on)
{
	if (!c) return DPG_ERR_INVALID;
	if (on && !c->pos_err) return DPG_ERR_UNSUPPORTED;   // density and pressure exist for the Euler equations only
	c->positivity = on ? 1 : 0;
	invalidate_graph(c);
	return DPG_OK;
}

extern "C" int dpg_gpu_enforce_positivity(dpg_gpu_ctx* c)
{
	if (!c) return DPG_ERR_INVALID;
	int rc = dpg::launch_positivity(c, c->sol);
	if (rc) return rc;
	const int e = dpg::positivity_error(c);
	return e < 0 ? DPG_ERR_CUDA : e ? DPG_ERR_NONFINITE : DPG_OK;
}

extern "C" int dpg_gpu_positivity_update(dpg_gpu_ctx* c, const double* du)
{
	if (!c || !du) return DPG_ERR_INVALID;
	if (!c->du_buf) {   // the update's device copy, allocated on first use and kept with the context
		int r = dalloc(c, &c->du_buf, (size_t)c->n_dof);
		if (r) return r;
	}
	double* d_du = c->du_buf;
	int rc = DPG_OK;
	if (cudaMemcpyAsync(d_du, du, sizeof(double) * c->n_dof, cudaMemcpyHostToDevice, c->stream) != cudaSuccess) rc = DPG_ERR_CUDA;
	if (!rc && c->positivity) {
		rc = dpg::launch_relaxed_update(c, c->sol, d_du);
		if (!rc) rc = dpg::launch_positivity(c, c->sol);
	} else if (!rc) {
		rc = dpg::launch_axpy(c, c->n_dof, 1.0, d_du, c->sol);
	}
	if (!rc) {
		const int e = dpg::positivity_error(c);
		rc = e < 0 ? DPG_ERR_CUDA : e ? DPG_ERR_NONFINITE : DPG_OK;
	}
	if (cudaStreamSynchronize(c->stream) != cudaSuccess && rc == DPG_OK) rc = DPG_ERR_CUDA;
	return rc;
}

extern "C" int dpg_gpu_upload_sol_coef(dpg_gpu_ctx* c, const double* h)
{
	if (!c || !h) return DPG_ERR_INVALID;
	CK(cudaMemcpyAsync(c->sol, h, sizeof(double) * c->n_dof, cudaMemcpyHostToDevice, c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return DPG_OK;
}

extern "C" int dpg_gpu_download_sol_coef(dpg_gpu_ctx* c, double* h)
{
	if (!c || !h) return DPG_ERR_INVALID;
	CK(cudaMemcpyAsync(h, c->sol, sizeof(double) * c->n_dof, cudaMemcpyDeviceToHost, c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return DPG_OK;
}

extern "C" int dpg_gpu_download_rhs(dpg_gpu_ctx* c, double* h)
{
	if (!c || !h) return DPG_ERR_INVALID;
	CK(cudaMemcpyAsync(h, c->rhs, sizeof(double) * c->n_dof, cudaMemcpyDeviceToHost, c->stream));
	CK(cudaStreamSynchronize(c->stream));
	return DPG_OK;
}

// One residual evaluation (optionally an RK stage) on the context stream; no synchronisation.
static int enqueue_residual(dpg_gpu_ctx* c, int stage, bool write_rhs, unsigned long long* max_slot)
{
	int rc;
	if (c->general) return dpg::gen_residual(c, stage, write_rhs, max_slot);
	if (c->hp) return dpg::hp_residual(c, stage, write_rhs, max_slot);
	if (c->prec_mode == DPG_PREC_FP64) {
		if ((rc = dpg::launch_trace(c))) return rc;
		if ((rc = dpg::launch_face(c))) return rc;
		return dpg::launch_volume(c, stage, write_rhs, max_slot);
	}
	if ((rc = dpg::split_launch_trace(c))) return rc;
	if ((rc = dpg::split_launch_face(c))) return rc;
	return dpg::split_launch_volume(c, stage, write_rhs, max_slot);
}

// One RK stage: the residual with the stage update, then the positivity limiter on the new state (the reference's
// enforce_positivity_highorder after every stage, solve_explicit.c:296).
static int enqueue_stage(dpg_gpu_ctx* c, int stage, unsigned long long* max_slot)
{
	const int rc = enqueue_residual(c, stage, false, max_slot);
	return rc ? rc : dpg::launch_positivity(c, c->sol);
}

int dpg::enqueue_residual_raw(dpg_gpu_ctx* c, unsigned long long* max_slot)
{
	return enqueue_residual(c, -1, true, max_slot);
}

static int read_max(dpg_gpu_ctx* c, int slot, double* out)
{
	unsigned long long bits = 0;
	CK(cudaMemcpyAsync(&bits, c->dmax + slot, sizeof bits, cudaMemcpyDeviceToHost, c->stream));
	CK(cudaStreamSynchronize(c->stream));
	double v;
	memcpy(&v, &bits, sizeof v);
	if (out) *out = v;
	if (c->prec_mode != DPG_PREC_FP64 && dpg::split_error(c)) return DPG_ERR_TIMEOUT;
	if (dpg::positivity_error(c)) return DPG_ERR_NONFINITE;   // the reference stops: average density / pressure ~ 0
	return std::isfinite(v) ? DPG_OK : DPG_ERR_NONFINITE;
}

extern "C" int dpg_gpu_compute_rhs(dpg_gpu_ctx* c, double* max_rhs)
{
	if (!c) return DPG_ERR_INVALID;
	CK(cudaMemsetAsync(c->dmax + dpg::kMaxStages, 0, sizeof(unsigned long long), c->stream));
	int rc = enqueue_residual(c, -1, true, c->dmax + dpg::kMaxStages);
	if (rc) return rc;
	return read_max(c, dpg::kMaxStages, max_rhs);
}

static int build_step_graph(dpg_gpu_ctx* c)
{
	invalidate_graph(c);
	cudaGraph_t graph = nullptr;
	CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
	int rc = DPG_OK;
	if (cudaMemsetAsync(c->dmax, 0, sizeof(unsigned long long) * dpg::kMaxStages, c->stream) != cudaSuccess) rc = DPG_ERR_CUDA;
	for (int stage = 0; stage < 3 && rc == DPG_OK; ++stage) rc = enqueue_stage(c, stage, c->dmax + stage);
	cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
	if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
	if (e != cudaSuccess) return DPG_ERR_CUDA;
	e = cudaGraphInstantiate(&c->step_graph, graph, 0);
	cudaGraphDestroy(graph);
	if (e != cudaSuccess) { c->step_graph = nullptr; return DPG_ERR_CUDA; }
	c->step_graph_mode = c->prec_mode * 16 + c->n_slices;
	return DPG_OK;
}

static int enqueue_steps(dpg_gpu_ctx* c, double dt, int n_steps)
{
	if (!c->step_graph || c->step_graph_mode != c->prec_mode * 16 + c->n_slices) {
		int rc = build_step_graph(c);
		if (rc) return rc;
	}
	CK(cudaMemcpyAsync(c->ddt, &dt, sizeof dt, cudaMemcpyHostToDevice, c->stream));
	for (int s = 0; s < n_steps; ++s) CK(cudaGraphLaunch(c->step_graph, c->stream));
	return DPG_OK;
}

extern "C" int dpg_gpu_rk_step(dpg_gpu_ctx* c, double dt, int n_steps, double* max_rhs)
{
	if (!c || n_steps < 0 || !(dt > 0.0)) return DPG_ERR_INVALID;
	if (n_steps == 0) { if (max_rhs) *max_rhs = 0.0; return DPG_OK; }
	// dt lives in device memory (read by the stage kernels), so host dt must stay valid until the copy is done:
	// enqueue_steps copies from a stack variable, hence the synchronisation in read_max below.
	int rc = enqueue_steps(c, dt, n_steps);
	if (rc) return rc;
	return read_max(c, 2, max_rhs);
}

extern "C" int dpg_gpu_solve_explicit(dpg_gpu_ctx* c, double t0, double time_final, double dt, int* n_steps_out,
                                      double* max_rhs)
{
	if (!c || !(dt > 0.0) || !(time_final >= t0)) return DPG_ERR_INVALID;
	// Same step control as solve_explicit: the last step is shortened to land on time_final.
	double t = t0;
	int n = 0;
	const double eps = 2.220446049250313e-16;
	int n_full = 0;
	{
		double tt = t0;
		while (!(tt + dt > time_final - 1e3 * eps)) { tt += dt; ++n_full; }
	}
	int rc = DPG_OK;
	if (n_full > 0) { rc = enqueue_steps(c, dt, n_full); if (rc) return rc; }
	for (int i = 0; i < n_full; ++i) t += dt;
	n = n_full;
	double mr = 0.0;
	if (n_full > 0) { rc = read_max(c, 2, &mr); if (rc) return rc; }
	const double dt_last = time_final - t;
	if (dt_last > 0.0) {
		rc = enqueue_steps(c, dt_last, 1);
		if (rc) return rc;
		rc = read_max(c, 2, &mr);
		if (rc) return rc;
		++n;
	}
	if (n_steps_out) *n_steps_out = n;
	if (max_rhs) *max_rhs = mr;
	return DPG_OK;
}

extern "C" int dpg_gpu_rk_step_host(dpg_gpu_ctx* c, double* sol_inout, double dt, int n_steps, double* max_rhs)
{
	if (!c || !sol_inout) return DPG_ERR_INVALID;
	CK(cudaMemcpyAsync(c->sol, sol_inout, sizeof(double) * c->n_dof, cudaMemcpyHostToDevice, c->stream));
	int rc = enqueue_steps(c, dt, n_steps);
	if (rc) return rc;
	CK(cudaMemcpyAsync(sol_inout, c->sol, sizeof(double) * c->n_dof, cudaMemcpyDeviceToHost, c->stream));
	return read_max(c, 2, max_rhs);
}

extern "C" int dpg_gpu_time_rk_steps(dpg_gpu_ctx* c, double dt, int n_steps, double* ms_out)
{
	if (!c || !ms_out || n_steps < 1 || !(dt > 0.0)) return DPG_ERR_INVALID;
	if (!c->step_graph || c->step_graph_mode != c->prec_mode * 16 + c->n_slices) {
		int rc = build_step_graph(c);
		if (rc) return rc;
	}
	CK(cudaMemcpyAsync(c->ddt, &dt, sizeof dt, cudaMemcpyHostToDevice, c->stream));
	cudaEvent_t e0, e1;
	CK(cudaEventCreate(&e0));
	CK(cudaEventCreate(&e1));
	CK(cudaEventRecord(e0, c->stream));
	for (int s = 0; s < n_steps; ++s) CK(cudaGraphLaunch(c->step_graph, c->stream));
	CK(cudaEventRecord(e1, c->stream));
	CK(cudaEventSynchronize(e1));
	float ms = 0.f;
	CK(cudaEventElapsedTime(&ms, e0, e1));
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	*ms_out = ms;
	double mr;
	return read_max(c, 2, &mr);
}

extern "C" int dpg_gpu_launches_per_rhs(dpg_gpu_ctx* c)
{
	if (!c) return 0;
	return c->general ? dpg::gen_launches_per_rhs(c) : 3;
}

extern "C" int dpg_gpu_kernel_times(dpg_gpu_ctx* c, int n_rep, double* ms_out, const char** names_out, int n_max)
{
	if (!c || !ms_out || n_rep < 1 || n_max < 3) return DPG_ERR_INVALID;
	static const char* names[3] = {"trace", "face", "volume"};
	cudaEvent_t ev[4];
	for (int i = 0; i < 4; ++i) CK(cudaEventCreate(&ev[i]));
	if (c->general) {   // the general chain is timed as one residual
		double acc1 = 0.0;
		for (int r = 0; r < n_rep; ++r) {
			CK(cudaEventRecord(ev[0], c->stream));
			int rc = dpg::gen_residual(c, -1, true, c->dmax + dpg::kMaxStages);
			if (rc) return rc;
			CK(cudaEventRecord(ev[1], c->stream));
			CK(cudaEventSynchronize(ev[1]));
			float ms = 0.f;
			CK(cudaEventElapsedTime(&ms, ev[0], ev[1]));
			acc1 += ms;
		}
		ms_out[0] = acc1 / n_rep;
		if (names_out) { names_out[0] = "residual"; names_out[1] = nullptr; names_out[2] = nullptr; if (n_max > 3) names_out[3] = nullptr; }
		for (int i = 0; i < 4; ++i) cudaEventDestroy(ev[i]);
		return DPG_OK;
	}
	double acc[3] = {0, 0, 0};
	unsigned long long* slot = c->dmax + dpg::kMaxStages;
	for (int r = 0; r < n_rep; ++r) {
		CK(cudaEventRecord(ev[0], c->stream));
		int rc = (c->hp ? dpg::hp_launch_part(c, 0, -1, true, slot)
		          : c->prec_mode == DPG_PREC_FP64 ? dpg::launch_trace(c) : dpg::split_launch_trace(c));
		if (rc) return rc;
		CK(cudaEventRecord(ev[1], c->stream));
		rc = (c->hp ? dpg::hp_launch_part(c, 1, -1, true, slot)
		      : c->prec_mode == DPG_PREC_FP64 ? dpg::launch_face(c) : dpg::split_launch_face(c));
		if (rc) return rc;
		CK(cudaEventRecord(ev[2], c->stream));
		rc = (c->hp ? dpg::hp_launch_part(c, 2, -1, true, slot)
		      : c->prec_mode == DPG_PREC_FP64 ? dpg::launch_volume(c, -1, true, slot)
		                                      : dpg::split_launch_volume(c, -1, true, slot));
		if (rc) return rc;
		CK(cudaEventRecord(ev[3], c->stream));
		CK(cudaEventSynchronize(ev[3]));
		for (int k = 0; k < 3; ++k) {
			float ms = 0.f;
			CK(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
			acc[k] += ms;
		}
	}
	for (int k = 0; k < 3; ++k) {
		ms_out[k] = acc[k] / n_rep;
		if (names_out) names_out[k] = names[k];
	}
	// the positivity limiter of an RK stage (on the current state; it changes no volume of a state that needs none)
	if (n_max > 3 && names_out) names_out[3] = nullptr;
	if (n_max > 3 && c->positivity) {
		double pacc = 0.0;
		for (int r = 0; r < n_rep; ++r) {
			CK(cudaEventRecord(ev[0], c->stream));
			int rc = dpg::launch_positivity(c, c->sol);
			if (rc) return rc;
			CK(cudaEventRecord(ev[1], c->stream));
			CK(cudaEventSynchronize(ev[1]));
			float ms = 0.f;
			CK(cudaEventElapsedTime(&ms, ev[0], ev[1]));
			pacc += ms;
		}
		ms_out[3] = pacc / n_rep;
		if (names_out) names_out[3] = "positivity";
		if (dpg::positivity_error(c)) return DPG_ERR_NONFINITE;
	}
	for (int i = 0; i < 4; ++i) cudaEventDestroy(ev[i]);
	return DPG_OK;
}

extern "C" void dpg_newton_params_default(struct dpg_newton_params* p)
{
	if (!p) return;
	memset(p, 0, sizeof *p);
	p->tol = 1e-10;
	p->max_newton = 50;
	p->gmres_restart = 200;
	p->max_gmres = 1000;
	p->gmres_rtol = 1e-4;
	p->dtau0 = 1.0;
	p->dtau_max = 1e12;
	p->precond = DPG_PRECOND_BLOCK_JACOBI;
}

namespace dpg {
// work buffers of the linearisation (tangents of the traces and face fluxes), allocated on first use
int ensure_tangent_buffers(dpg_gpu_ctx* c)
{
	if (c->trace_t && c->nnf_t) return DPG_OK;
	int rc;
	if ((rc = dalloc(c, &c->trace_t, (size_t)c->fc.n_face * 2 * c->n_var * c->fc.n_fc))) return rc;
	return dalloc(c, &c->nnf_t, (size_t)c->fc.n_face * c->n_var * c->fc.n_fc);
}
} // namespace dpg

extern "C" int dpg_gpu_jacobian_apply(dpg_gpu_ctx* c, const double* v, double* jv)
{
	if (!c || !v || !jv) return DPG_ERR_INVALID;
	if (c->hp) return DPG_ERR_UNSUPPORTED;   // the linearisation covers meshes of one order
	int rc;
	if ((rc = dpg::ensure_tangent_buffers(c))) return rc;
	double *dv = nullptr, *dj = nullptr;
	const size_t bytes = (size_t)c->n_dof * sizeof(double);
	if (cudaMalloc(&dv, bytes) != cudaSuccess) return DPG_ERR_CUDA;
	if (cudaMalloc(&dj, bytes) != cudaSuccess) { cudaFree(dv); return DPG_ERR_CUDA; }
	rc = DPG_OK;
	if (cudaMemcpyAsync(dv, v, bytes, cudaMemcpyHostToDevice, c->stream) != cudaSuccess) rc = DPG_ERR_CUDA;
	if (!rc) rc = dpg::jvp_fp64(c, c->sol, dv, dj, c->trace_t, c->nnf_t);
	if (!rc && cudaMemcpyAsync(jv, dj, bytes, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess) rc = DPG_ERR_CUDA;
	if (cudaStreamSynchronize(c->stream) != cudaSuccess && !rc) rc = DPG_ERR_CUDA;
	cudaFree(dv);
	cudaFree(dj);
	return rc;
}

extern "C" int dpg_gpu_newton_solve(dpg_gpu_ctx* c, const struct dpg_newton_params* prm, struct dpg_newton_stats* st)
{
	if (!c || !prm || !st) return DPG_ERR_INVALID;
	if (prm->precond < DPG_PRECOND_NONE || prm->precond > DPG_PRECOND_BLOCK_ILU || !(prm->tol > 0.0) || prm->max_newton < 0)
		return DPG_ERR_INVALID;
	if (c->hp) return DPG_ERR_UNSUPPORTED;                      // meshes of one order
	if (c->g.n_s * c->n_var > 128) return DPG_ERR_UNSUPPORTED;   // element blocks above 128 x 128
	return dpg::implicit_solve(c, prm, st);
}
