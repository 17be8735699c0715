// FP64 form of the DG residual: three kernels per residual evaluation.
//
//   k_trace   : per element, face traces  s_fc = cv0_vs_fc * sol_coef for every local face
//               (constructor_s_fc_interp_T, boundary_T.c:134-145), written to the face's slot of its side.
//   k_face    : per face node, numerical flux of (left trace, right trace reordered by nc_fc) with the left normal,
//               scaled by jacobian_det_fc (compute_face_rlhs_dg_T.c:88-114, scale_by_Jacobian_e_T).
//   k_volume  : per element, volume interpolation, Euler/advection flux with metric terms, the face fluxes of its
//               local faces gathered in a fixed order (right sides reordered and negated as in
//               compute_rhs_f_dg_like_T, compute_face_rlhs_T.c:297-310), one lift contraction
//               rhs = [tw1 | -tw0] * [fr ; nnf], the mass-matrix inverse, ||rhs||_inf and optionally the SSP-RK3
//               stage update of the element (time_step_ssp_rk_33, solve_explicit.c:252-301).
// Each element's residual is assembled by exactly one thread block in a fixed order: the face-to-element sums are
// deterministic and use no atomics.  The only atomic is the order-independent max of ||rhs||_inf.
#include <cmath>
#include <cstdio>
#include <cstring>

#include "dpg_gpu_internal.cuh"
#include "flux.cuh"

namespace dpg {

__device__ __forceinline__ void atomic_max_abs(unsigned long long* slot, double v)
{
	// |v| >= 0: the IEEE bit pattern orders like the value (NaN sorts above +inf and is kept).
	atomicMax(slot, (unsigned long long)__double_as_longlong(fabs(v)));
}

template <int NV>
__global__ void __launch_bounds__(256) k_trace(const double* __restrict__ sol, GroupDev g, double* __restrict__ trace, int E_b)
{
	extern __shared__ double sm[];
	const int n_s = g.n_s, n_fl = g.n_fl, n_fc = g.n_fc;
	const int e0 = blockIdx.x * E_b;
	const int ne = min(E_b, g.n_vol - e0);
	double* sU = sm;  // [ne][NV][n_s]
	const double* src = sol + (size_t)e0 * NV * n_s;
	for (int i = threadIdx.x; i < ne * NV * n_s; i += blockDim.x) sU[i] = src[i];
	__syncthreads();
	const int per_e = n_fl * NV * n_fc;
	for (int o = threadIdx.x; o < ne * per_e; o += blockDim.x) {
		const int e = o / per_e, r = o - e * per_e;
		const int lf = r / (NV * n_fc), r2 = r - lf * NV * n_fc;
		const int var = r2 / n_fc, q = r2 - var * n_fc;
		const double* op = g.Cf + (size_t)(lf * n_fc + q) * n_s;
		const double* u = sU + (e * NV + var) * n_s;
		double acc = 0.0;
		for (int s = 0; s < n_s; ++s) acc = fma(__ldg(op + s), u[s], acc);
		const int vf = g.vol_face[(size_t)(e0 + e) * n_fl + lf];
		trace[((size_t)vf * NV + var) * n_fc + q] = acc;   // vf = 2*face + side
	}
}

template <int D, int NV>
__global__ void __launch_bounds__(256) k_face(const double* __restrict__ trace, FaceDev fd, double* __restrict__ nnf,
                                              int num_flux, double bx, double by, double bz)
{
	const int n_fc = fd.n_fc;
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= fd.n_face * n_fc) return;
	const int f = t / n_fc, q = t - f * n_fc;
	const int qr = fd.nc[t];
	double WL[NV], WR[NV], n[D], nf[NV];
#pragma unroll
	for (int v = 0; v < NV; ++v) {
		WL[v] = trace[((size_t)(2 * f + 0) * NV + v) * n_fc + q];
		WR[v] = trace[((size_t)(2 * f + 1) * NV + v) * n_fc + qr];
	}
#pragma unroll
	for (int a = 0; a < D; ++a) n[a] = fd.nrm[(size_t)t * D + a];
	if constexpr (NV == D + 2) {
		if (num_flux == DPG_NUM_FLUX_ROE_PIKE) numflux_roe_pike<D>(WL, WR, n, nf);
		else                                   numflux_lax_friedrichs<D>(WL, WR, n, nf);
	} else {
		const double b[3] = {bx, by, bz};
		nf[0] = numflux_upwind<D>(b, WL[0], WR[0], n);
	}
	const double j = fd.jf[t];
#pragma unroll
	for (int v = 0; v < NV; ++v) nnf[((size_t)f * NV + v) * n_fc + q] = nf[v] * j;
}

// stage < 0: residual only.  stage 0..2: SSP-RK3 stage update of sol (solp holds the step's initial state).
template <int D, int NV>
__global__ void __launch_bounds__(256) k_volume(double* __restrict__ sol, double* __restrict__ solp, double* __restrict__ rhs,
                                                const double* __restrict__ nnf, GroupDev g, const double* __restrict__ dt_ptr,
                                                unsigned long long* max_slot, int stage, int write_rhs, int E_b,
                                                double bx, double by, double bz)
{
	extern __shared__ double sm[];
	const int n_s = g.n_s, n_c = g.n_c, n_fl = g.n_fl, n_fc = g.n_fc, K = g.K;
	const int e0 = blockIdx.x * E_b;
	const int ne = min(E_b, g.n_vol - e0);
	double* sU = sm;                          // [E_b][NV][n_s]
	double* sS = sU + (size_t)E_b * NV * n_s;  // [E_b][NV][n_c]  (reused for the unscaled residual)
	double* sX = sS + (size_t)E_b * NV * max(n_c, n_s); // [E_b][NV][K]
	const double* src = sol + (size_t)e0 * NV * n_s;
	for (int i = threadIdx.x; i < ne * NV * n_s; i += blockDim.x) sU[i] = src[i];
	__syncthreads();

	// 1. s_vc = cv0_vs_vc * sol_coef
	for (int o = threadIdx.x; o < ne * NV * n_c; o += blockDim.x) {
		const int ev = o / n_c, c = o - ev * n_c;
		const double* op = g.Cv + (size_t)c * n_s;
		const double* u = sU + (size_t)ev * n_s;
		double acc = 0.0;
		for (int s = 0; s < n_s; ++s) acc = fma(__ldg(op + s), u[s], acc);
		sS[o] = acc;
	}
	// 2. face fluxes of the local faces, in the element's own node order (negated on right sides)
	for (int o = threadIdx.x; o < ne * n_fl * n_fc; o += blockDim.x) {
		const int e = o / (n_fl * n_fc), r = o - e * n_fl * n_fc;
		const int lf = r / n_fc, q = r - lf * n_fc;
		const int vf = g.vol_face[(size_t)(e0 + e) * n_fl + lf];
		const int f = vf >> 1, side = vf & 1;
		const int qs = side ? g.nc_inv[(size_t)f * n_fc + q] : q;
		const double sgn = side ? -1.0 : 1.0;
#pragma unroll
		for (int v = 0; v < NV; ++v)
			sX[((size_t)e * NV + v) * K + D * n_c + r] = sgn * nnf[((size_t)f * NV + v) * n_fc + qs];
	}
	__syncthreads();
	// 3. physical flux and reference flux fr[eq][r][c] = sum_x m_{x r} f[x][eq]
	for (int o = threadIdx.x; o < ne * n_c; o += blockDim.x) {
		const int e = o / n_c, c = o - e * n_c;
		double s[NV];
#pragma unroll
		for (int v = 0; v < NV; ++v) s[v] = sS[((size_t)e * NV + v) * n_c + c];
		double m[D][D];
		const size_t ve = (size_t)(e0 + e);
#pragma unroll
		for (int x = 0; x < D; ++x)
#pragma unroll
			for (int r = 0; r < D; ++r)
				m[x][r] = g.affine ? g.met[ve * D * D + x + D * r] : g.met[(ve * D * D + x + D * r) * n_c + c];
		if constexpr (NV == D + 2) {
			double f[D][D + 2];
			flux_euler<D>(s, f);
#pragma unroll
			for (int eq = 0; eq < NV; ++eq)
#pragma unroll
				for (int r = 0; r < D; ++r) {
					double acc = 0.0;
#pragma unroll
					for (int x = 0; x < D; ++x) acc += m[x][r] * f[x][eq];
					sX[((size_t)e * NV + eq) * K + r * n_c + c] = acc;
				}
		} else {
			const double b[3] = {bx, by, bz};
#pragma unroll
			for (int r = 0; r < D; ++r) {
				double acc = 0.0;
#pragma unroll
				for (int x = 0; x < D; ++x) acc += m[x][r] * (b[x] * s[0]);
				sX[(size_t)e * K + r * n_c + c] = acc;
			}
		}
	}
	__syncthreads();
	// 4. lift: R = L * X  (K-long contraction per output)
	double* sR = sS;
	for (int o = threadIdx.x; o < ne * NV * n_s; o += blockDim.x) {
		const int ev = o / n_s, i = o - ev * n_s;
		const double* op = g.L + (size_t)i * K;
		const double* x = sX + (size_t)ev * K;
		double acc = 0.0;
		for (int k = 0; k < K; ++k) acc = fma(__ldg(op + k), x[k], acc);
		sR[o] = acc;
	}
	__syncthreads();
	// 5. mass-matrix inverse, RK stage, norm
	const double dt = (stage >= 0 ? *dt_ptr : 0.0);
	double lmax = 0.0;
	for (int o = threadIdx.x; o < ne * NV * n_s; o += blockDim.x) {
		const int ev = o / n_s, i = o - ev * n_s, e = ev / NV;
		double r;
		if (g.affine) {
			r = sR[o] * g.jinv[e0 + e];
		} else {
			const double* mi = g.minv + (size_t)(e0 + e) * n_s * n_s + (size_t)i * n_s;
			const double* x = sR + (size_t)ev * n_s;
			double acc = 0.0;
			for (int j = 0; j < n_s; ++j) acc = fma(mi[j], x[j], acc);
			r = acc;
		}
		lmax = fmax(lmax, fabs(r));
		if (isnan(r)) lmax = r;
		const size_t gi = (size_t)e0 * NV * n_s + o;
		if (write_rhs) rhs[gi] = r;
		if (stage == 0) { const double s0 = sU[o]; solp[gi] = s0; sol[gi] = s0 + dt * r; }
		else if (stage == 1) sol[gi] = (1.0 / 4.0) * (3.0 * solp[gi] + sU[o] + dt * r);
		else if (stage == 2) sol[gi] = (1.0 / 3.0) * (solp[gi] + 2.0 * sU[o] + 2.0 * dt * r);
	}
	// block max
	for (int off = 16; off > 0; off >>= 1) {
		const double other = __shfl_xor_sync(0xffffffffu, lmax, off);
		lmax = (isnan(other) || other > lmax) ? other : lmax;
	}
	if ((threadIdx.x & 31) == 0) atomic_max_abs(max_slot, lmax);
}

template <int D, int NV>
static int launch_all_impl(dpg_gpu_ctx* c, int which, int stage, bool write_rhs, unsigned long long* max_slot)
{
	const GroupDev& g = c->g;
	if (which == 0) {
		const int E_b = c->trace_block_elems;
		const size_t smem = (size_t)E_b * NV * g.n_s * sizeof(double);
		const int grid = (g.n_vol + E_b - 1) / E_b;
		k_trace<NV><<<grid, 256, smem, c->stream>>>(c->sol, g, c->trace, E_b);
	} else if (which == 1) {
		const int n = c->fc.n_face * c->fc.n_fc;
		k_face<D, NV><<<(n + 127) / 128, 128, 0, c->stream>>>(c->trace, c->fc, c->nnf, c->num_flux,
		                                                     c->b_adv[0], c->b_adv[1], c->b_adv[2]);
	} else {
		const int E_b = c->vol_block_elems;
		const size_t smem = (size_t)E_b * NV * (g.n_s + (g.n_c > g.n_s ? g.n_c : g.n_s) + g.K) * sizeof(double);
		const int grid = (g.n_vol + E_b - 1) / E_b;
		k_volume<D, NV><<<grid, 256, smem, c->stream>>>(c->sol, c->solp, c->rhs, c->nnf, g, c->ddt, max_slot, stage,
		                                               write_rhs ? 1 : 0, E_b, c->b_adv[0], c->b_adv[1], c->b_adv[2]);
	}
	return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

static int dispatch(dpg_gpu_ctx* c, int which, int stage, bool write_rhs, unsigned long long* max_slot)
{
	if (c->d == 2 && c->n_var == 4) return launch_all_impl<2, 4>(c, which, stage, write_rhs, max_slot);
	if (c->d == 3 && c->n_var == 5) return launch_all_impl<3, 5>(c, which, stage, write_rhs, max_slot);
	if (c->d == 2 && c->n_var == 1) return launch_all_impl<2, 1>(c, which, stage, write_rhs, max_slot);
	if (c->d == 3 && c->n_var == 1) return launch_all_impl<3, 1>(c, which, stage, write_rhs, max_slot);
	return DPG_ERR_UNSUPPORTED;
}

int launch_trace(dpg_gpu_ctx* c) { return dispatch(c, 0, -1, false, nullptr); }
int launch_face(dpg_gpu_ctx* c) { return dispatch(c, 1, -1, false, nullptr); }
int launch_volume(dpg_gpu_ctx* c, int stage, bool write_rhs, unsigned long long* max_slot)
{
	return dispatch(c, 2, stage, write_rhs, max_slot);
}

// ------------------------------------------------------------------------------------------------------------
// Linearisation: Jacobian-vector products J v = d(m_inv rhs)/du . v at the state u, by forward-mode tangents
// (dual.cuh) through the same formulas.  The traces are linear (k_trace on u and on v); the face kernel carries
// (trace, trace tangent) through the numerical flux; the volume kernel carries (s_vc, its tangent) through the
// physical flux and lifts the tangents of [fr ; nnf] with the same operators.  The products are exact to rounding
// (no difference quotient): the element blocks and the Krylov products of the implicit solver use them.
// ------------------------------------------------------------------------------------------------------------
template <int D, int NV>
__global__ void __launch_bounds__(256) k_face_tan(const double* __restrict__ trace, const double* __restrict__ trace_t,
                                                  FaceDev fd, double* __restrict__ nnf_t, int num_flux, double bx,
                                                  double by, double bz)
{
	const int n_fc = fd.n_fc;
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= fd.n_face * n_fc) return;
	const int f = t / n_fc, q = t - f * n_fc;
	const int qr = fd.nc[t];
	dual WL[NV], WR[NV], nf[NV];
	double n[D];
#pragma unroll
	for (int v = 0; v < NV; ++v) {
		const size_t iL = ((size_t)(2 * f + 0) * NV + v) * n_fc + q, iR = ((size_t)(2 * f + 1) * NV + v) * n_fc + qr;
		WL[v] = dual(trace[iL], trace_t[iL]);
		WR[v] = dual(trace[iR], trace_t[iR]);
	}
#pragma unroll
	for (int a = 0; a < D; ++a) n[a] = fd.nrm[(size_t)t * D + a];
	if constexpr (NV == D + 2) {
		if (num_flux == DPG_NUM_FLUX_ROE_PIKE) numflux_roe_pike<D>(WL, WR, n, nf);
		else                                   numflux_lax_friedrichs<D>(WL, WR, n, nf);
	} else {
		const double b[3] = {bx, by, bz};
		nf[0] = numflux_upwind<D>(b, WL[0], WR[0], n);
	}
	const double j = fd.jf[t];
#pragma unroll
	for (int v = 0; v < NV; ++v) nnf_t[((size_t)f * NV + v) * n_fc + q] = nf[v].d * j;
}

template <int D, int NV>
__global__ void __launch_bounds__(256) k_volume_tan(const double* __restrict__ u, const double* __restrict__ v,
                                                    const double* __restrict__ nnf_t, GroupDev g, double* __restrict__ out,
                                                    int E_b, double bx, double by, double bz)
{
	extern __shared__ double sm[];
	const int n_s = g.n_s, n_c = g.n_c, n_fl = g.n_fl, n_fc = g.n_fc, K = g.K;
	const int e0 = blockIdx.x * E_b;
	const int ne = min(E_b, g.n_vol - e0);
	double* sU = sm;                                    // [E_b][NV][n_s]  state
	double* sV = sU + (size_t)E_b * NV * n_s;           // [E_b][NV][n_s]  direction
	double* sS = sV + (size_t)E_b * NV * n_s;           // [E_b][NV][n_c]  s_vc (reused for the lifted tangent)
	double* sT = sS + (size_t)E_b * NV * max(n_c, n_s); // [E_b][NV][n_c]  tangent of s_vc
	double* sX = sT + (size_t)E_b * NV * n_c;           // [E_b][NV][K]    tangent of [fr ; nnf]
	for (int i = threadIdx.x; i < ne * NV * n_s; i += blockDim.x) {
		sU[i] = u[(size_t)e0 * NV * n_s + i];
		sV[i] = v[(size_t)e0 * NV * n_s + i];
	}
	__syncthreads();
	for (int o = threadIdx.x; o < ne * NV * n_c; o += blockDim.x) {
		const int ev = o / n_c, c = o - ev * n_c;
		const double* op = g.Cv + (size_t)c * n_s;
		double a0 = 0.0, a1 = 0.0;
		for (int s = 0; s < n_s; ++s) {
			const double w = __ldg(op + s);
			a0 = fma(w, sU[(size_t)ev * n_s + s], a0);
			a1 = fma(w, sV[(size_t)ev * n_s + s], a1);
		}
		sS[o] = a0;
		sT[o] = a1;
	}
	for (int o = threadIdx.x; o < ne * n_fl * n_fc; o += blockDim.x) {
		const int e = o / (n_fl * n_fc), r = o - e * n_fl * n_fc;
		const int lf = r / n_fc, q = r - lf * n_fc;
		const int vf = g.vol_face[(size_t)(e0 + e) * n_fl + lf];
		const int f = vf >> 1, side = vf & 1;
		const int qs = side ? g.nc_inv[(size_t)f * n_fc + q] : q;
		const double sgn = side ? -1.0 : 1.0;
#pragma unroll
		for (int w = 0; w < NV; ++w)
			sX[((size_t)e * NV + w) * K + D * n_c + r] = sgn * nnf_t[((size_t)f * NV + w) * n_fc + qs];
	}
	__syncthreads();
	for (int o = threadIdx.x; o < ne * n_c; o += blockDim.x) {
		const int e = o / n_c, c = o - e * n_c;
		dual sd[NV];
#pragma unroll
		for (int w = 0; w < NV; ++w) sd[w] = dual(sS[((size_t)e * NV + w) * n_c + c], sT[((size_t)e * NV + w) * n_c + c]);
		double m[D][D];
		const size_t ve = (size_t)(e0 + e);
#pragma unroll
		for (int x = 0; x < D; ++x)
#pragma unroll
			for (int r = 0; r < D; ++r)
				m[x][r] = g.affine ? g.met[ve * D * D + x + D * r] : g.met[(ve * D * D + x + D * r) * n_c + c];
		if constexpr (NV == D + 2) {
			dual f[D][D + 2];
			flux_euler<D>(sd, f);
#pragma unroll
			for (int eq = 0; eq < NV; ++eq)
#pragma unroll
				for (int r = 0; r < D; ++r) {
					double acc = 0.0;
#pragma unroll
					for (int x = 0; x < D; ++x) acc += m[x][r] * f[x][eq].d;
					sX[((size_t)e * NV + eq) * K + r * n_c + c] = acc;
				}
		} else {
			const double b[3] = {bx, by, bz};
#pragma unroll
			for (int r = 0; r < D; ++r) {
				double acc = 0.0;
#pragma unroll
				for (int x = 0; x < D; ++x) acc += m[x][r] * (b[x] * sd[0].d);
				sX[(size_t)e * K + r * n_c + c] = acc;
			}
		}
	}
	__syncthreads();
	double* sR = sS;
	for (int o = threadIdx.x; o < ne * NV * n_s; o += blockDim.x) {
		const int ev = o / n_s, i = o - ev * n_s;
		const double* op = g.L + (size_t)i * K;
		const double* x = sX + (size_t)ev * K;
		double acc = 0.0;
		for (int k = 0; k < K; ++k) acc = fma(__ldg(op + k), x[k], acc);
		sR[o] = acc;
	}
	__syncthreads();
	for (int o = threadIdx.x; o < ne * NV * n_s; o += blockDim.x) {
		const int ev = o / n_s, i = o - ev * n_s, e = ev / NV;
		double r;
		if (g.affine) {
			r = sR[o] * g.jinv[e0 + e];
		} else {
			const double* mi = g.minv + (size_t)(e0 + e) * n_s * n_s + (size_t)i * n_s;
			const double* x = sR + (size_t)ev * n_s;
			double acc = 0.0;
			for (int j = 0; j < n_s; ++j) acc = fma(mi[j], x[j], acc);
			r = acc;
		}
		out[(size_t)e0 * NV * n_s + o] = r;
	}
}

template <int D, int NV>
static int jvp_impl(dpg_gpu_ctx* c, const double* u, const double* v, double* out, double* trace_t, double* nnf_t)
{
	const GroupDev& g = c->g;
	const int E_t = c->trace_block_elems;
	const size_t smem_t = (size_t)E_t * NV * g.n_s * sizeof(double);
	const int grid_t = (g.n_vol + E_t - 1) / E_t;
	k_trace<NV><<<grid_t, 256, smem_t, c->stream>>>(u, g, c->trace, E_t);
	k_trace<NV><<<grid_t, 256, smem_t, c->stream>>>(v, g, trace_t, E_t);
	const int n = c->fc.n_face * c->fc.n_fc;
	k_face_tan<D, NV><<<(n + 127) / 128, 128, 0, c->stream>>>(c->trace, trace_t, c->fc, nnf_t, c->num_flux, c->b_adv[0],
	                                                         c->b_adv[1], c->b_adv[2]);
	const int E_b = c->tan_block_elems;
	const size_t smem = (size_t)E_b * NV * (2 * g.n_s + (g.n_c > g.n_s ? g.n_c : g.n_s) + g.n_c + g.K) * sizeof(double);
	k_volume_tan<D, NV><<<(g.n_vol + E_b - 1) / E_b, 256, smem, c->stream>>>(u, v, nnf_t, g, out, E_b, c->b_adv[0],
	                                                                       c->b_adv[1], c->b_adv[2]);
	return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

int jvp_fp64(dpg_gpu_ctx* c, const double* u, const double* v, double* out, double* trace_t, double* nnf_t)
{
	if (c->general) return gen_jvp(c, u, v, out);
	if (c->d == 2 && c->n_var == 4) return jvp_impl<2, 4>(c, u, v, out, trace_t, nnf_t);
	if (c->d == 3 && c->n_var == 5) return jvp_impl<3, 5>(c, u, v, out, trace_t, nnf_t);
	if (c->d == 2 && c->n_var == 1) return jvp_impl<2, 1>(c, u, v, out, trace_t, nnf_t);
	if (c->d == 3 && c->n_var == 1) return jvp_impl<3, 1>(c, u, v, out, trace_t, nnf_t);
	return DPG_ERR_UNSUPPORTED;
}

// Shared-memory opt-in for the dynamic sizes used above.
int fp64_configure(dpg_gpu_ctx* c)
{
	const GroupDev& g = c->g;
	const int NV = c->n_var;
	const size_t per_v = (size_t)NV * (g.n_s + (g.n_c > g.n_s ? g.n_c : g.n_s) + g.K) * sizeof(double);
	int E_b = (int)((96 * 1024) / per_v);
	if (E_b < 1) E_b = 1;
	if (E_b > 16) E_b = 16;
	c->vol_block_elems = E_b;
	const size_t per_t = (size_t)NV * g.n_s * sizeof(double);
	int E_t = (int)((32 * 1024) / per_t);
	if (E_t < 1) E_t = 1;
	if (E_t > 16) E_t = 16;
	c->trace_block_elems = E_t;
	const size_t per_j = (size_t)NV * (2 * g.n_s + (g.n_c > g.n_s ? g.n_c : g.n_s) + g.n_c + g.K) * sizeof(double);
	int E_j = (int)((96 * 1024) / per_j);
	if (E_j < 1) E_j = 1;
	if (E_j > 16) E_j = 16;
	c->tan_block_elems = E_j;
	const int smem_v = (int)(E_b * per_v), smem_t = (int)(E_t * per_t), smem_j = (int)(E_j * per_j);
	cudaError_t e = cudaSuccess;
#define SETATTR(KV, KT, KJ)                                                                                      \
	e = cudaFuncSetAttribute(KV, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_v); if (e) return DPG_ERR_CUDA; \
	e = cudaFuncSetAttribute(KT, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_t); if (e) return DPG_ERR_CUDA; \
	e = cudaFuncSetAttribute(KJ, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_j); if (e) return DPG_ERR_CUDA;
	if (c->d == 2 && NV == 4) { SETATTR((k_volume<2, 4>), (k_trace<4>), (k_volume_tan<2, 4>)) }
	else if (c->d == 3 && NV == 5) { SETATTR((k_volume<3, 5>), (k_trace<5>), (k_volume_tan<3, 5>)) }
	else if (c->d == 2 && NV == 1) { SETATTR((k_volume<2, 1>), (k_trace<1>), (k_volume_tan<2, 1>)) }
	else if (c->d == 3 && NV == 1) { SETATTR((k_volume<3, 1>), (k_trace<1>), (k_volume_tan<3, 1>)) }
	else return DPG_ERR_UNSUPPORTED;
#undef SETATTR
	return DPG_OK;
}

} // namespace dpg

// ------------------------------------------------------------------------------------------------------------
// Allocation-free residual (dpg_gpu_compute_rhs_noalloc).
//
// The face traces, face fluxes and the norm slot live in one statically declared device array.  Its name is a
// host-side stand-in in host code, so its device address is looked up once per device with cudaGetSymbolAddress
// (under a mutex) and passed to the kernels.  The first call on a device performs that look-up, so make it before
// any stream capture; every call sets the kernels' shared-memory limits for its sizes (a host-side setting that
// allocates nothing).  Every call reuses the array and
// overwrites what the previous call left in it (the norm slot is cleared on the stream at the start of each call);
// calls that overlap on the GPU race on it.
// ------------------------------------------------------------------------------------------------------------
#include <mutex>

namespace dpg {

static __device__ __align__(256) double g_noalloc_scratch[DPG_NOALLOC_SCRATCH_DOUBLES];

namespace {
constexpr int kNoallocMaxDevices = 64;
std::mutex g_noalloc_mutex;
double* g_noalloc_ptr[kNoallocMaxDevices] = {};
}

static int noalloc_setup(int dev, double** out)
{
	std::lock_guard<std::mutex> lock(g_noalloc_mutex);
	if (dev < 0 || dev >= kNoallocMaxDevices) return DPG_ERR_INVALID;
	if (!g_noalloc_ptr[dev]) {
		void* p = nullptr;
		if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess) return DPG_ERR_CUDA;
		g_noalloc_ptr[dev] = (double*)p;
	}
	*out = g_noalloc_ptr[dev];
	return DPG_OK;
}

template <int D, int NV>
static int noalloc_launch(const dpg_noalloc_mesh& m, const double* sol, double* rhs, double* scratch, cudaStream_t st)
{
	GroupDev g{};
	g.n_vol = m.n_vol; g.n_s = m.n_s; g.n_c = m.n_c; g.n_fl = m.n_fl; g.n_fc = m.n_fc;
	g.K = D * m.n_c + m.n_fl * m.n_fc;
	g.Cv = m.cv0_vs_vc; g.Cf = m.cv0_vs_fc; g.L = m.lift; g.met = m.metrics; g.jinv = m.jinv; g.minv = m.minv;
	g.vol_face = m.vol_face; g.nc_inv = m.nc_fc_inv; g.affine = (m.minv == nullptr);
	FaceDev fd{};
	fd.n_face = m.n_face; fd.n_fc = m.n_fc; fd.nrm = m.normals_fc; fd.jf = m.jacobian_det_fc; fd.nc = m.nc_fc;
	// scratch: [0, 32) doubles hold the norm slot; traces and face fluxes follow, 256-byte aligned
	unsigned long long* slot = (unsigned long long*)scratch;
	double* trace = scratch + 32;
	double* nnf = trace + (size_t)m.n_face * 2 * NV * m.n_fc;
	const size_t per_v = (size_t)NV * (g.n_s + (g.n_c > g.n_s ? g.n_c : g.n_s) + g.K) * sizeof(double);
	int E_b = (int)((96 * 1024) / per_v);
	E_b = E_b < 1 ? 1 : (E_b > 16 ? 16 : E_b);
	const size_t per_t = (size_t)NV * g.n_s * sizeof(double);
	int E_t = (int)((32 * 1024) / per_t);
	E_t = E_t < 1 ? 1 : (E_t > 16 ? 16 : E_t);
	if (cudaFuncSetAttribute(k_volume<D, NV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(E_b * per_v)) ||
	    cudaFuncSetAttribute(k_trace<NV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(E_t * per_t)))
		return DPG_ERR_CUDA;
	if (cudaMemsetAsync(slot, 0, sizeof(unsigned long long), st) != cudaSuccess) return DPG_ERR_CUDA;
	k_trace<NV><<<(g.n_vol + E_t - 1) / E_t, 256, E_t * per_t, st>>>(sol, g, trace, E_t);
	const int nq = fd.n_face * fd.n_fc;
	k_face<D, NV><<<(nq + 127) / 128, 128, 0, st>>>(trace, fd, nnf, m.num_flux, m.b_adv[0], m.b_adv[1], m.b_adv[2]);
	k_volume<D, NV><<<(g.n_vol + E_b - 1) / E_b, 256, E_b * per_v, st>>>(
	    const_cast<double*>(sol), nullptr, rhs, nnf, g, nullptr, slot, -1, 1, E_b, m.b_adv[0], m.b_adv[1], m.b_adv[2]);
	return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

} // namespace dpg

extern "C" int dpg_gpu_compute_rhs_noalloc(const struct dpg_noalloc_mesh* mesh, const double* sol_coef, double* rhs,
                                           double* max_rhs, void* cuda_stream)
{
	if (!mesh || !sol_coef || !rhs) return DPG_ERR_INVALID;
	const dpg_noalloc_mesh& m = *mesh;
	if (m.n_vol < 1 || m.n_face < 1 || m.n_s < 1 || m.n_c < 1 || m.n_fl < 1 || m.n_fc < 1) return DPG_ERR_INVALID;
	if (!m.cv0_vs_vc || !m.cv0_vs_fc || !m.lift || !m.metrics || !m.vol_face || !m.nc_fc || !m.nc_fc_inv ||
	    !m.normals_fc || !m.jacobian_det_fc || (!m.minv && !m.jinv))
		return DPG_ERR_INVALID;
	const size_t need = 32 + 3 * (size_t)m.n_face * m.n_var * m.n_fc;
	if (need > (size_t)DPG_NOALLOC_SCRATCH_DOUBLES) {
		fprintf(stderr, "dpg_gb300: dpg_gpu_compute_rhs_noalloc needs %zu scratch doubles, the fixed array holds %d\n",
		        need, DPG_NOALLOC_SCRATCH_DOUBLES);
		return DPG_ERR_TOO_LARGE;
	}
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess) return DPG_ERR_NO_DEVICE;
	double* scratch = nullptr;
	int rc = dpg::noalloc_setup(dev, &scratch);
	if (rc) return rc;
	cudaStream_t st = (cudaStream_t)cuda_stream;
	if (m.d == 2 && m.n_var == 4) rc = dpg::noalloc_launch<2, 4>(m, sol_coef, rhs, scratch, st);
	else if (m.d == 3 && m.n_var == 5) rc = dpg::noalloc_launch<3, 5>(m, sol_coef, rhs, scratch, st);
	else if (m.d == 2 && m.n_var == 1) rc = dpg::noalloc_launch<2, 1>(m, sol_coef, rhs, scratch, st);
	else if (m.d == 3 && m.n_var == 1) rc = dpg::noalloc_launch<3, 1>(m, sol_coef, rhs, scratch, st);
	else return DPG_ERR_UNSUPPORTED;
	if (rc || !max_rhs) return rc;
	unsigned long long bits = 0;
	if (cudaMemcpyAsync(&bits, scratch, sizeof bits, cudaMemcpyDeviceToHost, st) != cudaSuccess) return DPG_ERR_CUDA;
	if (cudaStreamSynchronize(st) != cudaSuccess) return DPG_ERR_CUDA;
	double v;
	memcpy(&v, &bits, sizeof v);
	*max_rhs = v;
	return std::isfinite(v) ? DPG_OK : DPG_ERR_NONFINITE;
}
