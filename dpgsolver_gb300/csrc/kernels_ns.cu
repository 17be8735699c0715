// FP64 residual with boundary faces and the BR2 Navier-Stokes terms (the general chain), templated on the scalar type:
// double for the residual and the RK stages, dual (dual.cuh) for the exact Jacobian-vector products of the
// linearisation.  Periodic Euler / advection meshes take the three-kernel path of kernels_fp64.cu; meshes with
// boundary faces, and the Navier-Stokes equations, take this one:
//
//   k_g_trace   per (element, local face, variable, node): face traces cv0_vs_fc * sol_coef into the (face, side)
//               slot (constructor_s_fc_interp_T, boundary_T.c:134-145);
//   k_g_ghost   per boundary face node: the boundary state into the side-1 slot (constructor_Boundary_Value_fcl,
//               face_solver_T.c:92-115; formulas in flux.cuh) -- from here on a boundary face reads like an interior
//               one with the identity node correspondence;
//   k_g_lift    BR2 only, per (face, side, direction, variable, basis function): tw0_vt_fc (jacobian_det_fc n_x
//               (s_num - s_side)) with the central s_num = (s_l + s_r)/2, the face part of grad_coef_f before the
//               mass-matrix inverse (compute_grad_coef_faces, dg/compute_grad_coef_dg_T.c:214-285, get_sol_scale); the
//               right side takes the same products in its own node order (the normal and s_num - s_r both change sign);
//   k_g_grad    BR2 only, per element: grad_coef_v = m_inv tw0_vt_vc (detJ d/dx) sol_coef (constructor_grad_xyz_p,
//               compute_grad_coef_volumes), the full gradient coefficients m_inv (tw0 (detJ d/dx) u + the faces' parts)
//               and, per local face, the partially corrected gradient cv0_vs_fc m_inv (.. + 1.01 NFMAX face part) at the
//               face nodes (constructor_partial_grad_fc_interp, compute_face_rlhs_dg_T.c:245-296); a boundary face
//               copies it to its side-1 slot (constructor_Boundary_Value_T_grad_from_internal);
//   k_g_face    per face node: inviscid numerical flux of the two traces, plus for BR2 the central flux of the
//               second-order fluxes at the two partial gradients (numerical_flux_central_T.c:75-100), the energy
//               component zero on adiabatic no-slip walls (set_provided_Numerical_Flux_members); times
//               jacobian_det_fc;
//   k_g_volume  per element: interpolation, inviscid (+ second-order at cv0_vs_vc grad_coef) flux with the metric
//               terms, the gathered face fluxes, one lift contraction [tw1 | -tw0] [fr ; nnf], m_inv, ||rhs||_inf and
//               the RK stage (double), or the tangent of m_inv rhs (dual).
// Every sum is formed by one thread in a fixed order: no atomics but the order-independent maximum of the norm.
#include <cstdio>
#include <cstring>
#include <vector>

#include "dpg_gpu_internal.cuh"
#include "dpg_host.h"
#include "flux.cuh"

namespace dpg {

struct GenDev {
	int n_vol, n_face, n_s, n_c, n_fl, n_fc, K, n_bface;
	int viscous, num_flux;
	double mu, Pr, scale;          // scale = 1.01 NFMAX (compute_scaling_weak_gradient)
	double b_adv[3];
	BcParams bp;
	const double* Cv;   // [n_c][n_s]
	const double* Cf;   // [n_fl n_fc][n_s]
	const double* Dv;   // [d][n_c][n_s]  d/dr of the basis at the volume cubature nodes
	const double* Wv;   // [n_s][n_c]     tw0_vt_vc
	const double* Tf;   // [n_fl][n_s][n_fc] tw0_vt_fc
	const double* L;    // [n_s][K]       [tw1 | -tw0]
	const double* met;  // [n_vol][d d][n_c]
	const double* minv; // [n_vol][n_s n_s]
	const int* vol_face;// [n_vol][n_fl] (face << 1) | side
	const int* face_lf; // [n_face][2] local face of each side (-1: boundary)
	const int* nc;      // [n_face][n_fc]
	const int* nc_inv;  // [n_face][n_fc]
	const double* nrm;  // [n_face][n_fc][d]
	const double* jf;   // [n_face][n_fc]
	const double* xyz;  // [n_face][n_fc][d]
	const int* bc;      // [n_face] 0 or the boundary code
	const int* bface;   // [n_bface] the boundary faces
};

struct GenBuffers {
	void* trace = nullptr;   // T [n_face][2][NV][n_fc]
	void* R = nullptr;       // T [n_face][2][d][NV][n_s]
	void* gc = nullptr;      // T [n_vol][d][NV][n_s]
	void* gf = nullptr;      // T [n_face][2][d][NV][n_fc]
	void* nnf = nullptr;     // T [n_face][NV][n_fc]
	void* u = nullptr;       // T [n_dof] (dual only: the state with the direction)
	void* out = nullptr;     // T [n_dof] (dual only: m_inv rhs with its tangent)
};

struct GenState {
	GenDev g{};
	GenBuffers buf[2];       // [0] double, [1] dual
	std::vector<void*> allocs;
	size_t smem_grad[2] = {0, 0}, smem_vol[2] = {0, 0};
};

template <class T> struct BufIndex { static constexpr int v = 0; };
template <> struct BufIndex<dual> { static constexpr int v = 1; };

__device__ __forceinline__ void atomic_max_abs_g(unsigned long long* slot, double v)
{
	atomicMax(slot, (unsigned long long)__double_as_longlong(fabs(v)));
}

// ---------------------------------------------------------------------------------------------------------------
template <class T, int NV>
__global__ void __launch_bounds__(256) k_g_trace(const T* __restrict__ u, GenDev g, T* __restrict__ trace)
{
	const int per_e = g.n_fl * NV * g.n_fc;
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= g.n_vol * per_e) return;
	const int e = t / per_e, r = t - e * per_e;
	const int lf = r / (NV * g.n_fc), r2 = r - lf * NV * g.n_fc;
	const int var = r2 / g.n_fc, q = r2 - var * g.n_fc;
	const double* op = g.Cf + (size_t)(lf * g.n_fc + q) * g.n_s;
	const T* x = u + ((size_t)e * NV + var) * g.n_s;
	T acc = 0.0;
	for (int s = 0; s < g.n_s; ++s) acc += __ldg(op + s) * x[s];
	const int vf = g.vol_face[(size_t)e * g.n_fl + lf];
	trace[((size_t)vf * NV + var) * g.n_fc + q] = acc;
}

template <class T, int D, int NV>
__global__ void __launch_bounds__(128) k_g_ghost(GenDev g, T* __restrict__ trace)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= g.n_bface * g.n_fc) return;
	const int f = g.bface[t / g.n_fc], q = t % g.n_fc;
	T sl[NV], sb[NV];
#pragma unroll
	for (int v = 0; v < NV; ++v) sl[v] = trace[((size_t)(2 * f) * NV + v) * g.n_fc + q];
	const size_t fq = (size_t)f * g.n_fc + q;
	double n[D], x[3] = {0, 0, 0};
#pragma unroll
	for (int a = 0; a < D; ++a) { n[a] = g.nrm[fq * D + a]; x[a] = g.xyz[fq * D + a]; }
	if constexpr (NV == D + 2) boundary_state<D>(g.bc[f], sl, n, x, g.bp, sb);
	else sb[0] = sl[0];
#pragma unroll
	for (int v = 0; v < NV; ++v) trace[((size_t)(2 * f + 1) * NV + v) * g.n_fc + q] = sb[v];
}

// One thread per (face, side, direction, variable, basis function).
template <class T, int D, int NV>
__global__ void __launch_bounds__(128) k_g_lift(const T* __restrict__ trace, GenDev g, T* __restrict__ R)
{
	const int n_fc = g.n_fc, per_side = D * NV * g.n_s;
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= g.n_face * 2 * per_side) return;
	const int fs = t / per_side, r = t - fs * per_side;
	const int f = fs >> 1, side = fs & 1;
	const int x = r / (NV * g.n_s), r2 = r - x * NV * g.n_s;
	const int var = r2 / g.n_s, i = r2 - var * g.n_s;
	const int lf = g.face_lf[fs];
	if (lf < 0) return;
	const double* tw = g.Tf + ((size_t)lf * g.n_s + i) * n_fc;
	T acc = 0.0;
	for (int qs = 0; qs < n_fc; ++qs) {
		const int q = side ? g.nc_inv[(size_t)f * n_fc + qs] : qs;   // the left node of this side's node qs
		const size_t fq = (size_t)f * n_fc + q;
		const T sl = trace[((size_t)(2 * f) * NV + var) * n_fc + q];
		const T sr = trace[((size_t)(2 * f + 1) * NV + var) * n_fc + g.nc[fq]];
		const T diff = -0.5 * sl + 0.5 * sr;
		acc += __ldg(tw + qs) * (g.jf[fq] * g.nrm[fq * D + x] * diff);
	}
	R[(size_t)fs * per_side + r] = acc;
}

// One block per element.  Shared memory (T): u [NV n_s], dr [D NV n_c], gx [D NV n_c], Gv [D NV n_s], A [D NV n_s].
template <class T, int D, int NV>
__global__ void __launch_bounds__(128) k_g_grad(const T* __restrict__ u, const T* __restrict__ R, GenDev g,
                                                T* __restrict__ gc, T* __restrict__ gf)
{
	extern __shared__ unsigned char smraw[];
	T* sm = reinterpret_cast<T*>(smraw);
	const int n_s = g.n_s, n_c = g.n_c, n_fc = g.n_fc, e = blockIdx.x;
	T* sU = sm;
	T* sDr = sU + NV * n_s;
	T* sGx = sDr + D * NV * n_c;
	T* sGv = sGx + D * NV * n_c;
	T* sA = sGv + D * NV * n_s;
	for (int k = threadIdx.x; k < NV * n_s; k += blockDim.x) sU[k] = u[(size_t)e * NV * n_s + k];
	__syncthreads();
	for (int k = threadIdx.x; k < D * NV * n_c; k += blockDim.x) {
		const int rr = k / (NV * n_c), k2 = k - rr * NV * n_c, var = k2 / n_c, c = k2 - var * n_c;
		const double* op = g.Dv + ((size_t)rr * n_c + c) * n_s;
		T acc = 0.0;
		for (int s = 0; s < n_s; ++s) acc += __ldg(op + s) * sU[var * n_s + s];
		sDr[k] = acc;
	}
	__syncthreads();
	for (int k = threadIdx.x; k < D * NV * n_c; k += blockDim.x) {
		const int x = k / (NV * n_c), k2 = k - x * NV * n_c, var = k2 / n_c, c = k2 - var * n_c;
		T acc = 0.0;
#pragma unroll
		for (int rr = 0; rr < D; ++rr)
			acc += g.met[((size_t)e * D * D + x + D * rr) * n_c + c] * sDr[(rr * NV + var) * n_c + c];
		sGx[k] = acc;
	}
	__syncthreads();
	for (int k = threadIdx.x; k < D * NV * n_s; k += blockDim.x) {
		const int xv = k / n_s, i = k - xv * n_s;
		const double* op = g.Wv + (size_t)i * n_c;
		T acc = 0.0;
		for (int c = 0; c < n_c; ++c) acc += __ldg(op + c) * sGx[xv * n_c + c];
		sGv[k] = acc;
	}
	__syncthreads();
	// full gradient coefficients
	for (int k = threadIdx.x; k < D * NV * n_s; k += blockDim.x) {
		T a = sGv[k];
		for (int lf = 0; lf < g.n_fl; ++lf) a += R[(size_t)g.vol_face[(size_t)e * g.n_fl + lf] * D * NV * n_s + k];
		sA[k] = a;
	}
	__syncthreads();
	const double* mi = g.minv + (size_t)e * n_s * n_s;
	for (int k = threadIdx.x; k < D * NV * n_s; k += blockDim.x) {
		const int xv = k / n_s, i = k - xv * n_s;
		T acc = 0.0;
		for (int j = 0; j < n_s; ++j) acc += mi[(size_t)i * n_s + j] * sA[xv * n_s + j];
		gc[(size_t)e * D * NV * n_s + k] = acc;
	}
	// partially corrected gradients at each local face's nodes
	for (int lf = 0; lf < g.n_fl; ++lf) {
		const int vf = g.vol_face[(size_t)e * g.n_fl + lf];
		const int f = vf >> 1, side = vf & 1;
		__syncthreads();
		for (int k = threadIdx.x; k < D * NV * n_s; k += blockDim.x) sA[k] = sGv[k] + g.scale * R[(size_t)vf * D * NV * n_s + k];
		__syncthreads();
		for (int k = threadIdx.x; k < D * NV * n_s; k += blockDim.x) {
			const int xv = k / n_s, i = k - xv * n_s;
			T acc = 0.0;
			for (int j = 0; j < n_s; ++j) acc += mi[(size_t)i * n_s + j] * sA[xv * n_s + j];
			sGx[k] = acc;   // m_inv (..) in the (unused now) gx array, n_c >= n_s
		}
		__syncthreads();
		const bool boundary = (side == 0 && g.bc[f] != 0);
		for (int k = threadIdx.x; k < D * NV * n_fc; k += blockDim.x) {
			const int xv = k / n_fc, q = k - xv * n_fc;
			const double* op = g.Cf + (size_t)(lf * n_fc + q) * n_s;
			T acc = 0.0;
			for (int i = 0; i < n_s; ++i) acc += __ldg(op + i) * sGx[xv * n_s + i];
			gf[(size_t)vf * D * NV * n_fc + k] = acc;
			if (boundary) gf[(size_t)(2 * f + 1) * D * NV * n_fc + k] = acc;
		}
	}
}

template <class T, int D, int NV>
__global__ void __launch_bounds__(128) k_g_face(const T* __restrict__ trace, const T* __restrict__ gf, GenDev g,
                                                T* __restrict__ nnf)
{
	const int n_fc = g.n_fc;
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= g.n_face * n_fc) return;
	const int f = t / n_fc, q = t - f * n_fc, qr = g.nc[t];
	T WL[NV], WR[NV], nf[NV];
#pragma unroll
	for (int v = 0; v < NV; ++v) {
		WL[v] = trace[((size_t)(2 * f) * NV + v) * n_fc + q];
		WR[v] = trace[((size_t)(2 * f + 1) * NV + v) * n_fc + qr];
	}
	double n[D];
#pragma unroll
	for (int a = 0; a < D; ++a) n[a] = g.nrm[(size_t)t * D + a];
	if constexpr (NV == D + 2) {
		if (g.num_flux == DPG_NUM_FLUX_ROE_PIKE) numflux_roe_pike<D>(WL, WR, n, nf);
		else                                     numflux_lax_friedrichs<D>(WL, WR, n, nf);
		if (g.viscous) {
			T gl[D][NV], gr[D][NV], fl[D][NV], fr[D][NV];
#pragma unroll
			for (int x = 0; x < D; ++x)
#pragma unroll
				for (int v = 0; v < NV; ++v) {
					gl[x][v] = gf[((size_t)(2 * f) * D * NV + x * NV + v) * n_fc + q];
					gr[x][v] = gf[((size_t)(2 * f + 1) * D * NV + x * NV + v) * n_fc + qr];
				}
			flux_viscous<D>(g.mu, g.Pr, WL, gl, fl);
			flux_viscous<D>(g.mu, g.Pr, WR, gr, fr);
#pragma unroll
			for (int x = 0; x < D; ++x)
#pragma unroll
				for (int v = 0; v < NV; ++v) nf[v] += n[x] * (0.5 * fl[x][v] + 0.5 * fr[x][v]);
			if (g.bc[f] == DPG_BC_NOSLIP_ADIABATIC) nf[D + 1] = T(0.0);
		}
	} else {
		nf[0] = numflux_upwind<D>(g.b_adv, WL[0], WR[0], n);
	}
	const double j = g.jf[t];
#pragma unroll
	for (int v = 0; v < NV; ++v) nnf[((size_t)f * NV + v) * n_fc + q] = nf[v] * j;
}

// One block per element.  Shared memory (T): u [NV n_s], s_vc [NV n_c], g_vc [D NV n_c] (BR2), X [NV K], R [NV n_s].
// Outputs: T = double: rhs (write_rhs), the RK stage (stage >= 0) and the norm; T = dual: out = m_inv rhs.
template <class T, int D, int NV>
__global__ void __launch_bounds__(128) k_g_volume(const T* __restrict__ u, const T* __restrict__ gc,
                                                  const T* __restrict__ nnf, GenDev g, T* __restrict__ out,
                                                  double* __restrict__ sol, double* __restrict__ solp,
                                                  const double* __restrict__ dt_ptr, unsigned long long* max_slot,
                                                  int stage, int write_rhs)
{
	extern __shared__ unsigned char smraw[];
	T* sm = reinterpret_cast<T*>(smraw);
	const int n_s = g.n_s, n_c = g.n_c, n_fl = g.n_fl, n_fc = g.n_fc, K = g.K, e = blockIdx.x;
	T* sU = sm;
	T* sS = sU + NV * n_s;
	T* sG = sS + NV * n_c;
	T* sX = sG + (g.viscous ? D * NV * n_c : 0);
	T* sR = sX + NV * K;
	for (int k = threadIdx.x; k < NV * n_s; k += blockDim.x) sU[k] = u[(size_t)e * NV * n_s + k];
	__syncthreads();
	for (int k = threadIdx.x; k < NV * n_c; k += blockDim.x) {
		const int var = k / n_c, c = k - var * n_c;
		const double* op = g.Cv + (size_t)c * n_s;
		T acc = 0.0;
		for (int s = 0; s < n_s; ++s) acc += __ldg(op + s) * sU[var * n_s + s];
		sS[k] = acc;
	}
	if (g.viscous)
		for (int k = threadIdx.x; k < D * NV * n_c; k += blockDim.x) {
			const int xv = k / n_c, c = k - xv * n_c;
			const double* op = g.Cv + (size_t)c * n_s;
			const T* gsrc = gc + (size_t)e * D * NV * n_s + (size_t)xv * n_s;
			T acc = 0.0;
			for (int s = 0; s < n_s; ++s) acc += __ldg(op + s) * gsrc[s];
			sG[k] = acc;
		}
	for (int k = threadIdx.x; k < n_fl * n_fc; k += blockDim.x) {
		const int lf = k / n_fc, q = k - lf * n_fc;
		const int vf = g.vol_face[(size_t)e * n_fl + lf];
		const int f = vf >> 1, side = vf & 1;
		const int qs = side ? g.nc_inv[(size_t)f * n_fc + q] : q;
		const double sgn = side ? -1.0 : 1.0;
#pragma unroll
		for (int v = 0; v < NV; ++v) sX[v * K + D * n_c + k] = sgn * nnf[((size_t)f * NV + v) * n_fc + qs];
	}
	__syncthreads();
	for (int c = threadIdx.x; c < n_c; c += blockDim.x) {
		T s[NV];
#pragma unroll
		for (int v = 0; v < NV; ++v) s[v] = sS[v * n_c + c];
		double m[D][D];
#pragma unroll
		for (int x = 0; x < D; ++x)
#pragma unroll
			for (int r = 0; r < D; ++r) m[x][r] = g.met[((size_t)e * D * D + x + D * r) * n_c + c];
		T f[D][NV];
		if constexpr (NV == D + 2) {
			flux_euler<D>(s, f);
			if (g.viscous) {
				T gv[D][NV], fv[D][NV];
#pragma unroll
				for (int x = 0; x < D; ++x)
#pragma unroll
					for (int v = 0; v < NV; ++v) gv[x][v] = sG[(x * NV + v) * n_c + c];
				flux_viscous<D>(g.mu, g.Pr, s, gv, fv);
#pragma unroll
				for (int x = 0; x < D; ++x)
#pragma unroll
					for (int v = 0; v < NV; ++v) f[x][v] += fv[x][v];
			}
		} else {
#pragma unroll
			for (int x = 0; x < D; ++x) f[x][0] = g.b_adv[x] * s[0];
		}
#pragma unroll
		for (int eq = 0; eq < NV; ++eq)
#pragma unroll
			for (int r = 0; r < D; ++r) {
				T acc = 0.0;
#pragma unroll
				for (int x = 0; x < D; ++x) acc += m[x][r] * f[x][eq];
				sX[eq * K + r * n_c + c] = acc;
			}
	}
	__syncthreads();
	for (int k = threadIdx.x; k < NV * n_s; k += blockDim.x) {
		const int v = k / n_s, i = k - v * n_s;
		const double* op = g.L + (size_t)i * K;
		T acc = 0.0;
		for (int kk = 0; kk < K; ++kk) acc += __ldg(op + kk) * sX[v * K + kk];
		sR[k] = acc;
	}
	__syncthreads();
	const double* mi = g.minv + (size_t)e * n_s * n_s;
	double lmax = 0.0;
	const double dt = (stage >= 0 ? *dt_ptr : 0.0);
	for (int k = threadIdx.x; k < NV * n_s; k += blockDim.x) {
		const int v = k / n_s, i = k - v * n_s;
		T r = 0.0;
		for (int j = 0; j < n_s; ++j) r += mi[(size_t)i * n_s + j] * sR[v * n_s + j];
		const size_t gi = (size_t)e * NV * n_s + k;
		if constexpr (BufIndex<T>::v == 1) {
			out[gi] = r;
		} else {
			lmax = fmax(lmax, fabs(r));
			if (isnan(r)) lmax = r;
			if (write_rhs) out[gi] = r;
			const double s0 = sU[k];
			if (stage == 0) { solp[gi] = s0; sol[gi] = s0 + dt * r; }
			else if (stage == 1) sol[gi] = (1.0 / 4.0) * (3.0 * solp[gi] + s0 + dt * r);
			else if (stage == 2) sol[gi] = (1.0 / 3.0) * (solp[gi] + 2.0 * s0 + 2.0 * dt * r);
		}
	}
	if constexpr (BufIndex<T>::v == 0) {
		for (int off = 16; off > 0; off >>= 1) {
			const double other = __shfl_xor_sync(0xffffffffu, lmax, off);
			lmax = (isnan(other) || other > lmax) ? other : lmax;
		}
		if ((threadIdx.x & 31) == 0 && max_slot) atomic_max_abs_g(max_slot, lmax);
	}
}

__global__ void k_g_pack(const double* __restrict__ u, const double* __restrict__ v, dual* __restrict__ w, int64_t n)
{
	const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) w[i] = dual(u[i], v[i]);
}

__global__ void k_g_unpack(const dual* __restrict__ w, double* __restrict__ out, int64_t n)
{
	const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) out[i] = w[i].d;
}

// ---------------------------------------------------------------------------------------------------------------
template <class T, int D, int NV>
static size_t smem_grad(const GenDev& g) { return sizeof(T) * (size_t)(NV * g.n_s + 2 * D * NV * g.n_c + 2 * D * NV * g.n_s); }
template <class T, int D, int NV>
static size_t smem_vol(const GenDev& g)
{
	return sizeof(T) * (size_t)(NV * g.n_s + NV * g.n_c + (g.viscous ? D * NV * g.n_c : 0) + NV * g.K + NV * g.n_s);
}

static int galloc(GenState* st, void** p, size_t bytes)
{
	if (cudaMalloc(p, bytes ? bytes : 8) != cudaSuccess) return DPG_ERR_CUDA;
	st->allocs.push_back(*p);
	return DPG_OK;
}

template <class T>
static int ensure_buffers(dpg_gpu_ctx* c, GenState* st)
{
	GenBuffers& b = st->buf[BufIndex<T>::v];
	if (b.trace) return DPG_OK;
	const GenDev& g = st->g;
	const int NV = c->n_var, D = c->d;
	int rc;
	if ((rc = galloc(st, &b.trace, sizeof(T) * (size_t)g.n_face * 2 * NV * g.n_fc))) return rc;
	if ((rc = galloc(st, &b.nnf, sizeof(T) * (size_t)g.n_face * NV * g.n_fc))) return rc;
	if (g.viscous) {
		if ((rc = galloc(st, &b.R, sizeof(T) * (size_t)g.n_face * 2 * D * NV * g.n_s))) return rc;
		if ((rc = galloc(st, &b.gc, sizeof(T) * (size_t)g.n_vol * D * NV * g.n_s))) return rc;
		if ((rc = galloc(st, &b.gf, sizeof(T) * (size_t)g.n_face * 2 * D * NV * g.n_fc))) return rc;
		if (cudaMemset(b.R, 0, sizeof(T) * (size_t)g.n_face * 2 * D * NV * g.n_s) != cudaSuccess) return DPG_ERR_CUDA;
	}
	if (BufIndex<T>::v == 1) {
		if ((rc = galloc(st, &b.u, sizeof(T) * (size_t)c->n_dof))) return rc;
		if ((rc = galloc(st, &b.out, sizeof(T) * (size_t)c->n_dof))) return rc;
	}
	return DPG_OK;
}

template <class T, int D, int NV>
static int configure(GenState* st)
{
	const size_t sg = smem_grad<T, D, NV>(st->g), sv = smem_vol<T, D, NV>(st->g);
	if (sg > 227 * 1024 || sv > 227 * 1024) return DPG_ERR_UNSUPPORTED;
	if (st->g.n_c < st->g.n_s) return DPG_ERR_UNSUPPORTED;   // k_g_grad reuses an [n_c] array for [n_s] values
	if (cudaFuncSetAttribute(k_g_grad<T, D, NV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sg) != cudaSuccess)
		return DPG_ERR_CUDA;
	if (cudaFuncSetAttribute(k_g_volume<T, D, NV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sv) != cudaSuccess)
		return DPG_ERR_CUDA;
	st->smem_grad[BufIndex<T>::v] = sg;
	st->smem_vol[BufIndex<T>::v] = sv;
	return DPG_OK;
}

// The chain on the state u (T), into out (T) or the RK stage of c->sol.
template <class T, int D, int NV>
static int run_chain(dpg_gpu_ctx* c, GenState* st, const T* u, T* out, int stage, bool write_rhs, unsigned long long* max_slot)
{
	const GenDev& g = st->g;
	GenBuffers& b = st->buf[BufIndex<T>::v];
	T* trace = (T*)b.trace;
	const int nt = g.n_vol * g.n_fl * NV * g.n_fc;
	k_g_trace<T, NV><<<(nt + 255) / 256, 256, 0, c->stream>>>(u, g, trace);
	if (g.n_bface) {
		const int nb = g.n_bface * g.n_fc;
		k_g_ghost<T, D, NV><<<(nb + 127) / 128, 128, 0, c->stream>>>(g, trace);
	}
	if (g.viscous) {
		const int nl = g.n_face * 2 * D * NV * g.n_s;
		k_g_lift<T, D, NV><<<(nl + 127) / 128, 128, 0, c->stream>>>(trace, g, (T*)b.R);
		k_g_grad<T, D, NV><<<g.n_vol, 128, st->smem_grad[BufIndex<T>::v], c->stream>>>(u, (const T*)b.R, g, (T*)b.gc, (T*)b.gf);
	}
	const int nf = g.n_face * g.n_fc;
	k_g_face<T, D, NV><<<(nf + 127) / 128, 128, 0, c->stream>>>(trace, (const T*)b.gf, g, (T*)b.nnf);
	k_g_volume<T, D, NV><<<g.n_vol, 128, st->smem_vol[BufIndex<T>::v], c->stream>>>(
		u, (const T*)b.gc, (const T*)b.nnf, g, out, c->sol, c->solp, c->ddt, max_slot, stage, write_rhs ? 1 : 0);
	return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

template <int D, int NV>
static int residual_impl(dpg_gpu_ctx* c, int stage, bool write_rhs, unsigned long long* max_slot)
{
	GenState* st = (GenState*)c->general;
	return run_chain<double, D, NV>(c, st, c->sol, c->rhs, stage, write_rhs, max_slot);
}

template <int D, int NV>
static int jvp_impl(dpg_gpu_ctx* c, const double* u, const double* v, double* out)
{
	GenState* st = (GenState*)c->general;
	int rc;
	if ((rc = ensure_buffers<dual>(c, st))) return rc;
	if (!st->smem_vol[1] && (rc = configure<dual, D, NV>(st))) return rc;
	GenBuffers& b = st->buf[1];
	const int64_t n = c->n_dof;
	k_g_pack<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>(u, v, (dual*)b.u, n);
	if ((rc = run_chain<dual, D, NV>(c, st, (const dual*)b.u, (dual*)b.out, -1, true, nullptr))) return rc;
	k_g_unpack<<<(unsigned)((n + 255) / 256), 256, 0, c->stream>>>((const dual*)b.out, out, n);
	return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

int gen_residual(dpg_gpu_ctx* c, int stage, bool write_rhs, unsigned long long* max_slot)
{
	if (c->d == 2 && c->n_var == 4) return residual_impl<2, 4>(c, stage, write_rhs, max_slot);
	if (c->d == 3 && c->n_var == 5) return residual_impl<3, 5>(c, stage, write_rhs, max_slot);
	if (c->d == 2 && c->n_var == 1) return residual_impl<2, 1>(c, stage, write_rhs, max_slot);
	if (c->d == 3 && c->n_var == 1) return residual_impl<3, 1>(c, stage, write_rhs, max_slot);
	return DPG_ERR_UNSUPPORTED;
}

int gen_jvp(dpg_gpu_ctx* c, const double* u, const double* v, double* out)
{
	if (c->d == 2 && c->n_var == 4) return jvp_impl<2, 4>(c, u, v, out);
	if (c->d == 3 && c->n_var == 5) return jvp_impl<3, 5>(c, u, v, out);
	if (c->d == 2 && c->n_var == 1) return jvp_impl<2, 1>(c, u, v, out);
	if (c->d == 3 && c->n_var == 1) return jvp_impl<3, 1>(c, u, v, out);
	return DPG_ERR_UNSUPPORTED;
}

int gen_launches_per_rhs(dpg_gpu_ctx* c)
{
	const GenState* st = (const GenState*)c->general;
	return 3 + (st->g.n_bface ? 1 : 0) + (st->g.viscous ? 2 : 0);
}

void gen_free(dpg_gpu_ctx* c)
{
	GenState* st = (GenState*)c->general;
	if (!st) return;
	for (void* p : st->allocs) cudaFree(p);
	delete st;
	c->general = nullptr;
}

template <class T>
static int upload(GenState* st, const T** dst, const T* src, size_t n)
{
	void* p = nullptr;
	int rc = galloc(st, &p, sizeof(T) * n);
	if (rc) return rc;
	if (n && cudaMemcpy(p, src, sizeof(T) * n, cudaMemcpyHostToDevice) != cudaSuccess) return DPG_ERR_CUDA;
	*dst = (const T*)p;
	return DPG_OK;
}

// Host set-up of the general chain: operators (the derivative operator of the basis at the volume cubature nodes
// from the Lagrange basis on the GLL nodes; tw0_vt_vc = cv0^T diag(w_vc); [tw1 | -tw0]), per-node metric terms and
// mass-matrix inverses of every volume, and the face tables with the boundary conditions.
int gen_prepare(dpg_gpu_ctx* c, const struct dpg_sim* sim)
{
	const dpg_element_ops& ops = sim->ops[0];
	const int d = sim->d, nv = sim->n_var, n_s = ops.n_s, n_c = ops.n_c, n_fl = ops.n_fl, n_fc = ops.n_fc;
	const int n_vol = sim->n_vol, n_face = sim->n_face, K = d * n_c + n_fl * n_fc;
	GenState* st = new GenState();
	c->general = st;
	GenDev& g = st->g;
	g.n_vol = n_vol; g.n_face = n_face; g.n_s = n_s; g.n_c = n_c; g.n_fl = n_fl; g.n_fc = n_fc; g.K = K;
	g.viscous = (sim->pde_index == DPG_PDE_NAVIER_STOKES);
	g.num_flux = sim->ind_num_flux[0];
	g.mu = sim->mu; g.Pr = sim->Pr; g.scale = 1.01 * n_fl;
	for (int a = 0; a < 3; ++a) g.b_adv[a] = sim->b_adv[a];
	g.bp.omega = sim->bc_omega; g.bp.rho_b = sim->bc_rho; g.bp.E_b = sim->bc_E;
	for (int k = 0; k < 5; ++k) g.bp.ext[k] = sim->bc_state[k];
	int rc;
	if ((rc = upload(st, &g.Cv, ops.cv0_vs_vc, (size_t)n_c * n_s))) return rc;
	if ((rc = upload(st, &g.Cf, ops.cv0_vs_fc, (size_t)n_fl * n_fc * n_s))) return rc;
	if ((rc = upload(st, &g.Tf, ops.tw0_vt_fc, (size_t)n_fl * n_s * n_fc))) return rc;
	std::vector<double> Dv((size_t)d * n_c * n_s), Wv((size_t)n_s * n_c), L((size_t)n_s * K);
	{
		const int n1 = ops.p + 1;
		double g1[16], val[125], grad[3 * 125];
		for (int i = 0; i < n1; ++i) g1[i] = ops.rst_vs[(size_t)i * d];
		for (int cc = 0; cc < n_c; ++cc) {
			dpg_tp_basis_at(d, n1, g1, &ops.rst_vc[(size_t)cc * d], val, grad);
			for (int a = 0; a < d; ++a)
				for (int s = 0; s < n_s; ++s) Dv[((size_t)a * n_c + cc) * n_s + s] = grad[(size_t)a * n_s + s];
		}
		for (int i = 0; i < n_s; ++i)
			for (int cc = 0; cc < n_c; ++cc) Wv[(size_t)i * n_c + cc] = ops.cv0_vs_vc[(size_t)cc * n_s + i] * ops.w_vc[cc];
		for (int i = 0; i < n_s; ++i) {
			for (int r = 0; r < d; ++r)
				for (int cc = 0; cc < n_c; ++cc) L[(size_t)i * K + r * n_c + cc] = ops.tw1_vt_vc[((size_t)r * n_s + i) * n_c + cc];
			for (int lf = 0; lf < n_fl; ++lf)
				for (int q = 0; q < n_fc; ++q)
					L[(size_t)i * K + d * n_c + lf * n_fc + q] = -ops.tw0_vt_fc[((size_t)lf * n_s + i) * n_fc + q];
		}
	}
	if ((rc = upload(st, &g.Dv, Dv.data(), Dv.size()))) return rc;
	if ((rc = upload(st, &g.Wv, Wv.data(), Wv.size()))) return rc;
	if ((rc = upload(st, &g.L, L.data(), L.size()))) return rc;
	if ((rc = upload(st, &g.met, sim->metrics_vc, (size_t)n_vol * n_c * d * d))) return rc;
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
	if ((rc = upload(st, &g.minv, minv.data(), minv.size()))) return rc;
	std::vector<int> vf((size_t)n_vol * n_fl), flf((size_t)2 * n_face), ncinv((size_t)n_face * n_fc), bc(n_face), bfaces;
	for (int v = 0; v < n_vol; ++v)
		for (int lf = 0; lf < n_fl; ++lf)
			vf[(size_t)v * n_fl + lf] = (sim->vol_face[v * DPG_NFL_MAX + lf] << 1) | sim->vol_face_side[v * DPG_NFL_MAX + lf];
	for (int f = 0; f < n_face; ++f) {
		flf[2 * f] = sim->face_lf[2 * f];
		flf[2 * f + 1] = sim->face_vol[2 * f + 1] < 0 ? -1 : sim->face_lf[2 * f + 1];
		bc[f] = sim->face_vol[2 * f + 1] < 0 ? sim->face_bc[f] : 0;
		if (bc[f]) bfaces.push_back(f);
		for (int q = 0; q < n_fc; ++q) ncinv[(size_t)f * n_fc + sim->nc_fc[(size_t)f * n_fc + q]] = q;
	}
	g.n_bface = (int)bfaces.size();
	std::vector<double> xyz((size_t)n_face * n_fc * d);
	for (int f = 0; f < n_face; ++f)
		for (int q = 0; q < n_fc; ++q)
			for (int a = 0; a < d; ++a)
				xyz[((size_t)f * n_fc + q) * d + a] = sim->xyz_fc[(size_t)sim->face_geo_off[f] * d + q + (size_t)n_fc * a];
	if ((rc = upload(st, &g.vol_face, vf.data(), vf.size()))) return rc;
	if ((rc = upload(st, &g.face_lf, flf.data(), flf.size()))) return rc;
	if ((rc = upload(st, &g.nc, sim->nc_fc, (size_t)n_face * n_fc))) return rc;
	if ((rc = upload(st, &g.nc_inv, ncinv.data(), ncinv.size()))) return rc;
	if ((rc = upload(st, &g.nrm, sim->normals_fc, (size_t)n_face * n_fc * d))) return rc;
	if ((rc = upload(st, &g.jf, sim->jacobian_det_fc, (size_t)n_face * n_fc))) return rc;
	if ((rc = upload(st, &g.xyz, xyz.data(), xyz.size()))) return rc;
	if ((rc = upload(st, &g.bc, bc.data(), bc.size()))) return rc;
	if ((rc = upload(st, &g.bface, bfaces.empty() ? nullptr : bfaces.data(), bfaces.size()))) return rc;
	if ((rc = ensure_buffers<double>(c, st))) return rc;
	if (d == 2 && nv == 4) rc = configure<double, 2, 4>(st);
	else if (d == 3 && nv == 5) rc = configure<double, 3, 5>(st);
	else if (d == 2 && nv == 1) rc = configure<double, 2, 1>(st);
	else if (d == 3 && nv == 1) rc = configure<double, 3, 1>(st);
	else rc = DPG_ERR_UNSUPPORTED;
	return rc;
}

} // namespace dpg
