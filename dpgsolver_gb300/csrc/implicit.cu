// Implicit path: matrix-free Newton-GMRES with pseudo-transient continuation, on the GPU.
//
// Follows solve_implicit / implicit_step (solve_implicit.c:95-110, 232-256): at each Newton step the system
//     (I / dtau - dF/du) du = F(u),      F(u) = m_inv * rhs(u)  (the residual of dpg_gpu_compute_rhs)
// is solved and u += du, until ||F||_inf < tol (the reference's exit rule max_rhs < exit_tol_i).  The reference
// assembles the full Jacobian into a PETSc matrix and adds -M/dt on the diagonal (compute_CFL_ramping,
// dg/solve_dg.c:223-248); here the same system, left-scaled by m_inv, is solved matrix-free:
//   - Jacobian-vector products are finite differences of the residual kernels (the same kernels as the explicit
//     path, in the context's precision mode);
//   - GMRES(m) with right preconditioning and classical Gram-Schmidt with one re-orthogonalisation; the Krylov
//     residual decides convergence;
//   - preconditioners: none, block-Jacobi (the element-diagonal blocks of I/dtau - dF/du assembled by
//     finite-difference probing over an element colouring in which no two face neighbours share a colour, then
//     factorised by a batched LU with partial pivoting), the learned block inverse (mlp.cu), or block ILU(0) in
//     its diagonal form (below: the diagonal and face-neighbour blocks, probed over a distance-2 colouring, with
//     level-scheduled factorisation and triangular solves) -- the GPU counterpart of the reference's default
//     PETSc method, GMRES(60) + ILU(1) with rtol 1e-4 (external/petsc/options_files/petsc_options_gmres_default.txt);
//   - dtau follows switched evolution relaxation: dtau_k = dtau_0 * ||F_0|| / ||F_k||.
// All vectors stay on the device; reductions are two-pass and deterministic.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "dpg_gpu_internal.cuh"

namespace dpg {

// ------------------------------------------------------------------------------------------------------------
// vector kernels
// ------------------------------------------------------------------------------------------------------------
constexpr int kRedBlocks = 304;   // 2 x 152 SMs
constexpr int kRedThreads = 256;

__global__ void k_axpby(int64_t n, double a, const double* __restrict__ x, double b, double* __restrict__ y)
{
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
		y[i] = a * x[i] + b * y[i];
}

__global__ void k_lincomb3(int64_t n, double a, const double* __restrict__ x, double b, const double* __restrict__ y,
                           double* __restrict__ z)
{
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
		z[i] = a * x[i] + b * y[i];
}

// partial[k][block] = sum_i V_k[i] * w[i] for k < nv; V_k = V + k * ld.  Vectors in chunks of 8 with their partial
// sums in registers (w[i] is re-read once per chunk, from L1/L2); per chunk one warp-shuffle and shared-memory
// reduction per vector.
constexpr int kDotChunk = 8;
__global__ void __launch_bounds__(kRedThreads) k_multidot_partial(int64_t n, int nv, const double* __restrict__ V, int64_t ld,
                                                                  const double* __restrict__ w, double* __restrict__ partial)
{
	__shared__ double red[kRedThreads / 32][kDotChunk];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	for (int k0 = 0; k0 < nv; k0 += kDotChunk) {
		double acc[kDotChunk];
#pragma unroll
		for (int k = 0; k < kDotChunk; ++k) acc[k] = 0.0;
		if (k0 + kDotChunk <= nv) {
			for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
				const double wi = w[i];
#pragma unroll
				for (int k = 0; k < kDotChunk; ++k) acc[k] += V[(k0 + k) * ld + i] * wi;
			}
		} else {
			for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
				const double wi = w[i];
#pragma unroll
				for (int k = 0; k < kDotChunk; ++k)
					if (k0 + k < nv) acc[k] += V[(k0 + k) * ld + i] * wi;
			}
		}
#pragma unroll
		for (int k = 0; k < kDotChunk; ++k) {
			double v = acc[k];
			for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
			if (lane == 0) red[warp][k] = v;
		}
		__syncthreads();
		if (threadIdx.x < kDotChunk && k0 + (int)threadIdx.x < nv) {
			double s = 0.0;
			for (int wv = 0; wv < kRedThreads / 32; ++wv) s += red[wv][threadIdx.x];
			partial[(int64_t)(k0 + threadIdx.x) * gridDim.x + blockIdx.x] = s;
		}
		__syncthreads();
	}
}

__global__ void k_reduce_partials(int nv, int nparts, const double* __restrict__ partial, double* __restrict__ out)
{
	const int k = blockIdx.x;
	if (k >= nv) return;
	__shared__ double red[32];
	double s = 0.0;
	for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += partial[(int64_t)k * nparts + i];
	for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
	if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
	__syncthreads();
	if (threadIdx.x == 0) {
		double t = 0.0;
		for (int i = 0; i < (int)(blockDim.x / 32); ++i) t += red[i];
		out[k] = t;
	}
}

// w -= sum_k V_k h_k   (h on the device)
__global__ void k_sub_combination(int64_t n, int nv, const double* __restrict__ V, int64_t ld,
                                  const double* __restrict__ h, double* __restrict__ w)
{
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		double s = 0.0;
		for (int k = 0; k < nv; ++k) s += V[k * ld + i] * h[k];
		w[i] -= s;
	}
}

// Arnoldi column j on the device: h[i] += h2[i] (the two Gram-Schmidt passes) and h[j+1] = ||w|| from h2[j+1] = w.w
__global__ void k_column_finish(int j, double* __restrict__ h, const double* __restrict__ h2)
{
	for (int i = threadIdx.x; i <= j; i += blockDim.x) h[i] += h2[i];
	if (threadIdx.x == 0) h[j + 1] = sqrt(fmax(h2[j + 1], 0.0));
}

// w /= *s when *s > 0 (the norm stays on the device)
__global__ void k_scale_inv(int64_t n, double* __restrict__ w, const double* __restrict__ s)
{
	const double v = *s;
	if (!(v > 0.0)) return;
	const double inv = 1.0 / v;
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) w[i] *= inv;
}

// x += sum_k Z_k y_k
__global__ void k_add_combination(int64_t n, int nv, const double* __restrict__ Z, int64_t ld,
                                  const double* __restrict__ y, double* __restrict__ x)
{
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		double s = 0.0;
		for (int k = 0; k < nv; ++k) s += Z[k * ld + i] * y[k];
		x[i] += s;
	}
}

__global__ void k_absmax_partial(int64_t n, const double* __restrict__ x, double* __restrict__ partial)
{
	__shared__ double red[32];
	double m = 0.0;
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const double v = fabs(x[i]);
		m = (v > m || isnan(v)) ? v : m;
	}
	for (int o = 16; o > 0; o >>= 1) {
		const double v = __shfl_xor_sync(0xffffffffu, m, o);
		m = (v > m || isnan(v)) ? v : m;
	}
	if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
	__syncthreads();
	if (threadIdx.x == 0) {
		double t = 0.0;
		for (int i = 0; i < (int)(blockDim.x / 32); ++i) t = (red[i] > t || isnan(red[i])) ? red[i] : t;
		partial[blockIdx.x] = t;
	}
}

// ------------------------------------------------------------------------------------------------------------
// block-Jacobi: probing, LU, solve
// ------------------------------------------------------------------------------------------------------------
// u_dst = u_src with eps added to local dof j of every element of colour `col`
__global__ void k_perturb(int n_vol, int nb, const double* __restrict__ u_src, double* __restrict__ u_dst,
                          const int* __restrict__ colour, int col, int j, double eps)
{
	const int64_t n = (int64_t)n_vol * nb;
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const int e = (int)(i / nb), k = (int)(i - (int64_t)e * nb);
		u_dst[i] = u_src[i] + ((k == j && colour[e] == col) ? eps : 0.0);
	}
}

// B_e[k][j] = shift_e * delta_kj - (F1_e[k] - F0_e[k]) / eps for the elements of colour `col` (shift_e = 1/dtau_e)
__global__ void k_extract_column(int n_vol, int nb, const double* __restrict__ F1, const double* __restrict__ F0,
                                 const int* __restrict__ colour, int col, int j, double inv_eps,
                                 const double* __restrict__ shift, double* __restrict__ blocks)
{
	const int64_t n = (int64_t)n_vol * nb;
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const int e = (int)(i / nb), k = (int)(i - (int64_t)e * nb);
		if (colour[e] != col) continue;
		blocks[((int64_t)e * nb + k) * nb + j] = (k == j ? shift[e] : 0.0) - (F1[i] - F0[i]) * inv_eps;
	}
}

// every element's 1/dtau_e: one value for all
__global__ void k_fill(int n, double v, double* __restrict__ out)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = v;
}

// 1/dtau_e of the reference's CFL ramping (compute_dt_cfl_constrained, dg/solve_dg.c:284-318): one warp per
// element; lambda_e = the largest |V| + c over the element's Bezier coefficients ccSB0 u read as conservative
// states (compute_max_wavespeed), |b| for advection; dtau_e = cfl min(h_e / lambda_e, h_e^2 / mu).
__global__ void k_pseudo_dt(int n_vol, int n_s, int nv, const double* __restrict__ u, const double* __restrict__ bez,
                            const double* __restrict__ h, double adv_speed, double mu, double cfl,
                            double* __restrict__ inv_dtau)
{
	const int e = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
	if (e >= n_vol) return;
	const int d = nv - 2;
	double lam = (nv == 1) ? adv_speed : 0.0;
	if (nv > 1)
		for (int i = lane; i < n_s; i += 32) {
			double b[5] = {0, 0, 0, 0, 0};
			for (int var = 0; var < nv; ++var) {
				double acc = 0.0;
				for (int j = 0; j < n_s; ++j) acc += bez[(int64_t)i * n_s + j] * u[(int64_t)e * n_s * nv + j + (int64_t)n_s * var];
				b[var] = acc;
			}
			if (!(b[0] > 0.0)) continue;
			double V2 = 0.0;
			for (int a = 0; a < d; ++a) V2 += (b[1 + a] / b[0]) * (b[1 + a] / b[0]);
			const double p = 0.4 * (b[d + 1] - 0.5 * b[0] * V2);
			lam = fmax(lam, sqrt(V2) + sqrt(fmax(1.4 * p / b[0], 0.0)));
		}
	for (int o = 16; o > 0; o >>= 1) lam = fmax(lam, __shfl_xor_sync(0xffffffffu, lam, o));
	if (lane == 0) {
		const double he = h[e];
		double dt = (lam > 0.0) ? he / lam : 1e300;
		if (mu > 0.0) dt = fmin(dt, he * he / mu);
		inv_dtau[e] = 1.0 / (cfl * dt);
	}
}

// out = shift_e z - J z  (J z given), per element shift_e = 1/dtau_e
__global__ void k_shift_minus(int64_t n, int nb, const double* __restrict__ shift, const double* __restrict__ z,
                              const double* __restrict__ jz, double* __restrict__ out)
{
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
		out[i] = shift[i / nb] * z[i] - jz[i];
}

// out = shift_e z - (F1 - F0) / eps
__global__ void k_shift_minus_fd(int64_t n, int nb, const double* __restrict__ shift, const double* __restrict__ z,
                                 const double* __restrict__ F1, const double* __restrict__ F0, double inv_eps,
                                 double* __restrict__ out)
{
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
		out[i] = shift[i / nb] * z[i] - (F1[i] - F0[i]) * inv_eps;
}

// partial[block] = sum over its elements of max_k sum_j |B_e[k][j] - shift_e delta_kj| (the inf-norm of -dF/du_ee)
__global__ void k_block_norm_partial(int n_vol, int nb, const double* __restrict__ blocks,
                                     const double* __restrict__ shift, double* __restrict__ partial)
{
	__shared__ double red[32];
	double acc = 0.0;
	for (int e = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); e < n_vol; e += gridDim.x * (blockDim.x / 32)) {
		double mx = 0.0;
		for (int k = threadIdx.x & 31; k < nb; k += 32) {
			double sr = 0.0;
			for (int j = 0; j < nb; ++j) sr += fabs(blocks[((int64_t)e * nb + k) * nb + j] - (k == j ? shift[e] : 0.0));
			mx = fmax(mx, sr);
		}
		for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
		acc += ((threadIdx.x & 31) == 0) ? mx : 0.0;
	}
	for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
	if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
	__syncthreads();
	if (threadIdx.x == 0) {
		double t = 0.0;
		for (int i = 0; i < (int)(blockDim.x / 32); ++i) t += red[i];
		partial[blockIdx.x] = t;
	}
}

// In-place LU with partial pivoting of one nb x nb block per thread block (nb <= 128), row-major.
__global__ void k_lu_batched(int nb, double* __restrict__ blocks, int* __restrict__ piv, int* __restrict__ info)
{
	extern __shared__ double a[];
	__shared__ int s_p;
	__shared__ double s_pivval;
	const int e = blockIdx.x;
	double* g = blocks + (int64_t)e * nb * nb;
	for (int i = threadIdx.x; i < nb * nb; i += blockDim.x) a[i] = g[i];
	__syncthreads();
	for (int k = 0; k < nb; ++k) {
		if (threadIdx.x == 0) {
			int p = k;
			double best = fabs(a[k * nb + k]);
			for (int i = k + 1; i < nb; ++i)
				if (fabs(a[i * nb + k]) > best) { best = fabs(a[i * nb + k]); p = i; }
			s_p = p;
			s_pivval = best;
			piv[(int64_t)e * nb + k] = p;
			if (best == 0.0) atomicExch(info, e + 1);
		}
		__syncthreads();
		const int p = s_p;
		if (p != k)
			for (int j = threadIdx.x; j < nb; j += blockDim.x) {
				const double t = a[k * nb + j]; a[k * nb + j] = a[p * nb + j]; a[p * nb + j] = t;
			}
		__syncthreads();
		if (s_pivval != 0.0) {
			const double inv = 1.0 / a[k * nb + k];
			for (int i = k + 1 + threadIdx.x; i < nb; i += blockDim.x) a[i * nb + k] *= inv;
			__syncthreads();
			const int rem = nb - k - 1;
			for (int t = threadIdx.x; t < rem * rem; t += blockDim.x) {
				const int i = k + 1 + t / rem, j = k + 1 + t % rem;
				a[i * nb + j] -= a[i * nb + k] * a[k * nb + j];
			}
		}
		__syncthreads();
	}
	for (int i = threadIdx.x; i < nb * nb; i += blockDim.x) g[i] = a[i];
}

// z_e = (LU_e)^-1 r_e, one warp per element
__global__ void k_lu_solve(int n_vol, int nb, const double* __restrict__ lu, const int* __restrict__ piv,
                           const double* __restrict__ r, double* __restrict__ z)
{
	const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
	if (warp >= n_vol) return;
	extern __shared__ double sh[];
	double* x = sh + (threadIdx.x >> 5) * nb;
	const double* a = lu + (int64_t)warp * nb * nb;
	for (int i = lane; i < nb; i += 32) x[i] = r[(int64_t)warp * nb + i];
	__syncwarp();
	if (lane == 0)
		for (int k = 0; k < nb; ++k) {
			const int p = piv[(int64_t)warp * nb + k];
			if (p != k) { const double t = x[k]; x[k] = x[p]; x[p] = t; }
		}
	__syncwarp();
	for (int i = 0; i < nb; ++i) {          // L y = P r (unit diagonal)
		double s = 0.0;
		for (int j = lane; j < i; j += 32) s += a[i * nb + j] * x[j];
		for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
		if (lane == 0) x[i] -= s;
		__syncwarp();
	}
	for (int i = nb - 1; i >= 0; --i) {     // U z = y
		double s = 0.0;
		for (int j = i + 1 + lane; j < nb; j += 32) s += a[i * nb + j] * x[j];
		for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
		if (lane == 0) x[i] = (x[i] - s) / a[i * nb + i];
		__syncwarp();
	}
	for (int i = lane; i < nb; i += 32) z[(int64_t)warp * nb + i] = x[i];
}

// z_e = P_e r_e / (shift_e + rho) with a dense per-element matrix (learned inverse), one warp per element
__global__ void k_block_apply(int n_vol, int nb, const float* __restrict__ P, const double* __restrict__ r,
                              double* __restrict__ z, const double* __restrict__ shift, double rho)
{
	const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
	if (warp >= n_vol) return;
	const float* a = P + (int64_t)warp * nb * nb;
	const double* x = r + (int64_t)warp * nb;
	const double scale = 1.0 / (shift[warp] + rho);
	for (int i = lane; i < nb; i += 32) {
		double s = 0.0;
		for (int j = 0; j < nb; ++j) s += (double)a[i * nb + j] * x[j];
		z[(int64_t)warp * nb + i] = scale * s;
	}
}

// ------------------------------------------------------------------------------------------------------------
// block ILU(0), diagonal form:  M = (D + L) D^-1 (D + U)
//   L, U the strictly lower / upper face-neighbour blocks of A = I/dtau - dF/du in the chosen element order (rank),
//   D_i = A_ii - sum_{k lower neighbour of i} A_ik D_k^-1 A_ki, so that M and A have the same diagonal and
//   neighbour blocks; on meshes whose face graph has no triangles (every mesh of this path except periodic
//   directions three elements wide) this is block ILU(0).  D_i^-1 is kept explicitly (Gauss-Jordan with partial
//   pivoting); each element's blocks of one level are independent, so the factorisation and both triangular
//   solves run level by level, one thread block per element.
// ------------------------------------------------------------------------------------------------------------
// the blocks of column j of every element of distance-2 colour `col`: the diagonal block of those elements and
// the neighbour block A_ik (k of colour col) of every other element i (at most one such k per i)
__global__ void k_extract_ilu(int n_vol, int nb, int n_fl, const double* __restrict__ F1, const double* __restrict__ F0,
                              const int* __restrict__ colour, const int* __restrict__ nbr, int col, int j,
                              double inv_eps, const double* __restrict__ shift, double* __restrict__ diag,
                              double* __restrict__ offd)
{
	const int64_t n = (int64_t)n_vol * nb;
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
		const int e = (int)(i / nb), k = (int)(i - (int64_t)e * nb);
		const double dF = (F1[i] - F0[i]) * inv_eps;
		if (colour[e] == col) {
			diag[((int64_t)e * nb + k) * nb + j] = (k == j ? shift[e] : 0.0) - dF;
			continue;
		}
		for (int s = 0; s < n_fl; ++s) {
			const int o = nbr[e * n_fl + s];
			if (o >= 0 && colour[o] == col) offd[(((int64_t)e * n_fl + s) * nb + k) * nb + j] = -dF;
		}
	}
}

// in-place inverse of the nb x nb row-major matrix a in shared memory (Gauss-Jordan, partial pivoting; the row
// exchanges are undone as column exchanges at the end); returns false for a zero pivot
__device__ bool gj_invert_shared(int nb, double* a, int* perm)
{
	__shared__ int s_p;
	__shared__ double s_best;
	for (int k = 0; k < nb; ++k) {
		if (threadIdx.x < 32) {
			int p = k;
			double best = -1.0;
			for (int i = k + threadIdx.x; i < nb; i += 32) {
				const double v = fabs(a[i * nb + k]);
				if (v > best) { best = v; p = i; }
			}
			for (int o = 16; o > 0; o >>= 1) {
				const double bv = __shfl_xor_sync(0xffffffffu, best, o);
				const int bp = __shfl_xor_sync(0xffffffffu, p, o);
				if (bv > best || (bv == best && bp < p)) { best = bv; p = bp; }
			}
			if (threadIdx.x == 0) { s_p = p; s_best = best; perm[k] = p; }
		}
		__syncthreads();
		if (!(s_best > 0.0)) return false;
		const int p = s_p;
		if (p != k)
			for (int c = threadIdx.x; c < nb; c += blockDim.x) {
				const double t = a[k * nb + c]; a[k * nb + c] = a[p * nb + c]; a[p * nb + c] = t;
			}
		__syncthreads();
		const double inv = 1.0 / a[k * nb + k];
		__syncthreads();
		for (int c = threadIdx.x; c < nb; c += blockDim.x) a[k * nb + c] = (c == k ? inv : a[k * nb + c] * inv);
		__syncthreads();
		for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
			const int i = t / nb, c = t - i * nb;
			if (i == k) continue;
			const double f = a[i * nb + k];
			if (c == k) continue;
			a[i * nb + c] -= f * a[k * nb + c];
		}
		__syncthreads();
		for (int i = threadIdx.x; i < nb; i += blockDim.x)
			if (i != k) a[i * nb + k] = -a[i * nb + k] * inv;
		__syncthreads();
	}
	for (int k = nb - 1; k >= 0; --k) {
		const int p = perm[k];
		if (p != k)
			for (int i = threadIdx.x; i < nb; i += blockDim.x) {
				const double t = a[i * nb + k]; a[i * nb + k] = a[i * nb + p]; a[i * nb + p] = t;
			}
		__syncthreads();
	}
	return true;
}

// slot of neighbour `want` in the list of element e, -1 if absent
__device__ __forceinline__ int nbr_slot(const int* __restrict__ nbr, int n_fl, int e, int want)
{
	for (int s = 0; s < n_fl; ++s) if (nbr[e * n_fl + s] == want) return s;
	return -1;
}

// D_i = A_ii - sum_{k lower} A_ik D_k^-1 A_ki and its inverse, for the elements of one level; diag holds A_ii on
// entry and D_i^-1 on exit (elements of earlier levels already hold D_k^-1)
__global__ void k_ilu_factor_level(const int* __restrict__ elems, int nb, int n_fl, const int* __restrict__ nbr,
                                   const int* __restrict__ rank, double* __restrict__ diag,
                                   const double* __restrict__ offd, int* __restrict__ info)
{
	extern __shared__ double sh[];
	double* D = sh;
	double* T = sh + nb * nb;
	int* perm = (int*)(T + nb * nb);
	const int i = elems[blockIdx.x];
	double* Di = diag + (int64_t)i * nb * nb;
	for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) D[t] = Di[t];
	__syncthreads();
	for (int s = 0; s < n_fl; ++s) {
		const int k = nbr[i * n_fl + s];
		if (k < 0 || rank[k] >= rank[i]) continue;
		const int sk = nbr_slot(nbr, n_fl, k, i);
		if (sk < 0) continue;
		const double* Dk = diag + (int64_t)k * nb * nb;                           // D_k^-1
		const double* Aki = offd + ((int64_t)k * n_fl + sk) * nb * nb;
		const double* Aik = offd + ((int64_t)i * n_fl + s) * nb * nb;
		for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {                   // T = D_k^-1 A_ki
			const int r = t / nb, c = t - r * nb;
			double acc = 0.0;
			for (int q = 0; q < nb; ++q) acc += Dk[r * nb + q] * Aki[q * nb + c];
			T[t] = acc;
		}
		__syncthreads();
		for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {                   // D -= A_ik T
			const int r = t / nb, c = t - r * nb;
			double acc = 0.0;
			for (int q = 0; q < nb; ++q) acc += Aik[r * nb + q] * T[q * nb + c];
			D[t] -= acc;
		}
		__syncthreads();
	}
	const bool ok = gj_invert_shared(nb, D, perm);
	if (!ok) {
		if (threadIdx.x == 0) atomicExch(info, i + 1);
		return;
	}
	for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) Di[t] = D[t];
}

// Triangular sweeps, one level, one thread block (kIluSweepThreads = 8 warps) per element.  Warp w owns the rows
// w, w + 8, ... (at most kIluRows of them) and lane l the columns l, l + 32, ... (at most kIluCols); the vector's
// entries a lane needs are loaded once into registers, and the block rows of all its rows are loaded before any
// sum is reduced, so a warp has all its loads in flight at once instead of one row after another.
constexpr int kIluSweepThreads = 256;
constexpr int kIluRows = 14;   // ceil(112 / 8)
constexpr int kIluCols = 4;    // ceil(112 / 32)

__device__ __forceinline__ double warp_sum(double v)
{
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
	return v;
}

// acc[t] += sum_c M[(warp + 8 t) * nb + c] x[c] over this lane's columns; NB > 0 fixes nb at compile time (no
// predicated padding rows or columns), NB = 0 takes it at run time (nb <= 112)
template <int NB>
__device__ __forceinline__ void ilu_rows_times(const double* __restrict__ M, const double* __restrict__ x, int nb_rt,
                                               int warp, int lane, double (&acc)[kIluRows])
{
	const int nb = NB > 0 ? NB : nb_rt;
	constexpr int R = NB > 0 ? (NB + 7) / 8 : kIluRows;
	constexpr int CC = NB > 0 ? (NB + 31) / 32 : kIluCols;
	double xv[CC];
#pragma unroll
	for (int j = 0; j < CC; ++j) {
		const int c = lane + 32 * j;
		xv[j] = (c < nb) ? x[c] : 0.0;
	}
#pragma unroll
	for (int t = 0; t < R; ++t) {
		const int row = warp + 8 * t;
		if (row < nb) {
#pragma unroll
			for (int j = 0; j < CC; ++j) {
				const int c = lane + 32 * j;
				if (c < nb) acc[t] += M[(int64_t)row * nb + c] * xv[j];
			}
		}
	}
}

// forward sweep: w_i = D_i^-1 (r_i - sum_{k lower} A_ik w_k)
template <int NB>
__global__ void __launch_bounds__(kIluSweepThreads) k_ilu_forward_level(const int* __restrict__ elems, int nb_rt, int n_fl,
                                                                        const int* __restrict__ nbr, const int* __restrict__ rank,
                                                                        const double* __restrict__ dinv, const double* __restrict__ offd,
                                                                        const double* __restrict__ r, double* __restrict__ w)
{
	extern __shared__ double y[];
	const int nb = NB > 0 ? NB : nb_rt;
	constexpr int R = NB > 0 ? (NB + 7) / 8 : kIluRows;
	const int i = elems[blockIdx.x];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	double acc[kIluRows];
#pragma unroll
	for (int t = 0; t < kIluRows; ++t) acc[t] = 0.0;
	for (int s = 0; s < n_fl; ++s) {
		const int k = nbr[i * n_fl + s];
		if (k < 0 || rank[k] >= rank[i]) continue;
		ilu_rows_times<NB>(offd + ((int64_t)i * n_fl + s) * nb * nb, w + (int64_t)k * nb, nb, warp, lane, acc);
	}
#pragma unroll
	for (int t = 0; t < R; ++t) {
		const int row = warp + 8 * t;
		const double v = warp_sum(acc[t]);
		if (lane == 0 && row < nb) y[row] = r[(int64_t)i * nb + row] - v;
	}
	__syncthreads();
#pragma unroll
	for (int t = 0; t < kIluRows; ++t) acc[t] = 0.0;
	ilu_rows_times<NB>(dinv + (int64_t)i * nb * nb, y, nb, warp, lane, acc);
#pragma unroll
	for (int t = 0; t < R; ++t) {
		const int row = warp + 8 * t;
		const double v = warp_sum(acc[t]);
		if (lane == 0 && row < nb) w[(int64_t)i * nb + row] = v;
	}
}

// backward sweep (levels in reverse): z_i = w_i - D_i^-1 sum_{j upper} A_ij z_j
template <int NB>
__global__ void __launch_bounds__(kIluSweepThreads) k_ilu_backward_level(const int* __restrict__ elems, int nb_rt, int n_fl,
                                                                         const int* __restrict__ nbr, const int* __restrict__ rank,
                                                                         const double* __restrict__ dinv, const double* __restrict__ offd,
                                                                         const double* __restrict__ w, double* __restrict__ z)
{
	extern __shared__ double y[];
	const int nb = NB > 0 ? NB : nb_rt;
	constexpr int R = NB > 0 ? (NB + 7) / 8 : kIluRows;
	const int i = elems[blockIdx.x];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	double acc[kIluRows];
#pragma unroll
	for (int t = 0; t < kIluRows; ++t) acc[t] = 0.0;
	for (int s = 0; s < n_fl; ++s) {
		const int j = nbr[i * n_fl + s];
		if (j < 0 || rank[j] <= rank[i]) continue;
		ilu_rows_times<NB>(offd + ((int64_t)i * n_fl + s) * nb * nb, z + (int64_t)j * nb, nb, warp, lane, acc);
	}
#pragma unroll
	for (int t = 0; t < R; ++t) {
		const int row = warp + 8 * t;
		const double v = warp_sum(acc[t]);
		if (lane == 0 && row < nb) y[row] = v;
	}
	__syncthreads();
#pragma unroll
	for (int t = 0; t < kIluRows; ++t) acc[t] = 0.0;
	ilu_rows_times<NB>(dinv + (int64_t)i * nb * nb, y, nb, warp, lane, acc);
#pragma unroll
	for (int t = 0; t < R; ++t) {
		const int row = warp + 8 * t;
		const double v = warp_sum(acc[t]);
		if (lane == 0 && row < nb) z[(int64_t)i * nb + row] = w[(int64_t)i * nb + row] - v;
	}
}

// One level of either sweep for blocks of a size fixed at compile time, with its operands staged in shared memory:
// every thread first issues asynchronous 16-byte copies (cp.async, completed by cp.async.wait_all, a wait on the
// thread's own copies) of D_i^-1 and of the blocks A_is of the neighbours the sweep uses, and plain loads of those
// neighbours' vector entries and of b_i, so a level costs one memory round trip instead of one per neighbour and a
// dependent one for D_i^-1.  The sums run in the order of the register kernels above (neighbours, then columns
// lane, lane + 32, ..., per row), so the results are the same bits.
//   FWD: x_i = D_i^-1 (b_i - sum_{k lower} A_ik x_k)    (b = r, x = w)
//   BWD: x_i = b_i - D_i^-1 sum_{j upper} A_ij x_j      (b = w, x = z)
constexpr int kIluStagedThreads = 512;
constexpr int kIluStagedMaxFl = 5;

__device__ __forceinline__ void ilu_stage_block(double* dst, const double* __restrict__ src, int n_chunks)
{
	for (int q = threadIdx.x; q < n_chunks; q += blockDim.x)
		asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst + 2 * q)),
		             "l"(src + 2 * q)
		             : "memory");
}

template <int NB, bool FWD>
__global__ void __launch_bounds__(kIluStagedThreads) k_ilu_level_staged(const int* __restrict__ elems, int n_fl,
                                                                        const int* __restrict__ nbr, const int* __restrict__ rank,
                                                                        const double* __restrict__ dinv, const double* __restrict__ offd,
                                                                        const double* __restrict__ b, double* __restrict__ x)
{
	extern __shared__ __align__(16) double sm[];   // [1 + used][NB][NB]: D_i^-1, then the used A_is in slot order
	__shared__ double xs[kIluStagedMaxFl][NB];
	__shared__ double y[NB];
	__shared__ int used[kIluStagedMaxFl], n_used;
	constexpr int NW = kIluStagedThreads / 32, R = (NB + NW - 1) / NW, CC = (NB + 31) / 32;
	constexpr int kChunks = NB * NB / 2;   // 16-byte copies per block
	static_assert(NB % 2 == 0, "blocks are copied in 16-byte pieces");
	const int i = elems[blockIdx.x];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	ilu_stage_block(sm, dinv + (int64_t)i * NB * NB, kChunks);
	if (threadIdx.x == 0) {
		const int ri = rank[i];
		int q = 0;
		for (int s = 0; s < n_fl; ++s) {
			const int k = nbr[i * n_fl + s];
			if (k >= 0 && (FWD ? rank[k] < ri : rank[k] > ri)) used[q++] = s;
		}
		n_used = q;
	}
	__syncthreads();
	const int nu = n_used;
	for (int q = 0; q < nu; ++q)
		ilu_stage_block(sm + (size_t)(q + 1) * NB * NB, offd + ((int64_t)i * n_fl + used[q]) * NB * NB, kChunks);
	asm volatile("cp.async.commit_group;" ::: "memory");
	for (int t = threadIdx.x; t < nu * NB; t += blockDim.x) {
		const int q = t / NB, c = t - q * NB;
		xs[q][c] = x[(int64_t)nbr[i * n_fl + used[q]] * NB + c];
	}
	double bv[R];
#pragma unroll
	for (int t = 0; t < R; ++t) {
		const int row = warp + NW * t;
		bv[t] = row < NB ? b[(int64_t)i * NB + row] : 0.0;
	}
	asm volatile("cp.async.wait_all;" ::: "memory");
	__syncthreads();
	double acc[R];
#pragma unroll
	for (int t = 0; t < R; ++t) acc[t] = 0.0;
	for (int q = 0; q < nu; ++q) {
		const double* M = sm + (size_t)(q + 1) * NB * NB;
#pragma unroll
		for (int t = 0; t < R; ++t) {
			const int row = warp + NW * t;
			if (row < NB) {
#pragma unroll
				for (int j = 0; j < CC; ++j) {
					const int c = lane + 32 * j;
					if (c < NB) acc[t] += M[row * NB + c] * xs[q][c];
				}
			}
		}
	}
#pragma unroll
	for (int t = 0; t < R; ++t) {
		const int row = warp + NW * t;
		const double v = warp_sum(acc[t]);
		if (lane == 0 && row < NB) y[row] = FWD ? bv[t] - v : v;
	}
	__syncthreads();
	double yv[CC];
#pragma unroll
	for (int j = 0; j < CC; ++j) yv[j] = (lane + 32 * j < NB) ? y[lane + 32 * j] : 0.0;
#pragma unroll
	for (int t = 0; t < R; ++t) {
		const int row = warp + NW * t;
		double a = 0.0;
		if (row < NB) {
#pragma unroll
			for (int j = 0; j < CC; ++j)
				if (lane + 32 * j < NB) a += sm[row * NB + lane + 32 * j] * yv[j];
		}
		const double v = warp_sum(a);
		if (lane == 0 && row < NB) x[(int64_t)i * NB + row] = FWD ? v : bv[t] - v;
	}
}

// ------------------------------------------------------------------------------------------------------------
// host orchestration
// ------------------------------------------------------------------------------------------------------------
struct Implicit {
	int nb = 0, m = 0, n_colours = 0;
	int64_t n = 0;
	double *u = nullptr, *F0 = nullptr, *F1 = nullptr, *up = nullptr, *du = nullptr, *w = nullptr;
	double *V = nullptr, *Z = nullptr, *h = nullptr, *h2 = nullptr, *partial = nullptr;
	double* hcol_host = nullptr;  // pinned [m + 2]: the Arnoldi column, one copy per iteration
	double *blocks = nullptr;
	int *piv = nullptr, *colour = nullptr, *info = nullptr;
	float* P = nullptr;           // learned inverses [n_vol][nb][nb] (owned by the MLP state)
	double* forcing = nullptr;    // subtracted from F (nullptr: none)
	double rho = 0.0;             // mean inf-norm of the element blocks of dF/du (last assembly)
	double* forcing_buf = nullptr;
	double* zero = nullptr;       // [n] zeros (tangent probing)
	double* inv_dtau = nullptr;   // [n_vol] 1/dtau_e of the current Newton step
	bool blocks_valid = false;
	bool tangent = true;          // Jacobian products by the analytic linearisation (false: finite differences)
	// block ILU (built on first use)
	int ilu_order = -1;           // element order of the levels: DPG_ILU_ORDER_* (-1: not built)
	int ilu_parts = 0;            // subdomains of the factorisation (contiguous ranges of the element order)
	int n_colours2 = 0;           // distance-2 colouring: no two elements within two face steps share a colour
	int* colour2 = nullptr;       // [n_vol]
	int* nbr = nullptr;           // [n_vol][n_fl] distinct face neighbours (-1: none)
	int* rank = nullptr;          // [n_vol] position in the element order
	int* level_elems = nullptr;   // [n_vol] elements grouped by level
	std::vector<int> level_ptr;   // [n_levels + 1]
	double* offd = nullptr;       // [n_vol][n_fl][nb][nb] A_{i, nbr[i][s]}
	double* wbuf = nullptr;       // [n] forward-sweep result
	double* ilu_in = nullptr;     // [n] right-hand side of the sweeps' graph
	double* ilu_out = nullptr;    // [n] result of the sweeps' graph
	cudaGraphExec_t ilu_graph = nullptr;   // forward and backward sweeps over all levels (one launch)
	bool ilu_valid = false;
};

static int grid_for(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 4 * 152 * 8); }

static Implicit* implicit_state(dpg_gpu_ctx* c, int m)
{
	Implicit* im = (Implicit*)c->implicit;
	if (im && im->m >= m) return im;
	if (im) implicit_free(c);
	im = new Implicit();
	im->nb = c->g.n_s * c->n_var;
	im->m = m;
	im->n = c->n_dof;
	const int64_t n = im->n;
	bool ok = true;
	auto al = [&](void** p, size_t bytes) { if (cudaMalloc(p, bytes ? bytes : 1) != cudaSuccess) ok = false; };
	al((void**)&im->u, n * 8); al((void**)&im->F0, n * 8); al((void**)&im->F1, n * 8); al((void**)&im->up, n * 8);
	al((void**)&im->du, n * 8); al((void**)&im->w, n * 8);
	al((void**)&im->V, (size_t)(m + 1) * n * 8); al((void**)&im->Z, (size_t)m * n * 8);
	al((void**)&im->h, (size_t)(m + 2) * 8); al((void**)&im->h2, (size_t)(m + 2) * 8);
	al((void**)&im->partial, (size_t)(m + 2) * kRedBlocks * 8);
	if (cudaMallocHost((void**)&im->hcol_host, (size_t)(m + 2) * 8) != cudaSuccess) ok = false;
	al((void**)&im->blocks, (size_t)c->g.n_vol * im->nb * im->nb * 8);
	al((void**)&im->piv, (size_t)c->g.n_vol * im->nb * 4); al((void**)&im->info, 4);
	al((void**)&im->colour, (size_t)c->g.n_vol * 4);
	al((void**)&im->zero, n * 8);
	al((void**)&im->inv_dtau, (size_t)c->g.n_vol * 8);
	if (ok && cudaMemset(im->zero, 0, n * 8) != cudaSuccess) ok = false;
	c->implicit = im;
	if (!ok) { implicit_free(c); return nullptr; }
	// greedy element colouring: face neighbours get different colours
	std::vector<int> vf((size_t)c->g.n_vol * c->g.n_fl), col(c->g.n_vol, -1);
	cudaMemcpy(vf.data(), c->g.vol_face, vf.size() * 4, cudaMemcpyDeviceToHost);
	std::vector<std::vector<int>> face_vols(c->fc.n_face);
	for (int e = 0; e < c->g.n_vol; ++e)
		for (int lf = 0; lf < c->g.n_fl; ++lf) face_vols[vf[(size_t)e * c->g.n_fl + lf] >> 1].push_back(e);
	int nc = 0;
	for (int e = 0; e < c->g.n_vol; ++e) {
		std::vector<char> used(64, 0);
		for (int lf = 0; lf < c->g.n_fl; ++lf)
			for (int o : face_vols[vf[(size_t)e * c->g.n_fl + lf] >> 1])
				if (o != e && col[o] >= 0 && col[o] < 64) used[col[o]] = 1;
		int k = 0;
		while (used[k]) ++k;
		col[e] = k;
		nc = std::max(nc, k + 1);
	}
	im->n_colours = nc;
	cudaMemcpy(im->colour, col.data(), col.size() * 4, cudaMemcpyHostToDevice);
	return im;
}

void implicit_free(dpg_gpu_ctx* c)
{
	Implicit* im = (Implicit*)c->implicit;
	if (!im) return;
	void* ptrs[] = {im->u, im->F0, im->F1, im->up, im->du, im->w, im->V, im->Z, im->h, im->h2, im->partial,
	                im->blocks, im->piv, im->info, im->colour, im->forcing_buf, im->zero, im->colour2, im->nbr,
	                im->rank, im->level_elems, im->offd, im->wbuf, im->inv_dtau, im->ilu_in, im->ilu_out};
	if (im->ilu_graph) cudaGraphExecDestroy(im->ilu_graph);
	for (void* p : ptrs) if (p) cudaFree(p);
	if (im->hcol_host) cudaFreeHost(im->hcol_host);
	delete im;
	c->implicit = nullptr;
}

// F = m_inv * rhs(u) (- forcing) through the residual kernels of the context's precision mode.
static int residual(dpg_gpu_ctx* c, const double* u, double* F)
{
	double* sol0 = c->sol;
	double* rhs0 = c->rhs;
	c->sol = const_cast<double*>(u);
	c->rhs = F;
	int rc = enqueue_residual_raw(c, c->dmax + kMaxStages);
	c->sol = sol0;
	c->rhs = rhs0;
	Implicit* im = (Implicit*)c->implicit;
	if (!rc && im && im->forcing)
		k_axpby<<<grid_for(im->n), 256, 0, c->stream>>>(im->n, -1.0, im->forcing, 1.0, F);
	return rc;
}

static int absmax(dpg_gpu_ctx* c, Implicit* im, const double* x, double* out)
{
	k_absmax_partial<<<kRedBlocks, kRedThreads, 0, c->stream>>>(im->n, x, im->partial);
	k_absmax_partial<<<1, kRedThreads, 0, c->stream>>>(kRedBlocks, im->partial, im->h);
	if (cudaMemcpyAsync(out, im->h, 8, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess) return DPG_ERR_CUDA;
	if (cudaStreamSynchronize(c->stream) != cudaSuccess) return DPG_ERR_CUDA;
	return std::isfinite(*out) ? DPG_OK : DPG_ERR_NONFINITE;
}

// h[0..nv) = V[0..nv)^T w   (device result in im->h, copied to host_h)
static int multidot(dpg_gpu_ctx* c, Implicit* im, int nv, const double* V, const double* w, double* host_h)
{
	k_multidot_partial<<<kRedBlocks, kRedThreads, 0, c->stream>>>(im->n, nv, V, im->n, w, im->partial);
	k_reduce_partials<<<nv, 256, 0, c->stream>>>(nv, kRedBlocks, im->partial, im->h);
	if (cudaMemcpyAsync(host_h, im->h, 8 * nv, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess) return DPG_ERR_CUDA;
	if (cudaStreamSynchronize(c->stream) != cudaSuccess) return DPG_ERR_CUDA;
	return DPG_OK;
}

static int assemble_block_jacobi(dpg_gpu_ctx* c, Implicit* im, const double* F0)
{
	const int nb = im->nb, n_vol = c->g.n_vol;
	const double eps = 1e-7;
	int rc;
	// block column j of every element of one colour at once (no two face neighbours share a colour): the tangent
	// along e_j on those elements (exact), or a forward difference of the residual
	for (int col = 0; col < im->n_colours; ++col)
		for (int j = 0; j < nb; ++j) {
			if (im->tangent) {
				k_perturb<<<grid_for(im->n), 256, 0, c->stream>>>(n_vol, nb, im->zero, im->up, im->colour, col, j, 1.0);
				if ((rc = jvp_fp64(c, im->u, im->up, im->F1, c->trace_t, c->nnf_t))) return rc;
				k_extract_column<<<grid_for(im->n), 256, 0, c->stream>>>(n_vol, nb, im->F1, im->zero, im->colour, col, j,
				                                                          1.0, im->inv_dtau, im->blocks);
			} else {
				k_perturb<<<grid_for(im->n), 256, 0, c->stream>>>(n_vol, nb, im->u, im->up, im->colour, col, j, eps);
				if ((rc = residual(c, im->up, im->F1))) return rc;
				k_extract_column<<<grid_for(im->n), 256, 0, c->stream>>>(n_vol, nb, im->F1, F0, im->colour, col, j,
				                                                          1.0 / eps, im->inv_dtau, im->blocks);
			}
		}
	{
		k_block_norm_partial<<<kRedBlocks, kRedThreads, 0, c->stream>>>(n_vol, nb, im->blocks, im->inv_dtau, im->partial);
		std::vector<double> parts(kRedBlocks);
		if (cudaMemcpyAsync(parts.data(), im->partial, 8 * kRedBlocks, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess)
			return DPG_ERR_CUDA;
		if (cudaStreamSynchronize(c->stream) != cudaSuccess) return DPG_ERR_CUDA;
		double t = 0.0;
		for (double v : parts) t += v;
		im->rho = t / n_vol;
	}
	if (cudaMemsetAsync(im->info, 0, 4, c->stream) != cudaSuccess) return DPG_ERR_CUDA;
	const size_t smem = (size_t)nb * nb * 8;
	if (smem > 48 * 1024 && cudaFuncSetAttribute(k_lu_batched, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem))
		return DPG_ERR_CUDA;
	k_lu_batched<<<n_vol, 256, smem, c->stream>>>(nb, im->blocks, im->piv, im->info);
	int info = 0;
	cudaMemcpyAsync(&info, im->info, 4, cudaMemcpyDeviceToHost, c->stream);
	if (cudaStreamSynchronize(c->stream) != cudaSuccess) return DPG_ERR_CUDA;
	im->blocks_valid = (info == 0);
	return info == 0 ? DPG_OK : DPG_ERR_NONFINITE;
}

// ---- block ILU: structure (once per element order), assembly and factorisation (every Newton step), solve ----
constexpr int kIluMaxNb = 112;   // D and the product T in shared memory: 2 nb^2 doubles <= 200 KB

static bool ilu_staged(int nb, int n_fl) { return nb == 64 && n_fl <= kIluStagedMaxFl; }

static size_t ilu_staged_smem(int nb, int n_fl) { return (size_t)(1 + n_fl) * nb * nb * 8; }

static void enqueue_block_ilu_sweeps(dpg_gpu_ctx* c, Implicit* im, const double* r, double* z)
{
	const int nb = im->nb, n_fl = c->g.n_fl;
	const int n_levels = (int)im->level_ptr.size() - 1;
	const int threads = kIluSweepThreads;
	const bool staged = ilu_staged(nb, n_fl);
	const size_t smem_staged = ilu_staged_smem(nb, n_fl);
	for (int l = 0; l < n_levels; ++l) {
		const int cnt = im->level_ptr[l + 1] - im->level_ptr[l];
		if (cnt <= 0) continue;
		if (staged)
			k_ilu_level_staged<64, true><<<cnt, kIluStagedThreads, smem_staged, c->stream>>>(
			    im->level_elems + im->level_ptr[l], n_fl, im->nbr, im->rank, im->blocks, im->offd, r, im->wbuf);
		else if (nb == 64)
			k_ilu_forward_level<64><<<cnt, threads, (size_t)nb * 8, c->stream>>>(im->level_elems + im->level_ptr[l], nb, n_fl,
			                                                                     im->nbr, im->rank, im->blocks, im->offd, r,
			                                                                     im->wbuf);
		else
			k_ilu_forward_level<0><<<cnt, threads, (size_t)nb * 8, c->stream>>>(im->level_elems + im->level_ptr[l], nb, n_fl,
			                                                                    im->nbr, im->rank, im->blocks, im->offd, r,
			                                                                    im->wbuf);
	}
	for (int l = n_levels - 1; l >= 0; --l) {
		const int cnt = im->level_ptr[l + 1] - im->level_ptr[l];
		if (cnt <= 0) continue;
		if (staged)
			k_ilu_level_staged<64, false><<<cnt, kIluStagedThreads, smem_staged, c->stream>>>(
			    im->level_elems + im->level_ptr[l], n_fl, im->nbr, im->rank, im->blocks, im->offd, im->wbuf, z);
		else if (nb == 64)
			k_ilu_backward_level<64><<<cnt, threads, (size_t)nb * 8, c->stream>>>(im->level_elems + im->level_ptr[l], nb,
			                                                                      n_fl, im->nbr, im->rank, im->blocks,
			                                                                      im->offd, im->wbuf, z);
		else
			k_ilu_backward_level<0><<<cnt, threads, (size_t)nb * 8, c->stream>>>(im->level_elems + im->level_ptr[l], nb,
			                                                                     n_fl, im->nbr, im->rank, im->blocks,
			                                                                     im->offd, im->wbuf, z);
	}
}

static int ilu_build(dpg_gpu_ctx* c, Implicit* im, int order, int parts)
{
	if (parts < 1) parts = 1;
	if (im->ilu_order == order && im->ilu_parts == parts) return DPG_OK;
	const int n_vol = c->g.n_vol, n_fl = c->g.n_fl, nb = im->nb;
	if (nb > kIluMaxNb) return DPG_ERR_UNSUPPORTED;
	std::vector<int> vf((size_t)n_vol * n_fl);
	if (cudaMemcpy(vf.data(), c->g.vol_face, vf.size() * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return DPG_ERR_CUDA;
	std::vector<std::vector<int>> face_vols(c->fc.n_face);
	for (int e = 0; e < n_vol; ++e)
		for (int lf = 0; lf < n_fl; ++lf) face_vols[vf[(size_t)e * n_fl + lf] >> 1].push_back(e);
	// distinct face neighbours (a periodic direction one or two elements wide repeats a neighbour, or the element)
	std::vector<int> nbr((size_t)n_vol * n_fl, -1);
	for (int e = 0; e < n_vol; ++e) {
		int cnt = 0;
		for (int lf = 0; lf < n_fl; ++lf)
			for (int o : face_vols[vf[(size_t)e * n_fl + lf] >> 1]) {
				if (o == e) continue;
				bool seen = false;
				for (int q = 0; q < cnt; ++q) seen |= (nbr[(size_t)e * n_fl + q] == o);
				if (!seen) nbr[(size_t)e * n_fl + cnt++] = o;
			}
	}
	// distance-2 colouring (greedy, volume order)
	std::vector<int> col2(n_vol, -1);
	int nc2 = 0;
	for (int e = 0; e < n_vol; ++e) {
		std::vector<char> used(256, 0);
		for (int a = 0; a < n_fl; ++a) {
			const int o = nbr[(size_t)e * n_fl + a];
			if (o < 0) continue;
			if (col2[o] >= 0) used[col2[o]] = 1;
			for (int b = 0; b < n_fl; ++b) {
				const int q = nbr[(size_t)o * n_fl + b];
				if (q >= 0 && q != e && col2[q] >= 0) used[col2[q]] = 1;
			}
		}
		int k = 0;
		while (k < 255 && used[k]) ++k;
		col2[e] = k;
		nc2 = std::max(nc2, k + 1);
	}
	// element order and levels: an element's level is one more than the highest level of its lower neighbours
	std::vector<int> col1(n_vol);
	if (cudaMemcpy(col1.data(), im->colour, (size_t)n_vol * 4, cudaMemcpyDeviceToHost) != cudaSuccess) return DPG_ERR_CUDA;
	std::vector<int64_t> key(n_vol);
	for (int e = 0; e < n_vol; ++e) key[e] = (order == DPG_ILU_ORDER_COLOUR ? (int64_t)col1[e] * n_vol : 0) + e;
	std::vector<int> by_rank(n_vol), rank(n_vol), level(n_vol, 0);
	for (int e = 0; e < n_vol; ++e) by_rank[e] = e;
	std::sort(by_rank.begin(), by_rank.end(), [&](int a, int b) { return key[a] < key[b]; });
	for (int r = 0; r < n_vol; ++r) rank[by_rank[r]] = r;
	// subdomains: `parts` contiguous ranges of the element order, factorised independently (the couplings between
	// them are left out of L and U, as in a block-Jacobi method with ILU(0) inside each block); the probing colouring
	// above keeps every neighbour, so a left-out coupling cannot alias a kept one
	if (parts > 1)
		for (int e = 0; e < n_vol; ++e)
			for (int a = 0; a < n_fl; ++a) {
				int& o = nbr[(size_t)e * n_fl + a];
				if (o >= 0 && (int64_t)rank[o] * parts / n_vol != (int64_t)rank[e] * parts / n_vol) o = -1;
			}
	int n_levels = 0;
	for (int r = 0; r < n_vol; ++r) {
		const int e = by_rank[r];
		int lv = 0;
		for (int a = 0; a < n_fl; ++a) {
			const int o = nbr[(size_t)e * n_fl + a];
			if (o >= 0 && rank[o] < r) lv = std::max(lv, level[o] + 1);
		}
		level[e] = lv;
		n_levels = std::max(n_levels, lv + 1);
	}
	im->level_ptr.assign(n_levels + 1, 0);
	for (int e = 0; e < n_vol; ++e) ++im->level_ptr[level[e] + 1];
	for (int l = 0; l < n_levels; ++l) im->level_ptr[l + 1] += im->level_ptr[l];
	std::vector<int> elems(n_vol), fill(im->level_ptr.begin(), im->level_ptr.end() - 1);
	for (int r = 0; r < n_vol; ++r) { const int e = by_rank[r]; elems[fill[level[e]]++] = e; }
	bool ok = true;
	auto al = [&](void** p, size_t bytes) { if (!*p && cudaMalloc(p, bytes ? bytes : 1) != cudaSuccess) ok = false; };
	al((void**)&im->colour2, (size_t)n_vol * 4); al((void**)&im->nbr, (size_t)n_vol * n_fl * 4);
	al((void**)&im->rank, (size_t)n_vol * 4); al((void**)&im->level_elems, (size_t)n_vol * 4);
	al((void**)&im->offd, (size_t)n_vol * n_fl * nb * nb * 8); al((void**)&im->wbuf, (size_t)im->n * 8);
	al((void**)&im->ilu_in, (size_t)im->n * 8); al((void**)&im->ilu_out, (size_t)im->n * 8);
	if (!ok) return DPG_ERR_CUDA;
	if (cudaMemcpy(im->colour2, col2.data(), (size_t)n_vol * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
	    cudaMemcpy(im->nbr, nbr.data(), nbr.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
	    cudaMemcpy(im->rank, rank.data(), (size_t)n_vol * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
	    cudaMemcpy(im->level_elems, elems.data(), (size_t)n_vol * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
	    cudaMemset(im->offd, 0, (size_t)n_vol * n_fl * nb * nb * 8) != cudaSuccess)
		return DPG_ERR_CUDA;
	const int smem = (int)(2 * (size_t)nb * nb * 8 + (size_t)nb * 4);
	if (cudaFuncSetAttribute(k_ilu_factor_level, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
		return DPG_ERR_CUDA;
	if (ilu_staged(nb, n_fl)) {
		const int ss = (int)ilu_staged_smem(nb, n_fl);
		if (cudaFuncSetAttribute(k_ilu_level_staged<64, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, ss) !=
		        cudaSuccess ||
		    cudaFuncSetAttribute(k_ilu_level_staged<64, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, ss) !=
		        cudaSuccess)
			return DPG_ERR_CUDA;
	}
	im->n_colours2 = nc2;
	// the sweeps of one application as a graph: 2 launches per level, replayed with the right-hand side copied into
	// ilu_in and the result taken from ilu_out (the operands' addresses stay fixed from here on)
	if (im->ilu_graph) { cudaGraphExecDestroy(im->ilu_graph); im->ilu_graph = nullptr; }
	{
		cudaGraph_t graph = nullptr;
		if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return DPG_ERR_CUDA;
		enqueue_block_ilu_sweeps(c, im, im->ilu_in, im->ilu_out);
		cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
		if (e != cudaSuccess) return DPG_ERR_CUDA;
		e = cudaGraphInstantiate(&im->ilu_graph, graph, 0);
		cudaGraphDestroy(graph);
		if (e != cudaSuccess) { im->ilu_graph = nullptr; return DPG_ERR_CUDA; }
	}
	im->ilu_order = order;
	im->ilu_parts = parts;
	return DPG_OK;
}

static int assemble_block_ilu(dpg_gpu_ctx* c, Implicit* im, const double* F0)
{
	const int nb = im->nb, n_vol = c->g.n_vol, n_fl = c->g.n_fl;
	const double eps = 1e-7;
	int rc;
	im->ilu_valid = false;
	for (int col = 0; col < im->n_colours2; ++col)
		for (int j = 0; j < nb; ++j) {
			if (im->tangent) {
				k_perturb<<<grid_for(im->n), 256, 0, c->stream>>>(n_vol, nb, im->zero, im->up, im->colour2, col, j, 1.0);
				if ((rc = jvp_fp64(c, im->u, im->up, im->F1, c->trace_t, c->nnf_t))) return rc;
				k_extract_ilu<<<grid_for(im->n), 256, 0, c->stream>>>(n_vol, nb, n_fl, im->F1, im->zero, im->colour2,
				                                                       im->nbr, col, j, 1.0, im->inv_dtau, im->blocks,
				                                                       im->offd);
			} else {
				k_perturb<<<grid_for(im->n), 256, 0, c->stream>>>(n_vol, nb, im->u, im->up, im->colour2, col, j, eps);
				if ((rc = residual(c, im->up, im->F1))) return rc;
				k_extract_ilu<<<grid_for(im->n), 256, 0, c->stream>>>(n_vol, nb, n_fl, im->F1, F0, im->colour2,
				                                                       im->nbr, col, j, 1.0 / eps, im->inv_dtau,
				                                                       im->blocks, im->offd);
			}
		}
	if (cudaMemsetAsync(im->info, 0, 4, c->stream) != cudaSuccess) return DPG_ERR_CUDA;
	const size_t smem = 2 * (size_t)nb * nb * 8 + (size_t)nb * 4;
	const int n_levels = (int)im->level_ptr.size() - 1;
	for (int l = 0; l < n_levels; ++l) {
		const int cnt = im->level_ptr[l + 1] - im->level_ptr[l];
		if (cnt <= 0) continue;
		k_ilu_factor_level<<<cnt, 256, smem, c->stream>>>(im->level_elems + im->level_ptr[l], nb, n_fl, im->nbr,
		                                                  im->rank, im->blocks, im->offd, im->info);
	}
	int info = 0;
	if (cudaMemcpyAsync(&info, im->info, 4, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess) return DPG_ERR_CUDA;
	if (cudaStreamSynchronize(c->stream) != cudaSuccess) return DPG_ERR_CUDA;
	im->ilu_valid = (info == 0);
	return info == 0 ? DPG_OK : DPG_ERR_NONFINITE;
}

static int apply_block_ilu(dpg_gpu_ctx* c, Implicit* im, const double* r, double* z)
{
	if (cudaMemcpyAsync(im->ilu_in, r, im->n * 8, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess) return DPG_ERR_CUDA;
	if (cudaGraphLaunch(im->ilu_graph, c->stream) != cudaSuccess) return DPG_ERR_CUDA;
	if (cudaMemcpyAsync(z, im->ilu_out, im->n * 8, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess) return DPG_ERR_CUDA;
	return DPG_OK;
}

static int apply_precond(dpg_gpu_ctx* c, Implicit* im, int precond, const double* r, double* z)
{
	const int nb = im->nb, n_vol = c->g.n_vol;
	const int wpb = 8;
	if (precond == DPG_PRECOND_BLOCK_JACOBI) {
		k_lu_solve<<<(n_vol + wpb - 1) / wpb, 32 * wpb, (size_t)wpb * nb * 8, c->stream>>>(n_vol, nb, im->blocks, im->piv, r, z);
	} else if (precond == DPG_PRECOND_BLOCK_ILU) {
		const int rc = apply_block_ilu(c, im, r, z);
		if (rc) return rc;
	} else if (precond == DPG_PRECOND_MLP) {
		k_block_apply<<<(n_vol + wpb - 1) / wpb, 32 * wpb, 0, c->stream>>>(n_vol, nb, im->P, r, z, im->inv_dtau,
		                                                                   mlp_rho(c));
	} else {
		if (cudaMemcpyAsync(z, r, im->n * 8, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess) return DPG_ERR_CUDA;
	}
	return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

// A z = z / dtau_e - dF/du z: the analytic tangent, or (F(u + eps z) - F(u)) / eps
static int apply_A(dpg_gpu_ctx* c, Implicit* im, const double* z, double* out, double u_norm, double z_norm)
{
	if (im->tangent) {
		int rc = jvp_fp64(c, im->u, z, im->F1, c->trace_t, c->nnf_t);
		if (rc) return rc;
		k_shift_minus<<<grid_for(im->n), 256, 0, c->stream>>>(im->n, im->nb, im->inv_dtau, z, im->F1, out);
		return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
	}
	const double eps = std::sqrt(2.2e-16) * (1.0 + u_norm) / std::max(z_norm, 1e-300);
	k_lincomb3<<<grid_for(im->n), 256, 0, c->stream>>>(im->n, 1.0, im->u, eps, z, im->up);
	int rc = residual(c, im->up, im->F1);
	if (rc) return rc;
	k_shift_minus_fd<<<grid_for(im->n), 256, 0, c->stream>>>(im->n, im->nb, im->inv_dtau, z, im->F1, im->F0, 1.0 / eps,
	                                                          out);
	return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

static double host_norm2(dpg_gpu_ctx* c, Implicit* im, const double* x, int* rc)
{
	double h;
	*rc = multidot(c, im, 1, x, x, &h);
	return std::sqrt(std::max(h, 0.0));
}

// GMRES(m), right preconditioned, for A du = F0; returns iterations; du in im->du.
static int gmres(dpg_gpu_ctx* c, Implicit* im, int precond, double rtol, int max_it, double u_norm,
                 int* iters, double* rel_res)
{
	const int m = im->m;
	const int64_t n = im->n;
	int rc;
	if (cudaMemsetAsync(im->du, 0, n * 8, c->stream) != cudaSuccess) return DPG_ERR_CUDA;
	const double bnorm = host_norm2(c, im, im->F0, &rc);
	if (rc) return rc;
	*iters = 0;
	*rel_res = 0.0;
	if (bnorm == 0.0) return DPG_OK;
	double rnorm = bnorm;
	// r = b - A du (du = 0 on the first cycle)
	if (cudaMemcpyAsync(im->V, im->F0, n * 8, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess) return DPG_ERR_CUDA;
	std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), hcol(m + 1);
	while (*iters < max_it) {
		k_axpby<<<grid_for(n), 256, 0, c->stream>>>(n, 1.0 / rnorm, im->V, 0.0, im->V);
		std::fill(g.begin(), g.end(), 0.0);
		g[0] = rnorm;
		int j = 0;
		for (; j < m && *iters < max_it; ++j) {
			double* vj = im->V + (int64_t)j * n;
			double* zj = im->Z + (int64_t)j * n;
			if ((rc = apply_precond(c, im, precond, vj, zj))) return rc;
			double znorm = 0.0;   // only the finite-difference product needs it (its step size)
			if (!im->tangent) {
				znorm = host_norm2(c, im, zj, &rc);
				if (rc) return rc;
			}
			double* w = im->V + (int64_t)(j + 1) * n;
			if ((rc = apply_A(c, im, zj, w, u_norm, znorm))) return rc;
			// classical Gram-Schmidt, twice, and the norm -- all on the device; one copy of the column per iteration
			k_multidot_partial<<<kRedBlocks, kRedThreads, 0, c->stream>>>(n, j + 1, im->V, n, w, im->partial);
			k_reduce_partials<<<j + 1, 256, 0, c->stream>>>(j + 1, kRedBlocks, im->partial, im->h);
			k_sub_combination<<<grid_for(n), 256, 0, c->stream>>>(n, j + 1, im->V, n, im->h, w);
			k_multidot_partial<<<kRedBlocks, kRedThreads, 0, c->stream>>>(n, j + 1, im->V, n, w, im->partial);
			k_reduce_partials<<<j + 1, 256, 0, c->stream>>>(j + 1, kRedBlocks, im->partial, im->h2);
			k_sub_combination<<<grid_for(n), 256, 0, c->stream>>>(n, j + 1, im->V, n, im->h2, w);
			k_multidot_partial<<<kRedBlocks, kRedThreads, 0, c->stream>>>(n, 1, w, n, w, im->partial);
			k_reduce_partials<<<1, 256, 0, c->stream>>>(1, kRedBlocks, im->partial, im->h2 + j + 1);
			k_column_finish<<<1, 256, 0, c->stream>>>(j, im->h, im->h2);
			k_scale_inv<<<grid_for(n), 256, 0, c->stream>>>(n, w, im->h + j + 1);
			if (cudaMemcpyAsync(im->hcol_host, im->h, 8 * (j + 2), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
			    cudaStreamSynchronize(c->stream) != cudaSuccess)
				return DPG_ERR_CUDA;
			for (int i = 0; i <= j + 1; ++i) hcol[i] = im->hcol_host[i];
			const double hn = hcol[j + 1];
			if (!std::isfinite(hn)) return DPG_ERR_NONFINITE;
			// Givens rotations
			for (int i = 0; i < j; ++i) {
				const double t = cs[i] * hcol[i] + sn[i] * hcol[i + 1];
				hcol[i + 1] = -sn[i] * hcol[i] + cs[i] * hcol[i + 1];
				hcol[i] = t;
			}
			const double den = std::hypot(hcol[j], hcol[j + 1]);
			cs[j] = den > 0 ? hcol[j] / den : 1.0;
			sn[j] = den > 0 ? hcol[j + 1] / den : 0.0;
			hcol[j] = den;
			hcol[j + 1] = 0.0;
			g[j + 1] = -sn[j] * g[j];
			g[j] = cs[j] * g[j];
			for (int i = 0; i <= j; ++i) H[(size_t)i * m + j] = hcol[i];
			++*iters;
			if (std::fabs(g[j + 1]) <= rtol * bnorm || hn == 0.0) { ++j; break; }
		}
		// y = H^-1 g (upper triangular j x j), du += Z y
		std::vector<double> y(j);
		for (int i = j - 1; i >= 0; --i) {
			double s = g[i];
			for (int k = i + 1; k < j; ++k) s -= H[(size_t)i * m + k] * y[k];
			y[i] = s / H[(size_t)i * m + i];
		}
		cudaMemcpyAsync(im->h, y.data(), 8 * j, cudaMemcpyHostToDevice, c->stream);
		k_add_combination<<<grid_for(n), 256, 0, c->stream>>>(n, j, im->Z, n, im->h, im->du);
		rnorm = std::fabs(g[j]);
		*rel_res = rnorm / bnorm;
		if (rnorm <= rtol * bnorm) break;
		// restart: r = b - A du
		const double dun = host_norm2(c, im, im->du, &rc);
		if (rc) return rc;
		if ((rc = apply_A(c, im, im->du, im->w, u_norm, dun))) return rc;
		k_lincomb3<<<grid_for(n), 256, 0, c->stream>>>(n, 1.0, im->F0, -1.0, im->w, im->V);
		rnorm = host_norm2(c, im, im->V, &rc);
		if (rc) return rc;
		*rel_res = rnorm / bnorm;
		if (rnorm <= rtol * bnorm) break;
	}
	return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

int implicit_solve(dpg_gpu_ctx* c, const dpg_newton_params* prm, dpg_newton_stats* st)
{
	const int m = std::max(2, std::min(prm->gmres_restart, 512));
	int rc;
	Implicit* im = implicit_state(c, m);
	if (!im) return DPG_ERR_CUDA;
	if (prm->precond == DPG_PRECOND_MLP && !c->mlp) return DPG_ERR_INVALID;
	if (prm->jacobian != DPG_JACOBIAN_TANGENT && prm->jacobian != DPG_JACOBIAN_FD) return DPG_ERR_INVALID;
	if (prm->precond < DPG_PRECOND_NONE || prm->precond > DPG_PRECOND_BLOCK_ILU) return DPG_ERR_INVALID;
	if (!(prm->cfl_initial >= 0.0)) return DPG_ERR_INVALID;
	if (prm->cfl_initial > 0.0 && c->n_var > 1 && !c->bez_full) return DPG_ERR_UNSUPPORTED;
	if (c->pos_dense) return DPG_ERR_UNSUPPORTED;   // the relaxed update of the Newton step: tensor-product volumes
	if (prm->precond == DPG_PRECOND_BLOCK_ILU) {
		if (prm->ilu_order != DPG_ILU_ORDER_VOLUME && prm->ilu_order != DPG_ILU_ORDER_COLOUR) return DPG_ERR_INVALID;
		if (prm->ilu_parts < 0) return DPG_ERR_INVALID;
		if ((rc = ilu_build(c, im, prm->ilu_order, prm->ilu_parts))) return rc;
	}
	im->tangent = prm->jacobian == DPG_JACOBIAN_TANGENT;
	if (im->tangent && ensure_tangent_buffers(c)) return DPG_ERR_CUDA;
	memset(st, 0, sizeof *st);
	const auto t0 = std::chrono::steady_clock::now();
	im->forcing = nullptr;
	if (prm->forcing) {
		if (!im->forcing_buf && cudaMalloc(&im->forcing_buf, im->n * 8) != cudaSuccess) return DPG_ERR_CUDA;
		if (cudaMemcpy(im->forcing_buf, prm->forcing, im->n * 8, cudaMemcpyHostToDevice) != cudaSuccess) return DPG_ERR_CUDA;
		im->forcing = im->forcing_buf;
	}
	if (cudaMemcpyAsync(im->u, c->sol, im->n * 8, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess) return DPG_ERR_CUDA;
	double fmax0 = 0.0;
	if ((rc = residual(c, im->u, im->F0))) return rc;
	if ((rc = absmax(c, im, im->F0, &fmax0))) return rc;
	double fmax = fmax0;
	st->residual_initial = fmax0;
	int k = 0;
	for (; k < prm->max_newton && fmax > prm->tol; ++k) {
		const double dtau = std::min(prm->dtau0 * fmax0 / fmax, prm->dtau_max);
		const double cfl = prm->cfl_initial * std::max(1.0, fmax0 / fmax);
		if (prm->cfl_initial > 0.0)
			k_pseudo_dt<<<(c->g.n_vol + 7) / 8, 256, 0, c->stream>>>(c->g.n_vol, c->g.n_s, c->n_var, im->u, c->bez_full,
			                                                         c->h_min, c->adv_speed, c->visc_mu, cfl,
			                                                         im->inv_dtau);
		else
			k_fill<<<grid_for(c->g.n_vol), 256, 0, c->stream>>>(c->g.n_vol, 1.0 / dtau, im->inv_dtau);
		const double u_norm = host_norm2(c, im, im->u, &rc);
		if (rc) return rc;
		int pc = prm->precond;
		if (pc == DPG_PRECOND_BLOCK_JACOBI) {
			const auto ta = std::chrono::steady_clock::now();
			if ((rc = assemble_block_jacobi(c, im, im->F0))) return rc;
			st->assembly_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - ta).count();
			if (prm->collect_blocks && c->mlp) mlp_collect(c, im->u, im->blocks, im->piv, im->inv_dtau, im->rho);
		} else if (pc == DPG_PRECOND_MLP) {
			if ((rc = mlp_predict(c, im->u, im->inv_dtau, &im->P))) return rc;
		} else if (pc == DPG_PRECOND_BLOCK_ILU) {
			const auto ta = std::chrono::steady_clock::now();
			if ((rc = assemble_block_ilu(c, im, im->F0))) return rc;
			st->assembly_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - ta).count();
		}
		int its = 0;
		double rel = 0.0;
		if ((rc = gmres(c, im, pc, prm->gmres_rtol, prm->max_gmres, u_norm, &its, &rel))) return rc;
		st->gmres_iterations += its;
		if (pc == DPG_PRECOND_MLP && rel > 10.0 * prm->gmres_rtol) {
			// the learned inverse did not give a converged Krylov solve: redo the step with exact block-Jacobi
			const auto ta = std::chrono::steady_clock::now();
			if ((rc = assemble_block_jacobi(c, im, im->F0))) return rc;
			st->assembly_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - ta).count();
			if ((rc = gmres(c, im, DPG_PRECOND_BLOCK_JACOBI, prm->gmres_rtol, prm->max_gmres, u_norm, &its, &rel)))
				return rc;
			st->gmres_iterations += its;
			++st->fallback_steps;
		}
		// u += du ; F0 = F(u).  With positivity (Euler) the update is under-relaxed per volume and limited as in the
		// reference (update_coef_s_v, solve_implicit.c:724-731, 821-873).  A step that produces a non-finite residual
		// or breaks positivity beyond repair (where the reference stops) is undone and the pseudo time step of the next
		// attempt is reduced (fmax0 scaled so that dtau halves).
		if (cudaMemcpyAsync(im->up, im->u, im->n * 8, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess)
			return DPG_ERR_CUDA;
		if (c->positivity) {
			if ((rc = launch_relaxed_update(c, im->u, im->du))) return rc;
			if ((rc = launch_positivity(c, im->u))) return rc;
		} else {
			k_axpby<<<grid_for(im->n), 256, 0, c->stream>>>(im->n, 1.0, im->du, 1.0, im->u);
		}
		const int pos_bad = positivity_error(c);
		if (pos_bad < 0) return DPG_ERR_CUDA;
		double fnew = 0.0;
		rc = pos_bad ? DPG_ERR_NONFINITE : residual(c, im->u, im->F0);
		if (rc == DPG_OK) rc = absmax(c, im, im->F0, &fnew);
		if (rc == DPG_ERR_NONFINITE) {
			if (cudaMemcpyAsync(im->u, im->up, im->n * 8, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess)
				return DPG_ERR_CUDA;
			if ((rc = residual(c, im->u, im->F0))) return rc;
			if ((rc = absmax(c, im, im->F0, &fnew))) return rc;
			fmax0 *= 0.5;
			++st->rejected_steps;
			if (prm->verbose) printf("newton %2d  rejected (non-finite state), dtau halved\n", k);
		} else if (rc) {
			return rc;
		}
		fmax = fnew;
		if (prm->verbose)
			printf("newton %2d  %s %.3e  gmres %3d (rel %.2e)  ||F||_inf %.3e\n", k,
			       prm->cfl_initial > 0.0 ? "cfl" : "dtau", prm->cfl_initial > 0.0 ? cfl : dtau, its, rel, fmax);
	}
	st->newton_iterations = k;
	st->residual_final = fmax;
	if (cudaMemcpyAsync(c->sol, im->u, im->n * 8, cudaMemcpyDeviceToDevice, c->stream) != cudaSuccess) return DPG_ERR_CUDA;
	if (cudaStreamSynchronize(c->stream) != cudaSuccess) return DPG_ERR_CUDA;
	st->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
	return fmax <= prm->tol ? DPG_OK : DPG_ERR_NOT_CONVERGED;
}

} // namespace dpg
