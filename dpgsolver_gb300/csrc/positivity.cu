// Positivity of density and pressure for the Euler equations, on the Bezier coefficients of the solution:
//   k_positivity     enforce_positivity_highorder (solve.c:187-233), run after every RK stage update, and after the
//                    Newton update, on every volume, as the reference does for the PDEs of
//                    test_case_requires_positivity (test_case.c:63-80);
//   k_relax_update   the Newton update u += relax du with the per-volume under-relaxation of compute_relaxation
//                    (solve_implicit.c:821-873, update_coef_s_v :724-731).
// Algorithm of the limiter (per volume): Bezier coefficients b = ccSB0 u, read as primitive variables (density,
// velocity, pressure: convert_variables, solution_euler_T.c:136-200); for density and then pressure, stop with an
// error when the coefficients' average is below EPS_PHYS, and where their minimum is below EPS_PHYS pull every
// variable's coefficients toward its average by p_ho = clamp((avg - EPS_PHYS) / (avg - min), 0, 1)
// (correct_coef, solve.c:356-374); back to conservative variables and u = ccBS0 b.
//
// GB300 form: one thread per (volume, solution node), several volumes per block; the tensor-product Bezier operators
// are applied one direction at a time (1D factors, shared memory).  Nearly every volume of a physical state is far
// from the thresholds, so a volume is first screened in FP32: its Bezier coefficients are bounded from below with a
// rigorous margin for the FP32 rounding, and only a block holding a volume whose bound does not clear EPS_PHYS
// repeats the transform in FP64 and runs the reference's serial algorithm for those volumes (one thread per volume,
// the reference's summation order).  Volumes that pass the screen are left as they are (the reference's round trip
// through the Bezier and primitive forms changes them only by rounding).
#include <algorithm>
#include <cmath>
#include <cstdio>

#include "dpg_gpu_internal.cuh"

namespace dpg {
namespace {

constexpr int kPosThreads = 256;

template <int D, int N1>
struct PosShape {
	static constexpr int NS = (D == 2 ? N1 * N1 : N1 * N1 * N1);
	static constexpr int NV = D + 2;
	static constexpr int EPB = kPosThreads / NS;   // volumes per block
	static constexpr int BUF = EPB * NV * NS;      // one [EPB][NV][NS] buffer
};

// One tensor-product operator (A ⊗ A [⊗ A], A row-major N1 x N1, output index = row) applied to the NV variables of
// every volume of the block: D one-direction passes between buf[0] and buf[1]; returns the buffer holding the result.
// All threads of the block call it (barriers inside); thread (el, node) computes its node of each variable.
template <int D, int N1, typename T>
__device__ T* tp_apply(const T* A, T* b0, T* b1, int el, int node, bool live)
{
	using S = PosShape<D, N1>;
	T* in = b0;
	T* out = b1;
	int stride = 1;
#pragma unroll
	for (int dir = 0; dir < D; ++dir) {
		if (live) {
			const int i = (node / stride) % N1, base = node - i * stride;
#pragma unroll
			for (int v = 0; v < S::NV; ++v) {
				const T* x = in + (el * S::NV + v) * S::NS + base;
				T acc = 0;
#pragma unroll
				for (int k = 0; k < N1; ++k) acc += A[i * N1 + k] * x[k * stride];
				out[(el * S::NV + v) * S::NS + node] = acc;
			}
		}
		__syncthreads();
		T* t = in; in = out; out = t;
		stride *= N1;
	}
	return in;
}

// FP32 value of a double by integer operations only, truncating the mantissa (relative error < 2^-23): a conversion
// instruction would run on GB300's FP64 pipe, which bounds the screen's throughput otherwise.  Magnitudes below
// 2^-126 become 0 (absolute error far below EPS_PHYS), above the FP32 range, infinities and NaN become infinity (the
// screen then flags the volume).
__device__ __forceinline__ float trunc_to_float(double x)
{
	const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
	const int t = (int)(hi & 0x7fffffffu) - ((1023 - 127) << 20);   // exponent rebiased, mantissa's top 20 bits
	unsigned bits = __funnelshift_l(lo, (unsigned)t, 3);            // (t << 3) | (lo >> 29)
	bits = t < (1 << 20) ? 0u : t >= (255 << 20) ? 0x7f800000u : bits;
	return __uint_as_float(bits | (hi & 0x80000000u));
}

// convert_variables 'c' -> 'p' / 'p' -> 'c' of one coefficient (the reference's operation order)
template <int D>
__device__ void cons_to_prim(double* w)
{
	const double rho_inv = 1.0 / w[0];
	double rho2V2 = 0.0;
#pragma unroll
	for (int a = 0; a < D; ++a) {
		rho2V2 += w[1 + a] * w[1 + a];
		w[1 + a] = w[1 + a] * rho_inv;
	}
	w[D + 1] = 0.4 * (w[D + 1] - 0.5 * rho2V2 * rho_inv);
}
template <int D>
__device__ void prim_to_cons(double* w)
{
	double V2 = 0.0;
#pragma unroll
	for (int a = 0; a < D; ++a) {
		V2 += w[1 + a] * w[1 + a];
		w[1 + a] = w[0] * w[1 + a];
	}
	w[D + 1] = w[D + 1] / 0.4 + 0.5 * w[0] * V2;
}

// the reference's average_T / minimum_T over n coefficients (sequential sum)
__device__ double avg_seq(const double* x, int n)
{
	double s = 0.0;
#pragma unroll 1
	for (int i = 0; i < n; ++i) s += x[i];
	return s / (double)n;
}
__device__ double min_seq(const double* x, int n)
{
	double m = 1.7976931348623157e308;
#pragma unroll 1
	for (int i = 0; i < n; ++i)
		if (x[i] < m) m = x[i];
	return m;
}

// The serial part of enforce_positivity_highorder on one volume's primitive Bezier coefficients w [NV][NS]; false
// where an average is below EPS_PHYS (the reference stops there).
template <int D, int NS>
__device__ bool limit_volume(double* w)
{
	constexpr int NV = D + 2;
#pragma unroll 1
	for (int vr = 0; vr < NV; vr += NV - 1) {
		const double avg = avg_seq(w + vr * NS, NS);
		if (!(avg >= DPG_EPS_PHYS)) return false;
		const double mn = min_seq(w + vr * NS, NS);
		if (mn < DPG_EPS_PHYS) {
			const double p_ho = fmax(0.0, fmin(1.0, (avg - DPG_EPS_PHYS) / (avg - mn)));
#pragma unroll 1
			for (int v = 0; v < NV; ++v) {
				double* x = w + v * NS;
				double a = avg_seq(x, NS);
				if ((v == 0 || v == NV - 1) && a < DPG_EPS_PHYS) a = DPG_EPS_PHYS;
#pragma unroll 1
				for (int i = 0; i < NS; ++i) x[i] = p_ho * x[i] + (1 - p_ho) * a;
			}
		}
	}
	return true;
}

// 1D operators of the limiter as kernel parameters (read from the constant bank at compile-time indices)
struct PosOps {
	float ai32[25];    // bez1_inv in FP32 (the screen)
	float rs;          // bound of bez1_inv's absolute row sums (the screen's error bound)
	double a64[25];    // bez1: Bezier -> solution coefficients
	double ai64[25];   // bez1_inv: solution -> Bezier coefficients
};

// Launch shape of the limiter: one thread per pencil (a line of n1 nodes along one direction), EPB volumes per
// block of at most 128 threads (small blocks: many resident per SM, even waves); the block's [EPB][NV][NS] doubles
// stay within 48 KB of static shared memory.
template <int D, int N1>
struct PencilShape {
	static constexpr int NS = (D == 2 ? N1 * N1 : N1 * N1 * N1);
	static constexpr int NV = D + 2;
	static constexpr int P = NS / N1;                     // pencils per volume
	static constexpr int THREADS = 128;
	static constexpr int MINB = (N1 == 5 ? 4 : 7);          // resident blocks per SM asked of the register allocation
	static constexpr int EPB = THREADS / P;
	static constexpr int NT = EPB * P;                    // threads of a block
	static constexpr int BUF = EPB * NV * NS;
};

// one 1D operator on n1 values (row-major A, output i = sum_k A[i][k] x[k])
template <int N1, typename T, typename A>
__device__ __forceinline__ void apply1(const A& a, const T (&x)[N1], T (&y)[N1])
{
#pragma unroll
	for (int i = 0; i < N1; ++i) {
		T acc = 0;
#pragma unroll
		for (int k = 0; k < N1; ++k) acc += (T)a[i * N1 + k] * x[k];
		y[i] = acc;
	}
}

// FP64 tensor-product operator applied in place to the NV variables of every volume of the block in shared memory
// (pencils of one direction are disjoint: one barrier per direction).  All threads call it.  Node k of pencil q along
// the direction of stride n1^dir: q % stride + stride (k + n1 (q / stride)).
template <int D, int N1, bool INV>
__device__ __forceinline__ void tp_pencils64(const PosOps& ops, double* s, int el, int q)
{
	using S = PencilShape<D, N1>;
#pragma unroll
	for (int dir = 0; dir < D; ++dir) {
		const int stride = dir == 0 ? 1 : dir == 1 ? N1 : N1 * N1;
#pragma unroll
		for (int v = 0; v < S::NV; ++v) {
			double* base = s + (el * S::NV + v) * S::NS;
			double x[N1], y[N1];
#pragma unroll
			for (int k = 0; k < N1; ++k) x[k] = base[q % stride + stride * (k + N1 * (q / stride))];
			if (INV) apply1<N1>(ops.ai64, x, y);
			else apply1<N1>(ops.a64, x, y);
#pragma unroll
			for (int k = 0; k < N1; ++k) base[q % stride + stride * (k + N1 * (q / stride))] = y[k];
		}
		__syncthreads();
	}
}

template <int D, int N1>
__global__ void __launch_bounds__(PencilShape<D, N1>::THREADS, PencilShape<D, N1>::MINB) k_positivity(double* __restrict__ sol, int n_vol,
                                                                          const __grid_constant__ PosOps ops,
                                                                          float amp, int* __restrict__ err)
{
	using S = PencilShape<D, N1>;
	constexpr int NS = S::NS, NV = S::NV, P = S::P, EPB = S::EPB;
	__shared__ double s64[S::BUF];   // FP64 path; before it the screen's (coefficient, magnitude sum) FP32 pairs
	__shared__ int sflag[EPB];
	float2* sbc = reinterpret_cast<float2*>(s64);

	const int tid = threadIdx.x, el = tid / P, q = tid - el * P;
	const int e = blockIdx.x * EPB + el;
	const bool live = e < n_vol;
	if (tid < EPB) sflag[tid] = 0;

	// 1. FP32 screen.  b = A^-1 u in FP32 differs from the exact coefficient by at most eps = amp * c, c = |A^-1| |u|
	//    (amp = 4 (D (n1 + 2) + 2) 2^-24: the truncation of u, the rounding of the operator and the n1-term sums of
	//    the D passes, with a factor 4 of margin; set by the host), so rho >= b_rho - eps_rho and
	//    p >= 0.4 (E_lo - 0.5 |m_hi|^2 / rho_lo); the FP32 evaluation of that bound is covered by a further 2^-20 of
	//    its terms.  c is carried as an upper bound: each pass replaces the pencil's n1 magnitudes by
	//    rs * (their maximum), rs >= the largest absolute row sum of A^-1.  Direction 0 from global memory (the
	//    pencil's n1 nodes are consecutive), the others through shared memory in place; the last direction's
	//    coefficients stay in registers.
	float b[NV][N1], c[NV][N1];
	{
		const double* src = sol + (size_t)e * NS * NV + q * N1;
		double raw[NV][N1];   // every load issued before the first use; 16-byte loads where n1 is even
#pragma unroll
		for (int v = 0; v < NV; ++v) {
			if constexpr (N1 % 2 == 0) {
#pragma unroll
				for (int k = 0; k < N1; k += 2) {
					const double2 t = live ? *reinterpret_cast<const double2*>(src + v * NS + k) : make_double2(1.0, 1.0);
					raw[v][k] = t.x;
					raw[v][k + 1] = t.y;
				}
			} else {
#pragma unroll
				for (int k = 0; k < N1; ++k) raw[v][k] = live ? src[v * NS + k] : 1.0;
			}
		}
#pragma unroll
		for (int v = 0; v < NV; ++v) {
			float x[N1], ax[N1];
#pragma unroll
			for (int k = 0; k < N1; ++k) {
				x[k] = trunc_to_float(raw[v][k]);
				ax[k] = fabsf(x[k]);
			}
			float mx = ax[0];
#pragma unroll
			for (int k = 1; k < N1; ++k) mx = fmaxf(mx, ax[k]);
#pragma unroll
			for (int i = 0; i < N1; ++i) {
				float yb = 0.f;
#pragma unroll
				for (int k = 0; k < N1; ++k) yb += ops.ai32[i * N1 + k] * x[k];
				b[v][i] = yb;
				c[v][i] = ops.rs * mx;
			}
		}
	}
#pragma unroll
	for (int dir = 1; dir < D; ++dir) {
		const int sp = dir == 1 ? 1 : N1, st = dir == 1 ? N1 : N1 * N1;   // strides of the previous / this direction
#pragma unroll
		for (int v = 0; v < NV; ++v)
#pragma unroll
			for (int k = 0; k < N1; ++k) {
				const int o = (el * NV + v) * NS + q % sp + sp * (k + N1 * (q / sp));
				sbc[o] = make_float2(b[v][k], c[v][k]);
			}
		__syncthreads();
#pragma unroll
		for (int v = 0; v < NV; ++v) {
			float x[N1], ax[N1];
#pragma unroll
			for (int k = 0; k < N1; ++k) {
				const int o = (el * NV + v) * NS + q % st + st * (k + N1 * (q / st));
				const float2 t = sbc[o];
				x[k] = t.x;
				ax[k] = t.y;
			}
			float mx = ax[0];
#pragma unroll
			for (int k = 1; k < N1; ++k) mx = fmaxf(mx, ax[k]);
#pragma unroll
			for (int i = 0; i < N1; ++i) {
				float yb = 0.f;
#pragma unroll
				for (int k = 0; k < N1; ++k) yb += ops.ai32[i * N1 + k] * x[k];
				b[v][i] = yb;
				c[v][i] = ops.rs * mx;
			}
		}
	}
	bool bad = false;
	if (live) {
#pragma unroll
		for (int i = 0; i < N1; ++i) {
			const float rho_lo = b[0][i] - amp * c[0][i];
			float m2 = 0.f;
#pragma unroll
			for (int a = 0; a < D; ++a) {
				const float m = fabsf(b[1 + a][i]) + amp * c[1 + a][i];
				m2 += m * m;
			}
			const float eE = amp * c[NV - 1][i];
			const float q2 = 0.5f * m2 / rho_lo, E_lo = b[NV - 1][i] - eE;
			const float p_lo = 0.4f * (E_lo - q2) - 9.5367431640625e-07f * (fabsf(b[NV - 1][i]) + eE + q2);
			bad |= !(rho_lo > 2.0f * (float)DPG_EPS_PHYS) || !(p_lo > 2.0f * (float)DPG_EPS_PHYS);
		}
		if (bad) sflag[el] = 1;
	}
	if (!__syncthreads_or(bad)) return;   // every volume of the block clears the thresholds (ends the FP32 reads)

	// 2. the reference's algorithm in FP64 for the flagged volumes of this block
	const size_t blk = (size_t)blockIdx.x * EPB * NV * NS;
	for (int i = tid; i < S::BUF; i += S::NT)
		s64[i] = (blockIdx.x * EPB + i / (NV * NS) < n_vol) ? sol[blk + i] : 1.0;
	__syncthreads();
	tp_pencils64<D, N1, true>(ops, s64, el, q);
	for (int i = tid; i < EPB * NS; i += S::NT) {   // to primitive variables, flagged volumes
		const int l = i / NS, node = i - l * NS;
		if (!sflag[l]) continue;
		double w[NV];
#pragma unroll
		for (int v = 0; v < NV; ++v) w[v] = s64[(l * NV + v) * NS + node];
		cons_to_prim<D>(w);
#pragma unroll
		for (int v = 0; v < NV; ++v) s64[(l * NV + v) * NS + node] = w[v];
	}
	__syncthreads();
	if (q == 0 && live && sflag[el]) {
		if (!limit_volume<D, NS>(s64 + el * NV * NS)) {
			atomicOr(err, 1);   // average density or pressure below EPS_PHYS: the volume is left unchanged
			sflag[el] = 0;
		}
	}
	__syncthreads();
	for (int i = tid; i < EPB * NS; i += S::NT) {   // back to conservative variables
		const int l = i / NS, node = i - l * NS;
		if (!sflag[l]) continue;
		double w[NV];
#pragma unroll
		for (int v = 0; v < NV; ++v) w[v] = s64[(l * NV + v) * NS + node];
		prim_to_cons<D>(w);
#pragma unroll
		for (int v = 0; v < NV; ++v) s64[(l * NV + v) * NS + node] = w[v];
	}
	__syncthreads();
	tp_pencils64<D, N1, false>(ops, s64, el, q);
	for (int i = tid; i < S::BUF; i += S::NT)
		if (sflag[i / (NV * NS)]) sol[blk + i] = s64[i];
}

// u += relax du per volume, relax = 2^-k from compute_relaxation: the Bezier coefficients of u + relax du, read as
// primitive variables, must have density and pressure averages of at least EPS_PHYS.  FP64 throughout (the Newton
// update runs once per Newton step).
template <int D, int N1>
__global__ void __launch_bounds__(kPosThreads) k_relax_update(double* __restrict__ u, const double* __restrict__ du,
                                                             int n_vol, const double* __restrict__ bez_inv,
                                                             int* __restrict__ err)
{
	using S = PosShape<D, N1>;
	constexpr int NS = S::NS, NV = S::NV, EPB = S::EPB;
	__shared__ double sb[2][S::BUF];
	__shared__ double sd[2][S::BUF];
	__shared__ double sAi[N1 * N1];
	__shared__ double srelax[EPB];

	const int tid = threadIdx.x, el = tid / NS, node = tid - el * NS;
	const int e = blockIdx.x * EPB + el;
	const bool live = el < EPB && e < n_vol;
	if (tid < N1 * N1) sAi[tid] = bez_inv[tid];
	const size_t off = (size_t)e * NS * NV + node;
	if (live) {
#pragma unroll
		for (int v = 0; v < NV; ++v) {
			sb[0][(el * NV + v) * NS + node] = u[off + v * NS];
			sd[0][(el * NV + v) * NS + node] = du[off + v * NS];
		}
	}
	__syncthreads();
	double* b = tp_apply<D, N1, double>(sAi, sb[0], sb[1], el, node, live);
	const double* db = tp_apply<D, N1, double>(sAi, sd[0], sd[1], el, node, live);
	if (live && node == 0) {
		double* w = b + el * NV * NS;
		const double* dw = db + el * NV * NS;
		double relax = 1.0;
		do {   // the reference's in-place sequence: add, convert, test, convert back, subtract, halve
#pragma unroll 1
			for (int i = 0; i < NV * NS; ++i) w[i] += relax * dw[i];
#pragma unroll 1
			for (int i = 0; i < NS; ++i) {
				double c[NV];
				for (int v = 0; v < NV; ++v) c[v] = w[v * NS + i];
				cons_to_prim<D>(c);
				for (int v = 0; v < NV; ++v) w[v * NS + i] = c[v];
			}
			if (!(avg_seq(w, NS) < DPG_EPS_PHYS || avg_seq(w + (NV - 1) * NS, NS) < DPG_EPS_PHYS)) break;
#pragma unroll 1
			for (int i = 0; i < NS; ++i) {
				double c[NV];
				for (int v = 0; v < NV; ++v) c[v] = w[v * NS + i];
				prim_to_cons<D>(c);
				for (int v = 0; v < NV; ++v) w[v * NS + i] = c[v];
			}
#pragma unroll 1
			for (int i = 0; i < NV * NS; ++i) w[i] -= relax * dw[i];
			relax /= 2.0;
		} while (relax > DPG_EPS);
		if (relax < DPG_EPS) {
			atomicOr(err, 2);   // under-relaxation approaching zero: the volume is not updated
			relax = 0.0;
		}
		srelax[el] = relax;
	}
	__syncthreads();
	if (live) {
		const double r = srelax[el];
#pragma unroll
		for (int v = 0; v < NV; ++v) u[off + v * NS] += r * du[off + v * NS];
	}
}

// The limiter on simplices (TRI, TET): dense Bezier operators (the Bernstein polynomials of a simplex have no 1D
// factors).  One warp per volume, grid-stride over the volumes; a lane per Bezier coefficient (n_s <= 64, two per
// lane).  The FP32 screen as above with b = ccSB0 u and c = |ccSB0| |u| summed directly (amp = 4 (n_s + 5) 2^-24,
// set by the host); a volume that does not clear it runs the reference's algorithm in FP64: ccSB0 u, primitive
// variables, limit_volume's serial steps on lane 0, conservative variables, u = ccBS0 b.  The operators sit in
// shared memory (FP32 ccSB0 for the screen, FP64 ccSB0 and ccBS0), with a [NV][n_s] FP32 and two FP64 buffers per
// warp.
constexpr int kDenseWarps = 4;

template <int D>
__device__ bool limit_volume_n(double* w, int ns)
{
	constexpr int NV = D + 2;
#pragma unroll 1
	for (int vr = 0; vr < NV; vr += NV - 1) {
		const double avg = avg_seq(w + vr * ns, ns);
		if (!(avg >= DPG_EPS_PHYS)) return false;
		const double mn = min_seq(w + vr * ns, ns);
		if (mn < DPG_EPS_PHYS) {
			const double p_ho = fmax(0.0, fmin(1.0, (avg - DPG_EPS_PHYS) / (avg - mn)));
#pragma unroll 1
			for (int v = 0; v < NV; ++v) {
				double* x = w + v * ns;
				double a = avg_seq(x, ns);
				if ((v == 0 || v == NV - 1) && a < DPG_EPS_PHYS) a = DPG_EPS_PHYS;
#pragma unroll 1
				for (int i = 0; i < ns; ++i) x[i] = p_ho * x[i] + (1 - p_ho) * a;
			}
		}
	}
	return true;
}

template <int D>
__global__ void __launch_bounds__(kDenseWarps * 32) k_positivity_dense(double* __restrict__ sol, int n_vol, int ns,
                                                                     const float* __restrict__ sb32,
                                                                     const double* __restrict__ sb64,
                                                                     const double* __restrict__ bs64, float amp,
                                                                     int* __restrict__ err,
                                                                     const int* __restrict__ vols,
                                                                     const int64_t* __restrict__ dof_off)
{
	constexpr int NV = D + 2;
	extern __shared__ double dsm[];
	const int nn = ns * ns, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	double* sSB = dsm;                                   // [ns][ns]
	double* sBS = sSB + nn;                              // [ns][ns]
	double* sW = sBS + nn + (size_t)warp * 2 * NV * ns;  // this warp's [2][NV][ns]
	float* sA32 = reinterpret_cast<float*>(sBS + nn + (size_t)kDenseWarps * 2 * NV * ns);   // [ns][ns]
	float* sX = sA32 + nn + (size_t)warp * NV * ns;       // this warp's [NV][ns]
	for (int i = threadIdx.x; i < nn; i += blockDim.x) {
		sSB[i] = sb64[i];
		sBS[i] = bs64[i];
		sA32[i] = sb32[i];
	}
	__syncthreads();
	for (int e = blockIdx.x * kDenseWarps + warp; e < n_vol; e += gridDim.x * kDenseWarps) {
		const int ev = vols ? vols[e] : e;   // mixed orders: the group's volume list and the volumes' offsets
		double* u = sol + (dof_off ? (size_t)dof_off[ev] : (size_t)ev * NV * ns);
		for (int i = lane; i < NV * ns; i += 32) sX[i] = trunc_to_float(u[i]);
		__syncwarp();
		bool bad = false;
		for (int i = lane; i < ns; i += 32) {
			float b[NV], c[NV];
#pragma unroll
			for (int v = 0; v < NV; ++v) {
				float yb = 0.f, yc = 0.f;
				for (int k = 0; k < ns; ++k) {
					const float a = sA32[i * ns + k], x = sX[v * ns + k];
					yb += a * x;
					yc += fabsf(a) * fabsf(x);
				}
				b[v] = yb;
				c[v] = yc;
			}
			const float rho_lo = b[0] - amp * c[0];
			float m2 = 0.f;
#pragma unroll
			for (int a = 0; a < D; ++a) {
				const float m = fabsf(b[1 + a]) + amp * c[1 + a];
				m2 += m * m;
			}
			const float eE = amp * c[NV - 1];
			const float q2 = 0.5f * m2 / rho_lo, E_lo = b[NV - 1] - eE;
			const float p_lo = 0.4f * (E_lo - q2) - 9.5367431640625e-07f * (fabsf(b[NV - 1]) + eE + q2);
			bad |= !(rho_lo > 2.0f * (float)DPG_EPS_PHYS) || !(p_lo > 2.0f * (float)DPG_EPS_PHYS);
		}
		if (!__any_sync(0xffffffffu, bad)) {
			__syncwarp();
			continue;
		}
		// the reference's algorithm in FP64
		double* w0 = sW;              // u, then the primitive Bezier coefficients
		double* w1 = sW + NV * ns;    // the Bezier coefficients, then the limited conservative ones
		for (int i = lane; i < NV * ns; i += 32) w0[i] = u[i];
		__syncwarp();
		for (int o = lane; o < NV * ns; o += 32) {
			const int v = o / ns, i = o - v * ns;
			double acc = 0.0;
			for (int k = 0; k < ns; ++k) acc += sSB[i * ns + k] * w0[v * ns + k];
			w1[o] = acc;
		}
		__syncwarp();
		for (int i = lane; i < ns; i += 32) {
			double x[NV];
#pragma unroll
			for (int v = 0; v < NV; ++v) x[v] = w1[v * ns + i];
			cons_to_prim<D>(x);
#pragma unroll
			for (int v = 0; v < NV; ++v) w1[v * ns + i] = x[v];
		}
		__syncwarp();
		int ok = 1;
		if (lane == 0 && !limit_volume_n<D>(w1, ns)) {
			atomicOr(err, 1);   // average density or pressure below EPS_PHYS: the volume is left unchanged
			ok = 0;
		}
		ok = __shfl_sync(0xffffffffu, ok, 0);
		__syncwarp();
		if (ok) {
			for (int i = lane; i < ns; i += 32) {
				double x[NV];
#pragma unroll
				for (int v = 0; v < NV; ++v) x[v] = w1[v * ns + i];
				prim_to_cons<D>(x);
#pragma unroll
				for (int v = 0; v < NV; ++v) w1[v * ns + i] = x[v];
			}
			__syncwarp();
			for (int o = lane; o < NV * ns; o += 32) {
				const int v = o / ns, i = o - v * ns;
				double acc = 0.0;
				for (int k = 0; k < ns; ++k) acc += sBS[i * ns + k] * w1[v * ns + k];
				u[o] = acc;
			}
		}
		__syncwarp();
	}
}

size_t dense_smem(int d, int ns)
{
	const int nv = d + 2;
	return sizeof(double) * (2 * (size_t)ns * ns + (size_t)kDenseWarps * 2 * nv * ns) +
	       sizeof(float) * ((size_t)ns * ns + (size_t)kDenseWarps * nv * ns);
}

void launch_limit_dense(dpg_gpu_ctx* c, double* sol, int n_vol, int ns, const float* sb32, const double* sb64,
                        const double* bs64, float amp, const int* vols, const int64_t* dof_off)
{
	const size_t smem = dense_smem(c->d, ns);
	const int blocks = std::max(1, std::min((n_vol + kDenseWarps - 1) / kDenseWarps, 152 * 8));
	if (smem > 48 * 1024) {   // n_s above 40 (TRI orders above 7)
		if (c->d == 2) cudaFuncSetAttribute(k_positivity_dense<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
		else cudaFuncSetAttribute(k_positivity_dense<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	}
	if (c->d == 2)
		k_positivity_dense<2><<<blocks, kDenseWarps * 32, smem, c->stream>>>(sol, n_vol, ns, sb32, sb64, bs64, amp,
		                                                                    c->pos_err, vols, dof_off);
	else
		k_positivity_dense<3><<<blocks, kDenseWarps * 32, smem, c->stream>>>(sol, n_vol, ns, sb32, sb64, bs64, amp,
		                                                                    c->pos_err, vols, dof_off);
}

template <int D, int N1>
void launch_limit(dpg_gpu_ctx* c, double* sol)
{
	using S = PencilShape<D, N1>;
	PosOps ops{};
	for (int i = 0; i < N1 * N1; ++i) {
		ops.ai32[i] = (float)c->bez1_host[i + 25];
		ops.a64[i] = c->bez1_host[i];
		ops.ai64[i] = c->bez1_host[i + 25];
	}
	double rs = 0.0;
	for (int i = 0; i < N1; ++i) {
		double r = 0.0;
		for (int k = 0; k < N1; ++k) r += std::fabs(c->bez1_host[25 + i * N1 + k]);
		rs = std::max(rs, r);
	}
	ops.rs = (float)(rs * (1.0 + 1e-6));
	const int blocks = (c->g.n_vol + S::EPB - 1) / S::EPB;
	k_positivity<D, N1><<<blocks, S::NT, 0, c->stream>>>(sol, c->g.n_vol, ops, c->pos_amp, c->pos_err);
}

template <int D, int N1>
void launch_relax(dpg_gpu_ctx* c, double* u, const double* du)
{
	using S = PosShape<D, N1>;
	const int blocks = (c->g.n_vol + S::EPB - 1) / S::EPB;
	k_relax_update<D, N1><<<blocks, S::EPB * S::NS, 0, c->stream>>>(u, du, c->g.n_vol, c->bez1_inv, c->pos_err);
}

} // namespace

// (d, points per direction) of the Euler element groups: QUAD and HEX, p = 1..4; simplices: the dense form
int launch_positivity(dpg_gpu_ctx* c, double* sol)
{
	if (!c->positivity) return DPG_OK;
	if (c->pos_dense) {
		if (c->n_pos_grp == 0)
			launch_limit_dense(c, sol, c->g.n_vol, c->g.n_s, c->bez_sb32, c->bez_full, c->bez_bs, c->pos_amp, nullptr,
			                   nullptr);
		for (int k = 0; k < c->n_pos_grp; ++k) {   // mixed orders: one launch per order group
			const dpg_gpu_ctx::PosGroup& g = c->pos_grp[k];
			launch_limit_dense(c, sol, g.n_vol, g.ns, g.sb32, g.sb64, g.bs64, g.amp, g.vols, c->pos_dof_off);
		}
		return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
	}
	const int n1 = c->pos_n1;
	if (c->d == 2 && n1 == 2) launch_limit<2, 2>(c, sol);
	else if (c->d == 2 && n1 == 3) launch_limit<2, 3>(c, sol);
	else if (c->d == 2 && n1 == 4) launch_limit<2, 4>(c, sol);
	else if (c->d == 2 && n1 == 5) launch_limit<2, 5>(c, sol);
	else if (c->d == 3 && n1 == 2) launch_limit<3, 2>(c, sol);
	else if (c->d == 3 && n1 == 3) launch_limit<3, 3>(c, sol);
	else if (c->d == 3 && n1 == 4) launch_limit<3, 4>(c, sol);
	else if (c->d == 3 && n1 == 5) launch_limit<3, 5>(c, sol);
	else return DPG_ERR_UNSUPPORTED;
	return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

int launch_relaxed_update(dpg_gpu_ctx* c, double* u, const double* du)
{
	if (!c->positivity) return DPG_ERR_INVALID;
	if (c->pos_dense) return DPG_ERR_UNSUPPORTED;   // the relaxed Newton update is built for tensor-product volumes
	const int n1 = c->pos_n1;
	if (c->d == 2 && n1 == 2) launch_relax<2, 2>(c, u, du);
	else if (c->d == 2 && n1 == 3) launch_relax<2, 3>(c, u, du);
	else if (c->d == 2 && n1 == 4) launch_relax<2, 4>(c, u, du);
	else if (c->d == 2 && n1 == 5) launch_relax<2, 5>(c, u, du);
	else if (c->d == 3 && n1 == 2) launch_relax<3, 2>(c, u, du);
	else if (c->d == 3 && n1 == 3) launch_relax<3, 3>(c, u, du);
	else if (c->d == 3 && n1 == 4) launch_relax<3, 4>(c, u, du);
	else if (c->d == 3 && n1 == 5) launch_relax<3, 5>(c, u, du);
	else return DPG_ERR_UNSUPPORTED;
	return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

namespace {
__global__ void k_axpy(int64_t n, double a, const double* __restrict__ x, double* __restrict__ y)
{
	for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
		y[i] += a * x[i];
}
} // namespace

int launch_axpy(dpg_gpu_ctx* c, int64_t n, double a, const double* x, double* y)
{
	const int blocks = (int)std::min<int64_t>((n + 255) / 256, 152 * 16);
	k_axpy<<<blocks, 256, 0, c->stream>>>(n, a, x, y);
	return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

int positivity_error(dpg_gpu_ctx* c)
{
	if (!c->pos_err) return 0;
	int e = 0;
	if (cudaMemcpyAsync(&e, c->pos_err, sizeof e, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
	    cudaStreamSynchronize(c->stream) != cudaSuccess)
		return -1;
	if (e && cudaMemsetAsync(c->pos_err, 0, sizeof e, c->stream) != cudaSuccess) return -1;
	return e;
}

} // namespace dpg
