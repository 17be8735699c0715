// Split-precision residual kernels: the DG operator contractions on the tcgen05 tensor cores.
//
// Three precision modes share one kernel structure (DPG_PREC_*):
//   BF16_SLICED : every operand is scaled by a power of two per operator row / per data column and cut into S
//                 signed 8-bit digits; digit s is stored as the BF16 value d * 2^(-8s) (exact).  The digit
//                 products with level a+b < S are accumulated in FP32 in TMEM: one accumulator for each of the
//                 levels 0..3, whose sums are exact (integers times 2^(-8L), |digit| <= 128, K <= 288), and one
//                 for the levels >= 4, whose FP32 rounding is below 2^-56 of the leading level.  The
//                 accumulators are combined in 64-bit integers and converted to FP64 once.  The error is
//                 ~ 2^(-8S) * K * max|row| * max|column|, i.e. FP64-like for S = 6..7.
//   BF16X3      : x = hi + lo in BF16, hi*hi + hi*lo + lo*hi in one FP32 accumulator (~1e-5 relative).
//   TF32X3      : the same with TF32 operands (kind::tf32, ~1e-7 relative).
// Fluxes, geometry, the numerical flux, RK stages and norms stay in FP64 (flux.cuh), exactly as in the FP64 form.
//
// Block = kEB elements, one warp per element; the data operand of a contraction is B (K x N, N = kEB * NV columns
// (element, variable)), the operator is A (M rows <= 128).  K is processed in chunks of 32: lane l of warp e owns K
// row 32*j + l of its element's columns, so per-column scales are warp reductions and the digits of one chunk are
// written by all threads at once.  Operator tiles [chunk][slice] are pre-sliced on the host in the shared-memory
// layout and fetched with cp.async.bulk into a double buffer; the next chunk's tiles are requested as soon as its
// buffer is free.  One elected thread issues all tcgen05.mma; completion is signalled through tcgen05.commit on
// an mbarrier, and every wait is bounded (a timeout sets an error flag read by the host).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "dpg_gpu_internal.cuh"
#include "flux.cuh"
#include "tc_sm100.cuh"

namespace dpg {

constexpr int kEB = 8;          // elements (warps) per block
constexpr int kThreads = 32 * kEB;
constexpr int kMaxS = 7;
constexpr int kAccSliced = 5;   // accumulators: levels 0, 1, 2, 3 and >= 4

struct SplitOp {
	int M_op = 0, M_pad = 0, K_pad = 0, n_chunks = 0, S = 0, es = 2;
	size_t tile_bytes = 0;       // one [slice] tile of M_pad x 32 elements
	uint8_t* tiles = nullptr;    // device: [chunk][slice] tiles
	int* row_exp = nullptr;      // device: [M_pad]
};

struct SplitState {
	int mode = 0, S = 0, fmt = 1, es = 2;
	int n_s_pad = 0, n_c_pad = 0, nf_pad = 0;
	int N_pad_vol = 0, N_pad_tr = 0;
	int tmem_vol = 0, tmem_tr = 0;
	SplitOp cv, cf, lift;
	int* err = nullptr;
	size_t smem_vol = 0, smem_trace = 0;
};

struct SplitArgs {
	const uint8_t* tiles;
	const int* row_exp;
	int M_pad;
	int tile_bytes;
};

// ------------------------------------------------------------------------------------------------------------
// digit / split helpers
// ------------------------------------------------------------------------------------------------------------
__device__ __forceinline__ int exp_bound(double x)
{
	const long long b = __double_as_longlong(x);
	const int be = (int)((b >> 52) & 0x7FF);
	return be == 0 ? -4000 : be - 1022;  // |x| < 2^e
}

__device__ __forceinline__ double pow2(int e)  // e in [-1022, 1023]
{
	return __longlong_as_double((long long)(e + 1023) << 52);
}

// BF16 bits of (u - 128) * 2^(-8s) for u in [0, 256], exactly: the integer is formed on the FP32 add pipe and the
// power of two is applied to the exponent field.
__device__ __forceinline__ uint16_t bf16_digit(int u, int s)
{
	const float f = __int_as_float(0x4B000000 | u) - 8388736.0f;
	const uint32_t b = __float_as_uint(f) >> 16;
	return (uint16_t)(b == 0 ? 0 : b - (uint32_t)(s << 10));
}

__device__ __forceinline__ int clamp_col_exp(int F, int S)
{
	const int lo = 8 * S - 1000, hi = 8 * S + 1000;
	return F < lo ? lo : (F > hi ? hi : F);
}

// Write the digits / split parts of value x for K position kk of column n into the slice tiles of a chunk buffer.
// Sliced mode: scale_exp = 8S - F of the column.
template <int FMT, bool SLICED>
__device__ __forceinline__ void write_parts(uint8_t* buf, int tile_bytes, int S, int n, int kk, double x, int scale_exp)
{
	if constexpr (SLICED) {
		// m = round(x * 2^(8S - F)) from the bits of x with integer operations only (the FP64 pipe is kept for
		// the fluxes): x = +-mant * 2^(be - 1075), so m = +-mant * 2^sh with sh = be - 1075 + 8S - F.
		const long long bits = __double_as_longlong(x);
		const int be = (int)((bits >> 52) & 0x7FF);
		long long m = 0;
		if (be != 0) {
			const long long mant = (bits & 0xFFFFFFFFFFFFFll) | (1ll << 52);
			const int sh = be - 1075 + scale_exp;
			if (sh >= 0) m = mant << sh;
			else if (sh > -63) m = (mant + (1ll << (-sh - 1))) >> (-sh);
			if (bits < 0) m = -m;
		}
		long long C = 0;
		for (int s = 1; s < S; ++s) C |= 128ll << (8 * (S - 1 - s));
		const long long mm = m + C;
		const uint32_t off = tc::kmajor_offset(n, kk, 32, 2);
		const int d0 = (int)(mm >> (8 * (S - 1)));
		*(uint16_t*)(buf + off) = bf16_digit(d0 + 128, 0);
		for (int s = 1; s < S; ++s) {
			const int u = (int)((mm >> (8 * (S - 1 - s))) & 255);
			*(uint16_t*)(buf + s * tile_bytes + off) = bf16_digit(u, s);
		}
	} else if constexpr (FMT == 1) {
		const float xf = (float)x;
		const __nv_bfloat16 hi = __float2bfloat16_rn(xf);
		const __nv_bfloat16 lo = __float2bfloat16_rn(xf - __bfloat162float(hi));
		const uint32_t off = tc::kmajor_offset(n, kk, 32, 2);
		*(__nv_bfloat16*)(buf + off) = hi;
		*(__nv_bfloat16*)(buf + tile_bytes + off) = lo;
	} else {
		const float xf = (float)x;
		uint32_t hi;
		asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(hi) : "f"(xf));
		const float lo_f = xf - __uint_as_float(hi);
		uint32_t lo;
		asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(lo) : "f"(lo_f));
		const uint32_t off = tc::kmajor_offset(n, kk, 32, 4);
		*(uint32_t*)(buf + off) = hi;
		*(uint32_t*)(buf + tile_bytes + off) = lo;
	}
}

// ------------------------------------------------------------------------------------------------------------
// Block GEMM: TMEM accumulators [M_pad x N_pad] = A (operator tiles) * B (digits written from registers), K-chunked.
// ------------------------------------------------------------------------------------------------------------
struct Pipe {
	uint64_t* bar_load;   // [2]
	uint64_t* bar_mma;    // [2]
	uint8_t* abuf[2];
	uint8_t* xbuf[2];
	uint32_t tmem;
	int* err;
	int n_load[2];        // waited phases per barrier (identical in every thread)
	int n_mma[2];
};

__device__ __forceinline__ void pipe_fail(Pipe& p, int code) { atomicExch(p.err, code); }

// All MMAs of one chunk (issued by one thread).  Kept out of line: one copy serves every chunk and kernel phase.
template <int FMT, bool SLICED>
__device__ __noinline__ void issue_chunk_mmas(uint32_t a0, uint32_t b0, int a_tile, int x_tile, int S, int N_pad,
                                              uint32_t tmem, uint32_t idesc, int first_chunk)
{
	const int es = (FMT == 1 ? 2 : 4);
	const uint32_t sbo = 32 * es / 16 * 128;
	for (int ks = 0; ks < es; ++ks) {
		if constexpr (SLICED) {
			for (int a = 0; a < S; ++a)
				for (int b = 0; a + b < S; ++b) {
					const int L = min(a + b, kAccSliced - 1);
					// the first product into accumulator L is (a = 0, b = L) (for the tail: (0, 4))
					const bool first = first_chunk && ks == 0 && a == 0 && b <= kAccSliced - 1;
					const uint64_t ad = tc::make_sdesc(a0 + (uint32_t)(a * a_tile) + ks * 256, 128, sbo);
					const uint64_t bd = tc::make_sdesc(b0 + (uint32_t)(b * x_tile) + ks * 256, 128, sbo);
					tc::mma_bf16(tmem + (uint32_t)(L * N_pad), ad, bd, idesc, first ? 0u : 1u);
				}
		} else {
			const int pa[3] = {0, 0, 1}, pb[3] = {0, 1, 0};
			for (int q = 0; q < 3; ++q) {
				const bool first = first_chunk && ks == 0 && q == 0;
				const uint64_t ad = tc::make_sdesc(a0 + (uint32_t)(pa[q] * a_tile) + ks * 256, 128, sbo);
				const uint64_t bd = tc::make_sdesc(b0 + (uint32_t)(pb[q] * x_tile) + ks * 256, 128, sbo);
				if constexpr (FMT == 1) tc::mma_bf16(tmem, ad, bd, idesc, first ? 0u : 1u);
				else tc::mma_tf32(tmem, ad, bd, idesc, first ? 0u : 1u);
			}
		}
	}
}

__device__ __forceinline__ void request_chunk(Pipe& p, const SplitArgs& A, int nparts, int c, int buf)
{
	const uint32_t bytes = (uint32_t)(A.tile_bytes * nparts);
	tc::mbar_expect_tx(&p.bar_load[buf], bytes);
	tc::bulk_g2s(p.abuf[buf], A.tiles + (size_t)c * A.tile_bytes * nparts, bytes, &p.bar_load[buf]);
}

template <int NV, int KCH, int FMT, bool SLICED>
__device__ void block_gemm(Pipe& p, const SplitArgs& A, int S, int N_pad, const double (&xv)[KCH][NV],
                           const int (&scale_exp)[NV], int e_local)
{
	const int tid = threadIdx.x, lane = tid & 31;
	const int es = (FMT == 1 ? 2 : 4);
	const int xtile = N_pad * 32 * es;
	const int nparts = SLICED ? S : 2;
	const uint32_t idesc = tc::make_idesc(A.M_pad, N_pad, FMT);
	// chunk 0 of this GEMM always uses buffer 0; the previous GEMM of the block has fully completed
	if (tid == 0) request_chunk(p, A, nparts, 0, 0);
	for (int c = 0; c < KCH; ++c) {
		const int buf = c & 1;
		// digits of chunk c (its buffer was released before this chunk's tiles were requested, see below)
#pragma unroll
		for (int v = 0; v < NV; ++v) {
			double x = 0.0;
#pragma unroll
			for (int q = 0; q < KCH; ++q)
				if (q == c) x = xv[q][v];
			write_parts<FMT, SLICED>(p.xbuf[buf], xtile, S, e_local * NV + v, lane, x, scale_exp[v]);
		}
		tc::fence_async_smem();
		tc::fence_before_sync();
		__syncthreads();
		if (tid < 32) {
			// warp 0 stays converged around the single-thread issue so that no lane of the issuing warp spins on
			// a barrier while lane 0 issues
			if (tid == 0) {
				tc::fence_after_sync();
				if (!tc::mbar_wait(&p.bar_load[buf], (uint32_t)(p.n_load[buf] & 1))) pipe_fail(p, 3);
				issue_chunk_mmas<FMT, SLICED>(tc::smem_u32(p.abuf[buf]), tc::smem_u32(p.xbuf[buf]), A.tile_bytes, xtile,
				                             S, N_pad, p.tmem, idesc, c == 0);
				tc::mma_commit(&p.bar_mma[buf]);
			}
			__syncwarp();
		}
		++p.n_load[buf];
		// release the other buffer: MMAs of chunk c-1 must be done before chunk c+1 overwrites it
		if (c + 1 < KCH) {
			const int nb = buf ^ 1;
			if (c >= 1) {
				if (!tc::mbar_wait(&p.bar_mma[nb], (uint32_t)(p.n_mma[nb] & 1))) pipe_fail(p, 2);
				++p.n_mma[nb];
			}
			if (tid < 32) {
				if (tid == 0) request_chunk(p, A, nparts, c + 1, nb);
				__syncwarp();
			}
		}
	}
	// drain: the last two commits (one per buffer in use) are still unconsumed
	const int last = (KCH - 1) & 1;
	if (KCH >= 2) {
		if (!tc::mbar_wait(&p.bar_mma[last ^ 1], (uint32_t)(p.n_mma[last ^ 1] & 1))) pipe_fail(p, 4);
		++p.n_mma[last ^ 1];
	}
	if (!tc::mbar_wait(&p.bar_mma[last], (uint32_t)(p.n_mma[last] & 1))) pipe_fail(p, 5);
	++p.n_mma[last];
	tc::fence_after_sync();
}

// Row of the accumulator held by (warp, lane) for M_pad rows (TMEM layouts of cta_group::1: M = 128 -> lane = row,
// M = 64 -> rows 16w..16w+15 in lanes 0..15 of sub-partition w).  -1 when the lane holds no row.
__device__ __forceinline__ int acc_row(int M_pad, int warp, int lane)
{
	const int w = warp & 3;
	if (M_pad == 128) return 32 * w + lane;
	return lane < 16 ? 16 * w + lane : -1;
}

// Combine the accumulators of (row, column chunk c8) into 8 FP64 values (before the row/column scaling 2^(e+F-48)).
// nacc = min(S, 5) accumulators were written (levels >= S do not exist).
template <bool SLICED>
__device__ __forceinline__ void read_combine(uint32_t tmem_row, int N_pad, int c8, int nacc, double* out8)
{
	if constexpr (SLICED) {
#pragma unroll
		for (int h = 0; h < 2; ++h) {
			float a[kAccSliced][4];
#pragma unroll
			for (int L = 0; L < kAccSliced; ++L) {
				if (L < nacc) {
					tc::tmem_ld4(tmem_row + (uint32_t)(L * N_pad + 8 * c8 + 4 * h), a[L]);
				} else {
#pragma unroll
					for (int j = 0; j < 4; ++j) a[L][j] = 0.f;
				}
			}
			tc::tmem_ld_wait();
#pragma unroll
			for (int j = 0; j < 4; ++j) {
				long long V = 0;
#pragma unroll
				for (int L = 0; L < kAccSliced; ++L) V += __float2ll_rn(a[L][j] * 4294967296.0f);  // units of 2^-32
				out8[4 * h + j] = (double)V;
			}
		}
	} else {
		float a[8];
		tc::tmem_ld8(tmem_row + (uint32_t)(8 * c8), a);
		tc::tmem_ld_wait();
#pragma unroll
		for (int j = 0; j < 8; ++j) out8[j] = (double)a[j];
	}
}

struct SmemLayout {
	uint8_t* abuf[2];
	uint8_t* xbuf[2];
	double* sS;
	int* colF;     // [kEB * 8]
	uint64_t* bars;
	uint32_t* tmem_slot;
};

__device__ __forceinline__ SmemLayout carve(uint8_t* sm, size_t abuf_bytes, size_t xbuf_bytes, int n_s_vals)
{
	SmemLayout L;
	size_t off = 0;
	L.abuf[0] = sm + off; off += abuf_bytes;
	L.abuf[1] = sm + off; off += abuf_bytes;
	L.xbuf[0] = sm + off; off += xbuf_bytes;
	L.xbuf[1] = sm + off; off += xbuf_bytes;
	L.sS = (double*)(sm + off); off += sizeof(double) * n_s_vals;
	L.colF = (int*)(sm + off); off += sizeof(int) * kEB * 8;
	off = (off + 15) & ~(size_t)15;
	L.bars = (uint64_t*)(sm + off); off += sizeof(uint64_t) * 4;
	L.tmem_slot = (uint32_t*)(sm + off);
	return L;
}

__device__ __forceinline__ void pipe_init(Pipe& p, const SmemLayout& L, int* err, int tmem_cols, size_t xbuf_bytes)
{
	const int tid = threadIdx.x;
	p.bar_load = L.bars;
	p.bar_mma = L.bars + 2;
	p.abuf[0] = L.abuf[0]; p.abuf[1] = L.abuf[1];
	p.xbuf[0] = L.xbuf[0]; p.xbuf[1] = L.xbuf[1];
	p.err = err;
	p.n_load[0] = p.n_load[1] = p.n_mma[0] = p.n_mma[1] = 0;
	// zero the digit buffers once: padding columns are never written again
	for (size_t i = (size_t)tid * 16; i < 2 * xbuf_bytes; i += kThreads * 16)
		*(uint4*)(L.xbuf[0] + i) = make_uint4(0, 0, 0, 0);
	if (tid < 32) { tc::tmem_alloc(L.tmem_slot, (uint32_t)tmem_cols); tc::tmem_relinquish(); }
	if (tid == 0) {
		for (int i = 0; i < 4; ++i) tc::mbar_init(&L.bars[i], 1);
		tc::fence_mbar_init();
	}
	tc::fence_async_smem();
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	p.tmem = *L.tmem_slot;
}

__device__ __forceinline__ void pipe_finish(const Pipe& p, int tmem_cols)
{
	tc::fence_before_sync();
	__syncthreads();
	if (threadIdx.x < 32) tc::tmem_dealloc(p.tmem, (uint32_t)tmem_cols);
}

// per-column scale: warp max of the exponents of the lane's values for each variable
template <int NV, int KCH>
__device__ __forceinline__ void column_scales(const double (&xv)[KCH][NV], int S, int (&scale_exp)[NV], int (&F)[NV])
{
#pragma unroll
	for (int v = 0; v < NV; ++v) {
		int e = -4000;
#pragma unroll
		for (int c = 0; c < KCH; ++c) e = max(e, exp_bound(xv[c][v]));
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
		int Fv = (e < -3000 ? 0 : e + 1);
		Fv = clamp_col_exp(Fv, S);
		F[v] = Fv;
		scale_exp[v] = 8 * S - Fv;
	}
}

// Scale a combined accumulator value by 2^(row_exp + col_exp - 16 - 32) (sliced mode) through its exponent field.
__device__ __forceinline__ double scale_out(double y, int re, int F)
{
	if (y == 0.0) return 0.0;
	return __longlong_as_double(__double_as_longlong(y) + ((long long)(re + F - 48) << 52));
}

// ------------------------------------------------------------------------------------------------------------
// trace kernel
// ------------------------------------------------------------------------------------------------------------
template <int NV, int KCH_S, int FMT, bool SLICED>
__global__ void __launch_bounds__(kThreads, 1)
ks_trace(const double* __restrict__ sol, GroupDev g, double* __restrict__ trace, SplitArgs Acf, int S, int N_pad,
         int tmem_cols, size_t abuf_bytes, size_t xbuf_bytes, int* err)
{
	extern __shared__ __align__(1024) uint8_t sm[];
	const SmemLayout L = carve(sm, abuf_bytes, xbuf_bytes, 0);
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int n_s = g.n_s, n_fl = g.n_fl, n_fc = g.n_fc;
	const int e_glob = blockIdx.x * kEB + warp;
	const bool valid = e_glob < g.n_vol;
	Pipe p;
	pipe_init(p, L, err, tmem_cols, xbuf_bytes);

	double xv[KCH_S][NV];
#pragma unroll
	for (int c = 0; c < KCH_S; ++c)
#pragma unroll
		for (int v = 0; v < NV; ++v) {
			const int k = 32 * c + lane;
			xv[c][v] = (valid && k < n_s) ? sol[((size_t)e_glob * NV + v) * n_s + k] : 0.0;
		}
	int scale[NV];
	int F[NV];
	column_scales<NV, KCH_S>(xv, S, scale, F);
	if (SLICED && lane == 0)
		for (int v = 0; v < NV; ++v) L.colF[warp * NV + v] = F[v];
	block_gemm<NV, KCH_S, FMT, SLICED>(p, Acf, S, N_pad, xv, scale, warp);
	__syncthreads();

	const int row = acc_row(Acf.M_pad, warp, lane);
	const int rows_valid = n_fl * n_fc;
	const int e0 = blockIdx.x * kEB;
	const uint32_t trow = p.tmem + ((uint32_t)(32 * (warp & 3)) << 16);
	const int re = (SLICED && row >= 0 && row < rows_valid) ? Acf.row_exp[row] : 0;
	for (int c8 = (warp >> 2); c8 < N_pad / 8; c8 += 2) {
		double vals[8];
		read_combine<SLICED>(trow, N_pad, c8, min(S, kAccSliced), vals);
		if (row < 0 || row >= rows_valid) continue;
		const int lf = row / n_fc, q = row - lf * n_fc;
#pragma unroll
		for (int j = 0; j < 8; ++j) {
			const int n = 8 * c8 + j;
			const int el = n / NV, v = n - el * NV;
			if (el >= kEB || e0 + el >= g.n_vol) continue;
			double y = vals[j];
			if constexpr (SLICED) y = scale_out(y, re, L.colF[el * NV + v]);
			const int vf = g.vol_face[(size_t)(e0 + el) * n_fl + lf];
			trace[((size_t)vf * NV + v) * n_fc + q] = y;
		}
	}
	pipe_finish(p, tmem_cols);
}

// ------------------------------------------------------------------------------------------------------------
// volume kernel
// ------------------------------------------------------------------------------------------------------------
template <int D, int NV, int KCH_S, int KCH_L, int FMT, bool SLICED>
__global__ void __launch_bounds__(kThreads, 1)
ks_volume(double* __restrict__ sol, double* __restrict__ solp, double* __restrict__ rhs,
          const double* __restrict__ nnf, GroupDev g, SplitArgs Acv, SplitArgs Alift, int S, int N_pad, int tmem_cols,
          size_t abuf_bytes, size_t xbuf_bytes, int n_c_pad, const double* __restrict__ dt_ptr,
          unsigned long long* max_slot, int stage, int write_rhs, double bx, double by, double bz, int* err)
{
	extern __shared__ __align__(1024) uint8_t sm[];
	const int n_s = g.n_s, n_c = g.n_c, n_fl = g.n_fl, n_fc = g.n_fc;
	const SmemLayout L = carve(sm, abuf_bytes, xbuf_bytes, kEB * NV * n_c_pad);
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int e0 = blockIdx.x * kEB;
	const int e_glob = e0 + warp;
	const bool valid = e_glob < g.n_vol;
	Pipe p;
	pipe_init(p, L, err, tmem_cols, xbuf_bytes);

	// 1. state of the warp's element
	double uv[KCH_S][NV];
#pragma unroll
	for (int c = 0; c < KCH_S; ++c)
#pragma unroll
		for (int v = 0; v < NV; ++v) {
			const int k = 32 * c + lane;
			uv[c][v] = (valid && k < n_s) ? sol[((size_t)e_glob * NV + v) * n_s + k] : 0.0;
		}
	int scale[NV];
	int F[NV];
	column_scales<NV, KCH_S>(uv, S, scale, F);
	if (SLICED && lane == 0)
		for (int v = 0; v < NV; ++v) L.colF[warp * NV + v] = F[v];

	// 2. s_vc = cv0_vs_vc * sol_coef
	block_gemm<NV, KCH_S, FMT, SLICED>(p, Acv, S, N_pad, uv, scale, warp);
	__syncthreads();
	{
		const int row = acc_row(Acv.M_pad, warp, lane);
		const uint32_t trow = p.tmem + ((uint32_t)(32 * (warp & 3)) << 16);
		const int re = (SLICED && row >= 0 && row < n_c) ? Acv.row_exp[row] : 0;
		for (int c8 = (warp >> 2); c8 < N_pad / 8; c8 += 2) {
			double vals[8];
			read_combine<SLICED>(trow, N_pad, c8, min(S, kAccSliced), vals);
			if (row < 0 || row >= n_c) continue;
#pragma unroll
			for (int j = 0; j < 8; ++j) {
				const int n = 8 * c8 + j;
				if (n >= kEB * NV) continue;
				double y = vals[j];
				if constexpr (SLICED) y = scale_out(y, re, L.colF[n]);
				L.sS[n * n_c_pad + row] = y;
			}
		}
	}
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();

	// 3. reference fluxes at the volume nodes and gathered face fluxes -> lift operand (registers)
	double xv[KCH_L][NV];
	const int ch_r = n_c_pad / 32;
	double m[D][D];
#pragma unroll
	for (int x = 0; x < D; ++x)
#pragma unroll
		for (int r = 0; r < D; ++r) m[x][r] = valid ? g.met[(size_t)e_glob * D * D + x + D * r] : 0.0;
#pragma unroll
	for (int j = 0; j < KCH_L; ++j)
#pragma unroll
		for (int v = 0; v < NV; ++v) xv[j][v] = 0.0;
	for (int jc = 0; jc < ch_r; ++jc) {
		const int c = 32 * jc + lane;
		if (!valid || c >= n_c) continue;
		double s[NV];
#pragma unroll
		for (int v = 0; v < NV; ++v) s[v] = L.sS[(warp * NV + v) * n_c_pad + c];
		double fr[D][NV];
		if constexpr (NV == D + 2) {
			double f[D][D + 2];
			flux_euler<D>(s, f);
#pragma unroll
			for (int r = 0; r < D; ++r)
#pragma unroll
				for (int eq = 0; eq < NV; ++eq) {
					double acc = 0.0;
#pragma unroll
					for (int x = 0; x < D; ++x) acc += m[x][r] * f[x][eq];
					fr[r][eq] = acc;
				}
		} else {
			const double b[3] = {bx, by, bz};
#pragma unroll
			for (int r = 0; r < D; ++r) {
				double acc = 0.0;
#pragma unroll
				for (int x = 0; x < D; ++x) acc += m[x][r] * (b[x] * s[0]);
				fr[r][0] = acc;
			}
		}
#pragma unroll
		for (int q = 0; q < KCH_L; ++q)
#pragma unroll
			for (int r = 0; r < D; ++r)
				if (q == r * ch_r + jc)
#pragma unroll
					for (int eq = 0; eq < NV; ++eq) xv[q][eq] = fr[r][eq];
	}
	const int nfq = n_fl * n_fc;
	const int ch_f = KCH_L - D * ch_r;
	for (int jf = 0; jf < ch_f; ++jf) {
		const int fq = 32 * jf + lane;
		if (!valid || fq >= nfq) continue;
		const int lf = fq / n_fc, q = fq - lf * n_fc;
		const int vf = g.vol_face[(size_t)e_glob * n_fl + lf];
		const int f = vf >> 1, side = vf & 1;
		const int qs = side ? g.nc_inv[(size_t)f * n_fc + q] : q;
		const double sgn = side ? -1.0 : 1.0;
		double val[NV];
#pragma unroll
		for (int v = 0; v < NV; ++v) val[v] = sgn * nnf[((size_t)f * NV + v) * n_fc + qs];
#pragma unroll
		for (int qq = 0; qq < KCH_L; ++qq)
			if (qq == D * ch_r + jf)
#pragma unroll
				for (int v = 0; v < NV; ++v) xv[qq][v] = val[v];
	}
	column_scales<NV, KCH_L>(xv, S, scale, F);
	__syncthreads();   // colF of the interpolation is no longer read
	if (SLICED && lane == 0)
		for (int v = 0; v < NV; ++v) L.colF[warp * NV + v] = F[v];

	// 4. lift: rhs = L' * [fr ; nnf]   (L' = m_inv_ref [tw1 | -tw0]; affine elements: times 1/detJ)
	block_gemm<NV, KCH_L, FMT, SLICED>(p, Alift, S, N_pad, xv, scale, warp);
	__syncthreads();
	const double dt = (stage >= 0 ? *dt_ptr : 0.0);
	double lmax = 0.0;
	{
		const int row = acc_row(Alift.M_pad, warp, lane);
		const uint32_t trow = p.tmem + ((uint32_t)(32 * (warp & 3)) << 16);
		const int re = (SLICED && row >= 0 && row < n_s) ? Alift.row_exp[row] : 0;
		for (int c8 = (warp >> 2); c8 < N_pad / 8; c8 += 2) {
			double vals[8];
			read_combine<SLICED>(trow, N_pad, c8, min(S, kAccSliced), vals);
			if (row < 0 || row >= n_s) continue;
#pragma unroll
			for (int j = 0; j < 8; ++j) {
				const int n = 8 * c8 + j;
				const int el = n / NV, v = n - el * NV;
				if (el >= kEB || e0 + el >= g.n_vol) continue;
				double r = vals[j];
				if constexpr (SLICED) r = scale_out(r, re, L.colF[n]);
				r *= g.jinv[e0 + el];
				lmax = fmax(lmax, fabs(r));
				if (isnan(r)) lmax = r;
				const size_t gi = ((size_t)(e0 + el) * NV + v) * n_s + row;
				if (write_rhs) rhs[gi] = r;
				if (stage >= 0) {
					const double u0 = sol[gi];
					if (stage == 0) { solp[gi] = u0; sol[gi] = u0 + dt * r; }
					else if (stage == 1) sol[gi] = (1.0 / 4.0) * (3.0 * solp[gi] + u0 + dt * r);
					else sol[gi] = (1.0 / 3.0) * (solp[gi] + 2.0 * u0 + 2.0 * dt * r);
				}
			}
		}
	}
	for (int off = 16; off > 0; off >>= 1) {
		const double other = __shfl_xor_sync(0xffffffffu, lmax, off);
		lmax = (isnan(other) || other > lmax) ? other : lmax;
	}
	if (lane == 0) atomicMax(max_slot, (unsigned long long)__double_as_longlong(fabs(lmax)));
	pipe_finish(p, tmem_cols);
}

// ------------------------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------------------------
static int host_exp_bound(double x)
{
	if (x == 0.0) return -4000;
	int e;
	std::frexp(std::fabs(x), &e);   // |x| = f * 2^e, f in [0.5, 1)  ->  |x| < 2^e
	return e;
}

static uint16_t host_bf16(float f)
{
	uint32_t u;
	memcpy(&u, &f, 4);
	const uint32_t r = u + 0x7FFF + ((u >> 16) & 1);
	return (uint16_t)(r >> 16);
}

// Slice an operator [M_op x K_real] (row-major, K column k placed at kmap[k] of the padded K) into device tiles.
static int build_split_op(SplitOp& op, const std::vector<double>& Aop, int M_op, int K_real, const std::vector<int>& kmap,
                          int K_pad, int mode, int S, int es)
{
	op.M_op = M_op;
	if (M_op > 128) return DPG_ERR_UNSUPPORTED;
	op.M_pad = (M_op <= 64 ? 64 : 128);
	op.K_pad = K_pad;
	op.n_chunks = K_pad / 32;
	op.S = (mode == DPG_PREC_BF16_SLICED ? S : 2);
	op.es = es;
	op.tile_bytes = (size_t)op.M_pad * 32 * es;
	std::vector<uint8_t> tiles(op.tile_bytes * op.S * op.n_chunks, 0);
	std::vector<int> rexp(op.M_pad, 0);
	for (int i = 0; i < M_op; ++i) {
		double mx = 0.0;
		for (int k = 0; k < K_real; ++k) mx = std::fmax(mx, std::fabs(Aop[(size_t)i * K_real + k]));
		const int E = (mx == 0.0 ? 0 : host_exp_bound(mx) + 1);   // |A_ik| 2^-E < 1/2
		rexp[i] = E;
		for (int k = 0; k < K_real; ++k) {
			const double a = Aop[(size_t)i * K_real + k];
			const int kp = kmap[k];
			const int c = kp / 32, kk = kp % 32;
			const size_t base = ((size_t)c * op.S) * op.tile_bytes;
			const uint32_t o = dpg::tc::kmajor_offset(i, kk, 32, es);
			if (mode == DPG_PREC_BF16_SLICED) {
				const long long m = std::llrint(std::ldexp(a, 8 * S - E));
				long long C = 0;
				for (int s = 1; s < S; ++s) C |= 128ll << (8 * (S - 1 - s));
				const long long mm = m + C;
				for (int s = 0; s < S; ++s) {
					const int d = (s == 0) ? (int)(mm >> (8 * (S - 1))) : (int)((mm >> (8 * (S - 1 - s))) & 255) - 128;
					const uint16_t bs = host_bf16((float)std::ldexp((double)d, -8 * s));
					memcpy(&tiles[base + s * op.tile_bytes + o], &bs, 2);
				}
			} else if (mode == DPG_PREC_BF16X3) {
				const float af = (float)a;
				const uint16_t hi = host_bf16(af);
				uint32_t hu = (uint32_t)hi << 16;
				float hf;
				memcpy(&hf, &hu, 4);
				const uint16_t lo = host_bf16(af - hf);
				memcpy(&tiles[base + o], &hi, 2);
				memcpy(&tiles[base + op.tile_bytes + o], &lo, 2);
			} else {
				const float af = (float)a;
				uint32_t u;
				memcpy(&u, &af, 4);
				const uint32_t hi = (u + 0x1000u) & 0xFFFFE000u;   // round half away from zero to TF32
				float hf;
				memcpy(&hf, &hi, 4);
				const float lf = af - hf;
				uint32_t ul;
				memcpy(&ul, &lf, 4);
				const uint32_t lo = (ul + 0x1000u) & 0xFFFFE000u;
				memcpy(&tiles[base + o], &hi, 4);
				memcpy(&tiles[base + op.tile_bytes + o], &lo, 4);
			}
		}
	}
	if (cudaMalloc(&op.tiles, tiles.size()) != cudaSuccess) return DPG_ERR_CUDA;
	if (cudaMemcpy(op.tiles, tiles.data(), tiles.size(), cudaMemcpyHostToDevice) != cudaSuccess) return DPG_ERR_CUDA;
	if (cudaMalloc(&op.row_exp, sizeof(int) * op.M_pad) != cudaSuccess) return DPG_ERR_CUDA;
	if (cudaMemcpy(op.row_exp, rexp.data(), sizeof(int) * op.M_pad, cudaMemcpyHostToDevice) != cudaSuccess)
		return DPG_ERR_CUDA;
	return DPG_OK;
}

static void free_op(SplitOp& op)
{
	if (op.tiles) cudaFree(op.tiles);
	if (op.row_exp) cudaFree(op.row_exp);
	op.tiles = nullptr;
	op.row_exp = nullptr;
}

void split_free(dpg_gpu_ctx* c)
{
	SplitState* st = (SplitState*)c->split;
	if (!st) return;
	free_op(st->cv); free_op(st->cf); free_op(st->lift);
	if (st->err) cudaFree(st->err);
	delete st;
	c->split = nullptr;
}

static SplitArgs args_of(const SplitOp& op) { return SplitArgs{op.tiles, op.row_exp, op.M_pad, (int)op.tile_bytes}; }

struct KernelPair { void* vol; void* tr; };

template <int D, int NV, int KS, int KL, int FMT, bool SL>
static KernelPair kernels_of() { return KernelPair{(void*)ks_volume<D, NV, KS, KL, FMT, SL>, (void*)ks_trace<NV, KS, FMT, SL>}; }

// The (d, NV, K chunks) combinations instantiated: Euler/advection on QUAD p1..4 and HEX p1..3.
#define DPG_SPLIT_CASES(X)  \
	X(3, 5, 2, 9)  /* HEX p3 Euler  */ \
	X(3, 5, 1, 5)  /* HEX p2 Euler  */ \
	X(3, 5, 1, 4)  /* HEX p1 Euler  */ \
	X(2, 4, 1, 3)  /* QUAD p1..4 Euler */ \
	X(2, 1, 1, 3)  /* QUAD advection */ \
	X(3, 1, 2, 9)  /* HEX p3 advection */ \
	X(3, 1, 1, 5)  /* HEX p2 advection */

template <int FMT, bool SL>
static KernelPair pick(int d, int nv, int ks, int kl)
{
#define DPG_PICK(D_, NV_, KS_, KL_) if (d == D_ && nv == NV_ && ks == KS_ && kl == KL_) return kernels_of<D_, NV_, KS_, KL_, FMT, SL>();
	DPG_SPLIT_CASES(DPG_PICK)
#undef DPG_PICK
	return KernelPair{nullptr, nullptr};
}

static KernelPair pick_all(int mode, int d, int nv, int ks, int kl)
{
	if (mode == DPG_PREC_BF16_SLICED) return pick<1, true>(d, nv, ks, kl);
	if (mode == DPG_PREC_BF16X3) return pick<1, false>(d, nv, ks, kl);
	return pick<2, false>(d, nv, ks, kl);
}

static int pow2_cols(int n)
{
	int t = 32;
	while (t < n) t <<= 1;
	return t;
}

int split_prepare(dpg_gpu_ctx* c)
{
	split_free(c);
	const GroupDev& g = c->g;
	if (!g.affine) return DPG_ERR_UNSUPPORTED;  // per-element m_inv on the split path: not provided
	SplitState* st = new SplitState();
	c->split = st;
	st->mode = c->prec_mode;
	st->S = (st->mode == DPG_PREC_BF16_SLICED ? c->n_slices : 2);
	if (st->mode == DPG_PREC_BF16_SLICED && (st->S < 2 || st->S > kMaxS)) { split_free(c); return DPG_ERR_INVALID; }
	st->fmt = (st->mode == DPG_PREC_TF32X3 ? 2 : 1);
	st->es = (st->fmt == 1 ? 2 : 4);
	const int d = c->d, NV = c->n_var;
	const int n_s = g.n_s, n_c = g.n_c, n_fl = g.n_fl, n_fc = g.n_fc;
	st->n_s_pad = (n_s + 31) / 32 * 32;
	st->n_c_pad = (n_c + 31) / 32 * 32;
	st->nf_pad = (n_fl * n_fc + 31) / 32 * 32;
	const int KS = st->n_s_pad / 32;
	const int KL = (d * st->n_c_pad + st->nf_pad) / 32;
	KernelPair kp = pick_all(st->mode, d, NV, KS, KL);
	if (!kp.vol) { split_free(c); return DPG_ERR_UNSUPPORTED; }

	// host copies of the FP64 operators (as uploaded for the FP64 form)
	std::vector<double> Cv((size_t)n_c * n_s), Cf((size_t)n_fl * n_fc * n_s), Lm((size_t)n_s * g.K);
	if (cudaMemcpy(Cv.data(), g.Cv, sizeof(double) * Cv.size(), cudaMemcpyDeviceToHost) ||
	    cudaMemcpy(Cf.data(), g.Cf, sizeof(double) * Cf.size(), cudaMemcpyDeviceToHost) ||
	    cudaMemcpy(Lm.data(), g.L, sizeof(double) * Lm.size(), cudaMemcpyDeviceToHost)) { split_free(c); return DPG_ERR_CUDA; }
	std::vector<int> kmap_s(n_s), kmap_l(g.K);
	for (int k = 0; k < n_s; ++k) kmap_s[k] = k;
	for (int r = 0; r < d; ++r)
		for (int cc = 0; cc < n_c; ++cc) kmap_l[r * n_c + cc] = r * st->n_c_pad + cc;
	for (int fq = 0; fq < n_fl * n_fc; ++fq) kmap_l[d * n_c + fq] = d * st->n_c_pad + fq;
	int rc;
	if ((rc = build_split_op(st->cv, Cv, n_c, n_s, kmap_s, st->n_s_pad, st->mode, st->S, st->es))) { split_free(c); return rc; }
	if ((rc = build_split_op(st->cf, Cf, n_fl * n_fc, n_s, kmap_s, st->n_s_pad, st->mode, st->S, st->es))) { split_free(c); return rc; }
	if ((rc = build_split_op(st->lift, Lm, n_s, g.K, kmap_l, 32 * KL, st->mode, st->S, st->es))) { split_free(c); return rc; }
	if (cudaMalloc(&st->err, sizeof(int)) != cudaSuccess || cudaMemset(st->err, 0, sizeof(int)) != cudaSuccess) {
		split_free(c);
		return DPG_ERR_CUDA;
	}
	// column padding: M = 64 MMAs take N in steps of 8, M = 128 in steps of 16
	const int N = kEB * NV;
	const bool vol64 = st->cv.M_pad == 64 && st->lift.M_pad == 64;
	st->N_pad_vol = vol64 ? (N + 7) / 8 * 8 : (N + 15) / 16 * 16;
	st->N_pad_tr = st->cf.M_pad == 64 ? (N + 7) / 8 * 8 : (N + 15) / 16 * 16;
	const int nacc = (st->mode == DPG_PREC_BF16_SLICED ? kAccSliced : 1);
	st->tmem_vol = pow2_cols(nacc * st->N_pad_vol);
	st->tmem_tr = pow2_cols(nacc * st->N_pad_tr);
	if (st->tmem_vol > 512 || st->tmem_tr > 512) { split_free(c); return DPG_ERR_UNSUPPORTED; }
	const int nparts = st->S;
	const size_t xbuf_vol = (size_t)nparts * st->N_pad_vol * 32 * st->es;
	const size_t xbuf_tr = (size_t)nparts * st->N_pad_tr * 32 * st->es;
	const size_t abuf_vol = (size_t)nparts * std::max(st->cv.tile_bytes, st->lift.tile_bytes);
	const size_t abuf_tr = (size_t)nparts * st->cf.tile_bytes;
	const size_t tail = sizeof(int) * kEB * 8 + 16 + sizeof(uint64_t) * 4 + 16;
	st->smem_vol = 2 * abuf_vol + 2 * xbuf_vol + sizeof(double) * kEB * NV * st->n_c_pad + tail;
	st->smem_trace = 2 * abuf_tr + 2 * xbuf_tr + tail;
	if (st->smem_vol > 227 * 1024 || st->smem_trace > 227 * 1024) { split_free(c); return DPG_ERR_UNSUPPORTED; }
	if (cudaFuncSetAttribute(kp.vol, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)st->smem_vol) ||
	    cudaFuncSetAttribute(kp.tr, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)st->smem_trace)) {
		split_free(c);
		return DPG_ERR_CUDA;
	}
	return DPG_OK;
}

template <int D, int NV, int KS, int KL, int FMT, bool SL>
static void launch_pair(dpg_gpu_ctx* c, SplitState* st, bool trace_kernel, int stage, bool write_rhs,
                        unsigned long long* max_slot)
{
	const GroupDev& g = c->g;
	const int grid = (g.n_vol + kEB - 1) / kEB;
	if (trace_kernel) {
		const size_t xbuf = (size_t)st->S * st->N_pad_tr * 32 * st->es;
		const size_t abuf = (size_t)st->S * st->cf.tile_bytes;
		ks_trace<NV, KS, FMT, SL><<<grid, kThreads, st->smem_trace, c->stream>>>(
		    c->sol, g, c->trace, args_of(st->cf), st->S, st->N_pad_tr, st->tmem_tr, abuf, xbuf, st->err);
	} else {
		const size_t xbuf = (size_t)st->S * st->N_pad_vol * 32 * st->es;
		const size_t abuf = (size_t)st->S * std::max(st->cv.tile_bytes, st->lift.tile_bytes);
		ks_volume<D, NV, KS, KL, FMT, SL><<<grid, kThreads, st->smem_vol, c->stream>>>(
		    c->sol, c->solp, c->rhs, c->nnf, g, args_of(st->cv), args_of(st->lift), st->S, st->N_pad_vol, st->tmem_vol,
		    abuf, xbuf, st->n_c_pad, c->ddt, max_slot, stage, write_rhs ? 1 : 0, c->b_adv[0], c->b_adv[1],
		    c->b_adv[2], st->err);
	}
}

template <int FMT, bool SL>
static int launch_sel(dpg_gpu_ctx* c, SplitState* st, bool trace_kernel, int stage, bool write_rhs,
                      unsigned long long* max_slot)
{
	const int d = c->d, nv = c->n_var, ks = st->n_s_pad / 32, kl = (d * st->n_c_pad + st->nf_pad) / 32;
#define DPG_LAUNCH(D_, NV_, KS_, KL_) \
	if (d == D_ && nv == NV_ && ks == KS_ && kl == KL_) { launch_pair<D_, NV_, KS_, KL_, FMT, SL>(c, st, trace_kernel, stage, write_rhs, max_slot); return DPG_OK; }
	DPG_SPLIT_CASES(DPG_LAUNCH)
#undef DPG_LAUNCH
	return DPG_ERR_UNSUPPORTED;
}

static int launch_any(dpg_gpu_ctx* c, bool trace_kernel, int stage, bool write_rhs, unsigned long long* max_slot)
{
	SplitState* st = (SplitState*)c->split;
	if (!st) return DPG_ERR_INVALID;
	int rc;
	if (st->mode == DPG_PREC_BF16_SLICED) rc = launch_sel<1, true>(c, st, trace_kernel, stage, write_rhs, max_slot);
	else if (st->mode == DPG_PREC_BF16X3) rc = launch_sel<1, false>(c, st, trace_kernel, stage, write_rhs, max_slot);
	else rc = launch_sel<2, false>(c, st, trace_kernel, stage, write_rhs, max_slot);
	if (rc) return rc;
	return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

int split_launch_trace(dpg_gpu_ctx* c) { return launch_any(c, true, -1, false, nullptr); }
int split_launch_volume(dpg_gpu_ctx* c, int stage, bool write_rhs, unsigned long long* max_slot)
{
	return launch_any(c, false, stage, write_rhs, max_slot);
}

int split_error(dpg_gpu_ctx* c)
{
	SplitState* st = (SplitState*)c->split;
	if (!st) return 0;
	int e = 0;
	cudaMemcpy(&e, st->err, sizeof(int), cudaMemcpyDeviceToHost);
	return e;
}

} // namespace dpg
