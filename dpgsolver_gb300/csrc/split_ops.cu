// Split-precision residual kernels: the DG operator contractions on the tcgen05 tensor cores.
//
// Three precision modes share one kernel structure (DPG_PREC_*):
//   BF16_SLICED : every operand is scaled by a power of two per operator row / per data column and cut into S
//                 signed 8-bit digits; digit s is stored as the BF16 value d * 2^(-8s) (exact).  The digit
//                 products with level a+b < S are accumulated in FP32 in TMEM: one accumulator for each of the
//                 levels 0..3 and one for the levels >= 4.  Level sums are integers times 2^(-8L) below 2^24 in
//                 those units (exact) except in a contrived worst case of level 3 at K = 288, where the FP32
//                 rounding is 2^-48 of the leading level, like the tail accumulator's.  The accumulators are
//                 combined in 64-bit integers and converted to FP64 once.  The error is
//                 ~ 2^(-8S) * K * max|row| * max|column|, i.e. FP64-like for S = 6..7.
//   BF16X3      : x = hi + lo in BF16, hi*hi + hi*lo + lo*hi in one FP32 accumulator (~1e-5 relative).
//   TF32X3      : the same with TF32 operands (kind::tf32, ~1e-7 relative).
// Fluxes, geometry, the numerical flux, RK stages and norms stay in FP64 (flux.cuh), as in the FP64 form.
//
// Shapes.  One tcgen05.mma (K = 16) occupies the tensor pipe for max(64, N/2) cycles whatever M <= 128 and
// N <= 128 are, so every contraction is laid out for M = 128: the data operand (A) has one row per (element,
// variable) of a block of EB elements (EB * NV <= 128), the operator slice (B) one row per operator row (N = 64
// for the volume interpolation and the lift, 96 for the face interpolation of HEX p=3).  TMEM holds the
// accumulators [128 lanes = data rows][N columns] x 5 levels; one block per SM owns all 512 columns.
//
// Kernels of one residual (split path):
//   ks_interp : sol_coef -> digits (kept for both contractions) -> s_vc = Cv * U (TMEM) -> FP64 reference volume
//               fluxes written to global memory with a per-column exponent bound, while the tensor pipe runs
//               U_fc = Cf * U -> face traces (coalesced through shared memory)
//   ks_face   : numerical flux per face node (FP64, as the FP64 form) and a per-(face, variable) exponent bound
//   ks_lift   : digits of [face fluxes | reference volume fluxes] streamed chunk by chunk from global memory
//               (column scales known from the two exponent bounds), rhs = L' * X (TMEM), 1/detJ, ||rhs||_inf and
//               the SSP-RK3 stage update through a coalesced epilogue.
// Operator tiles [chunk][slice] are pre-sliced on the host in the shared-memory layout and streamed with
// cp.async.bulk through a ring; one warp issues the MMAs (warp-uniform, elect.sync), completion is signalled by
// tcgen05.commit on mbarriers and every wait is bounded (a timeout sets an error flag read by the host).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "dpg_gpu_internal.cuh"
#include "flux.cuh"
#include "tc_sm100.cuh"

namespace dpg {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kRows = 128;      // data rows (element, variable) of one block: the MMA M
constexpr int kMaxS = 7;
constexpr int kAccSliced = 5;   // accumulators: levels 0, 1, 2, 3 and >= 4
constexpr int kRingMax = 6;     // operator ring stages (at most)
constexpr int kSmemMax = 227 * 1024;
constexpr int kSmemOneBlock = 116 * 1024;   // requests at least this much: one block per SM (512 TMEM columns)

struct SplitOp {
	int N_op = 0, N_pad = 0, K_pad = 0, n_chunks = 0, S = 0, es = 2;
	size_t tile_bytes = 0;       // one [slice] tile of N_pad rows x 32 K
	uint8_t* tiles = nullptr;    // device: [chunk][slice] tiles
	int* row_exp = nullptr;      // device: [N_pad]
};

struct SplitArgs {
	const uint8_t* tiles;
	const int* row_exp;
	int N_pad;
	int tile_bytes;
};

// Shared-memory plan of one kernel (computed on the host).
struct Plan {
	int nst, stage_bytes;        // operator ring
	int part_bytes, chunk_bytes; // data digits: one part (128 rows x 32 K) and one chunk (all parts)
	int off_dig, off_st, off_colF, off_bars;
	int smem_bytes;
};

struct SplitState {
	int mode = 0, S = 0, fmt = 1, es = 2;
	int n_s_pad = 0, n_c_pad = 0, nf_pad = 0;
	int EB = 0, n_blocks = 0, n_face_warps = 0;
	SplitOp cv, cf, lift;
	Plan pi{}, pl{};
	double* xfr = nullptr;       // [n_vol][NV][d * n_c_pad] reference volume fluxes (lift operand)
	int* colE = nullptr;         // [n_vol][NV] exponent bound of xfr per column
	int* face_exp = nullptr;     // [n_face][NV] exponent bound of the scaled numerical flux
	int* err = nullptr;
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

__device__ __forceinline__ int clamp_col_exp(int F, int S)
{
	const int lo = 8 * S - 1000, hi = 8 * S + 1000;
	return F < lo ? lo : (F > hi ? hi : F);
}

// Column scale F (|x| 2^-F < 1/2) from the largest exponent bound of the column.
__device__ __forceinline__ int col_exp_of(int emax, int S) { return clamp_col_exp(emax < -3000 ? 0 : emax + 1, S); }

// round(x * 2^sc) from the bits of x with integer operations only (the FP64 pipe is kept for the fluxes):
// x = +-mant * 2^(be - 1075), so the result is +-mant * 2^(be - 1075 + sc) (|result| < 2^(8S-1) by the choice of sc).
__device__ __forceinline__ long long scaled_mantissa(double x, int sc)
{
	const long long bits = __double_as_longlong(x);
	const int be = (int)((bits >> 52) & 0x7FF);
	if (be == 0) return 0;
	const long long mant = (bits & 0xFFFFFFFFFFFFFll) | (1ll << 52);
	const int sh = be - 1075 + sc;
	long long m = 0;
	if (sh >= 0) m = mant << sh;
	else if (sh > -63) m = (mant + (1ll << (-sh - 1))) >> (-sh);
	return bits < 0 ? -m : m;
}

// offset that turns the digits below the leading one into unsigned bytes (balanced digits in [-128, 127])
__device__ __forceinline__ long long digit_bias(int S)
{
	long long C = 0;
	for (int s = 1; s < S; ++s) C |= 128ll << (8 * (S - 1 - s));
	return C;
}

// Digit s of the biased integer mm as the float (d) * 2^(-8s), exactly: the integer d = u - 128 is formed on the
// FP32 add pipe from the byte u (the leading digit is biased by +128 here), then scaled by a power of two.
__device__ __forceinline__ float digit_f32(long long mm, int s, int S)
{
	const int u = (s == 0) ? (int)(mm >> (8 * (S - 1))) + 128 : (int)((mm >> (8 * (S - 1 - s))) & 255);
	const float d = __int_as_float(0x4B000000 | u) - 8388736.0f;
	return d * __int_as_float((127 - 8 * s) << 23);
}

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi)
{
	const __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
	return *(const uint32_t*)&p;
}

__device__ __forceinline__ uint32_t tf32_bits(float x)
{
	uint32_t r;
	asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
	return r;
}

// Digits / split parts of 8 consecutive K values (kk0 .. kk0+7 of a 32-K chunk) of data row m, written as one
// 16-byte core-matrix row per part (two for TF32).  Eight consecutive threads taking eight consecutive rows of one
// K group fill one whole 128-byte core matrix (conflict-free).  F = column scale (sliced mode).
template <int FMT, bool SLICED>
__device__ __forceinline__ void store_digits8(uint8_t* chunk, int part_bytes, int m, int kk0, const double (&x)[8], int F,
                                              int S)
{
	if constexpr (SLICED) {
		const int sc = 8 * S - F;
		const long long C = digit_bias(S);
		long long mm[8];
#pragma unroll
		for (int j = 0; j < 8; ++j) mm[j] = scaled_mantissa(x[j], sc) + C;
		uint8_t* dst = chunk + tc::kmajor_offset(m, kk0, 32, 2);
		for (int s = 0; s < S; ++s) {
			uint4 w;
			w.x = pack_bf16x2(digit_f32(mm[0], s, S), digit_f32(mm[1], s, S));
			w.y = pack_bf16x2(digit_f32(mm[2], s, S), digit_f32(mm[3], s, S));
			w.z = pack_bf16x2(digit_f32(mm[4], s, S), digit_f32(mm[5], s, S));
			w.w = pack_bf16x2(digit_f32(mm[6], s, S), digit_f32(mm[7], s, S));
			*(uint4*)(dst + s * part_bytes) = w;
		}
	} else if constexpr (FMT == 1) {
		float hi[8], lo[8];
#pragma unroll
		for (int j = 0; j < 8; ++j) {
			const float xf = (float)x[j];
			hi[j] = __bfloat162float(__float2bfloat16_rn(xf));
			lo[j] = xf - hi[j];
		}
		uint8_t* dst = chunk + tc::kmajor_offset(m, kk0, 32, 2);
		*(uint4*)dst = make_uint4(pack_bf16x2(hi[0], hi[1]), pack_bf16x2(hi[2], hi[3]), pack_bf16x2(hi[4], hi[5]),
		                          pack_bf16x2(hi[6], hi[7]));
		*(uint4*)(dst + part_bytes) = make_uint4(pack_bf16x2(lo[0], lo[1]), pack_bf16x2(lo[2], lo[3]),
		                                         pack_bf16x2(lo[4], lo[5]), pack_bf16x2(lo[6], lo[7]));
	} else {
		uint32_t hi[8], lo[8];
#pragma unroll
		for (int j = 0; j < 8; ++j) {
			const float xf = (float)x[j];
			hi[j] = tf32_bits(xf);
			lo[j] = tf32_bits(xf - __uint_as_float(hi[j]));
		}
#pragma unroll
		for (int h = 0; h < 2; ++h) {
			uint8_t* dst = chunk + tc::kmajor_offset(m, kk0 + 4 * h, 32, 4);
			*(uint4*)dst = make_uint4(hi[4 * h], hi[4 * h + 1], hi[4 * h + 2], hi[4 * h + 3]);
			*(uint4*)(dst + part_bytes) = make_uint4(lo[4 * h], lo[4 * h + 1], lo[4 * h + 2], lo[4 * h + 3]);
		}
	}
}

// ------------------------------------------------------------------------------------------------------------
// Contraction engine: operator ring, digit-chunk hand-off, TMEM accumulators [128 x N_pad] x levels.
// The operator tiles of all contractions of a kernel form one sequence t = 0..T-1 (tile t uses stage t % nst).
// ------------------------------------------------------------------------------------------------------------
struct Eng {
	uint8_t* ring;
	int nst, stage_bytes;
	uint8_t* dig;        // digit chunks: chunk buffer b at dig + b * chunk_bytes
	int part_bytes, chunk_bytes;
	uint64_t* full;      // [nst]  tile landed (expect_tx)
	uint64_t* empty;     // [nst]  MMAs reading the stage done (tcgen05.commit)
	uint64_t* xready;    // [2]    all threads wrote the chunk's digits
	uint64_t* xfree;     // [2]    MMAs of the chunk done (tcgen05.commit)
	uint64_t* done;      //        a whole contraction done (tcgen05.commit)
	uint32_t tmem;
	int* err;
	const uint8_t* src0;
	const uint8_t* src1;
	int tb0, tb1, T0, T;
	int n_req;           // tiles requested (issuing warp)
	int q, consumed;     // double-buffered chunks started / releases waited for (identical in every thread)
};

__device__ __forceinline__ void eng_fail(const Eng& E, int code) { atomicExch(E.err, code); }

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
	asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(bar)) : "memory");
}

// Issuing warp (all lanes, converged): load tile t into its ring stage (one elected lane issues the copy).
__device__ __forceinline__ void eng_load(Eng& E, int t)
{
	const int st = t % E.nst;
	const uint8_t* src = t < E.T0 ? E.src0 + (size_t)t * E.tb0 : E.src1 + (size_t)(t - E.T0) * E.tb1;
	const uint32_t bytes = (uint32_t)(t < E.T0 ? E.tb0 : E.tb1);
	if (tc::elect_one()) {
		tc::mbar_expect_tx(&E.full[st], bytes);
		tc::bulk_g2s(E.ring + (size_t)st * E.stage_bytes, src, bytes, &E.full[st]);
	}
	__syncwarp();
}

// Issuing warp: request every tile below lim, waiting for its stage to be free (tile t reuses the stage of tile
// t - nst).
__device__ __forceinline__ void eng_request(Eng& E, int lim)
{
	if (lim > E.T) lim = E.T;
	while (E.n_req < lim) {
		const int t = E.n_req;
		if (t >= E.nst && !tc::mbar_wait(&E.empty[t % E.nst], (uint32_t)((t / E.nst - 1) & 1))) eng_fail(E, 1);
		eng_load(E, t);
		++E.n_req;
	}
}

// Issuing warp: request the tiles below lim whose stage is already free, without waiting.
__device__ __forceinline__ void eng_request_ready(Eng& E, int lim)
{
	if (lim > E.T) lim = E.T;
	while (E.n_req < lim) {
		const int t = E.n_req;
		if (t >= E.nst && !tc::mbar_test(&E.empty[t % E.nst], (uint32_t)((t / E.nst - 1) & 1))) return;
		eng_load(E, t);
		++E.n_req;
	}
}

__device__ __forceinline__ void eng_init(Eng& E, uint8_t* sm, const Plan& P, int* err, const SplitArgs& A0, int T0,
                                         const SplitArgs& A1, int T1)
{
	const int tid = threadIdx.x;
	E.ring = sm;
	E.nst = P.nst;
	E.stage_bytes = P.stage_bytes;
	E.dig = sm + P.off_dig;
	E.part_bytes = P.part_bytes;
	E.chunk_bytes = P.chunk_bytes;
	uint64_t* bars = (uint64_t*)(sm + P.off_bars);
	E.full = bars;
	E.empty = bars + P.nst;
	E.xready = bars + 2 * P.nst;
	E.xfree = bars + 2 * P.nst + 2;
	E.done = bars + 2 * P.nst + 4;
	uint32_t* slot = (uint32_t*)(bars + 2 * P.nst + 5);
	E.err = err;
	E.src0 = A0.tiles; E.tb0 = A0.tile_bytes; E.T0 = T0;
	E.src1 = A1.tiles; E.tb1 = A1.tile_bytes; E.T = T0 + T1;
	E.n_req = 0;
	E.q = 0;
	E.consumed = 0;
	if (tid < 32) { tc::tmem_alloc(slot, 512u); tc::tmem_relinquish(); }
	if (tid == 0) {
		for (int i = 0; i < P.nst; ++i) { tc::mbar_init(&E.full[i], 1); tc::mbar_init(&E.empty[i], 1); }
		for (int i = 0; i < 2; ++i) { tc::mbar_init(&E.xready[i], kThreads); tc::mbar_init(&E.xfree[i], 1); }
		tc::mbar_init(E.done, 1);
		tc::fence_mbar_init();
	}
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	E.tmem = *slot;
	if (tid < 32) eng_request(E, E.nst);
}

// Issuing warp: all MMAs of one data chunk (digits at shared address dig_addr) against the operator tiles
// g0 .. g0 + nparts - 1 of the sequence: operator slice a times data part b with a + b < S, accumulator min(a+b, 4).
// Descriptors are formed once and advanced by adding 16-byte-unit offsets to their address field.
template <int FMT, bool SLICED>
__device__ __forceinline__ void eng_issue_chunk(Eng& E, uint32_t dig_addr, int g0, bool first, int S, int N_pad,
                                                uint32_t idesc)
{
	constexpr int es = (FMT == 1 ? 2 : 4);
	constexpr uint32_t sbo = 32 * es / 16 * 128;
	const int nparts = SLICED ? S : 2;
	const uint64_t xd0 = tc::make_sdesc(dig_addr, 128, sbo);
	const uint64_t ad_ring = tc::make_sdesc(tc::smem_u32(E.ring), 128, sbo);
	const uint32_t pstep = (uint32_t)E.part_bytes >> 4;
	for (int a = 0; a < nparts; ++a) {
		const int g = g0 + a, st = g % E.nst;
		eng_request(E, g + 1);
		if (!tc::mbar_wait(&E.full[st], (uint32_t)((g / E.nst) & 1))) eng_fail(E, 3);
		tc::fence_after_sync();
		const uint64_t od = ad_ring + (uint64_t)((uint32_t)(st * E.stage_bytes) >> 4);
		const int nb = SLICED ? S - a : (a == 0 ? 2 : 1);
#pragma unroll
		for (int ks = 0; ks < es; ++ks) {
			for (int b = 0; b < nb; ++b) {
				const int L = SLICED ? min(a + b, kAccSliced - 1) : 0;
				// the first product into accumulator L is (a = 0, b = L) (for the tail: (0, 4)); unsliced: (0, 0)
				const bool init = first && ks == 0 && a == 0 && (SLICED ? b <= kAccSliced - 1 : b == 0);
				const uint64_t dd = xd0 + (uint64_t)(b * pstep + 16 * ks);
				if constexpr (FMT == 1) tc::mma_bf16_elect(E.tmem + (uint32_t)(L * N_pad), dd, od + 16 * ks, idesc, init ? 0u : 1u);
				else tc::mma_tf32_elect(E.tmem + (uint32_t)(L * N_pad), dd, od + 16 * ks, idesc, init ? 0u : 1u);
			}
		}
		tc::mma_commit_elect(&E.empty[st]);
		eng_request_ready(E, g + E.nst);   // refill every stage whose MMAs already completed
	}
}

// All threads: wait for phase `ph` of the contraction-done barrier.
__device__ __forceinline__ void eng_wait_done(Eng& E, int ph)
{
	if (!tc::mbar_wait(E.done, (uint32_t)(ph & 1))) eng_fail(E, 5);
	tc::fence_after_sync();
}

// Double-buffered chunks (lift).  All threads: wait until the MMAs of chunk q-2 released the buffer chunk q
// writes; returns that buffer.
__device__ __forceinline__ uint8_t* eng_begin_chunk(Eng& E)
{
	while (E.consumed <= E.q - 2) {
		if (!tc::mbar_wait(&E.xfree[E.consumed & 1], (uint32_t)((E.consumed >> 1) & 1))) eng_fail(E, 2);
		++E.consumed;
	}
	return E.dig + (E.q & 1) * E.chunk_bytes;
}

// All threads, after writing chunk q's digits: publish them; warp 0 issues the chunk's MMAs and commits its
// release.
template <int FMT, bool SLICED>
__device__ __forceinline__ void eng_end_chunk(Eng& E, int g0, bool first, int S, int N_pad, uint32_t idesc)
{
	tc::fence_async_smem();
	tc::fence_before_sync();
	mbar_arrive(&E.xready[E.q & 1]);
	if (threadIdx.x < 32) {
		__syncwarp();
		if (!tc::mbar_wait(&E.xready[E.q & 1], (uint32_t)((E.q >> 1) & 1))) eng_fail(E, 6);
		tc::fence_after_sync();
		eng_issue_chunk<FMT, SLICED>(E, tc::smem_u32(E.dig + (E.q & 1) * E.chunk_bytes), g0, first, S, N_pad, idesc);
		tc::mma_commit_elect(&E.xfree[E.q & 1]);
		__syncwarp();
	}
	++E.q;
}

// All threads: wait until every issued chunk's MMAs completed (accumulators final).
__device__ __forceinline__ void eng_drain(Eng& E)
{
	while (E.consumed < E.q) {
		if (!tc::mbar_wait(&E.xfree[E.consumed & 1], (uint32_t)((E.consumed >> 1) & 1))) eng_fail(E, 4);
		++E.consumed;
	}
	tc::fence_after_sync();
}

__device__ __forceinline__ void eng_finish(const Eng& E)
{
	tc::fence_before_sync();
	__syncthreads();
	if (threadIdx.x < 32) tc::tmem_dealloc(E.tmem, 512u);
}

// Eight accumulator columns c0..c0+7 of this thread's TMEM lane combined into FP64 (before the row/column scaling
// 2^(e+F-48) in sliced mode).  nacc = min(S, 5) accumulators were written (levels >= S do not exist).
template <bool SLICED>
__device__ __forceinline__ void combine8(uint32_t trow, int N_pad, int c0, int nacc, double (&out)[8])
{
	if constexpr (SLICED) {
		float a[kAccSliced][8];
#pragma unroll
		for (int L = 0; L < kAccSliced; ++L) {
			if (L < nacc) {
				tc::tmem_ld8(trow + (uint32_t)(L * N_pad + c0), a[L]);
			} else {
#pragma unroll
				for (int j = 0; j < 8; ++j) a[L][j] = 0.f;
			}
		}
		tc::tmem_ld_wait();
#pragma unroll
		for (int j = 0; j < 8; ++j) {
			// accumulator L times 2^(8L) is an integer below 2^25 in magnitude (the tail: rounded to one), so
			// 32-bit conversions suffice; the sum is formed in units of 2^-32
			long long V = 0;
#pragma unroll
			for (int L = 0; L < kAccSliced; ++L)
				V += (long long)__float2int_rn(a[L][j] * __int_as_float((127 + 8 * L) << 23)) << (32 - 8 * L);
			out[j] = (double)V;
		}
	} else {
		float a[8];
		tc::tmem_ld8(trow + (uint32_t)c0, a);
		tc::tmem_ld_wait();
#pragma unroll
		for (int j = 0; j < 8; ++j) out[j] = (double)a[j];
	}
}

// Scale a combined accumulator value by 2^(row_exp + col_exp - 16 - 32) (sliced mode) through its exponent field.
__device__ __forceinline__ double scale_out(double y, int re, int F)
{
	if (y == 0.0) return 0.0;
	return __longlong_as_double(__double_as_longlong(y) + ((long long)(re + F - 48) << 52));
}

// Reference-space volume flux fr[r][eq] = sum_x m[x][r] f[x][eq] (m_xr = detJ dr/dx, the cofactor metrics).
// Euler: the contraction is taken through W_r = sum_x m[x][r] u_x (fewer FP64 operations than forming f first;
// same value up to rounding).
template <int D, int NV>
__device__ __forceinline__ void ref_flux(const double* s, const double (&m)[D][D], const double* b, double (&fr)[D][NV])
{
	if constexpr (NV == D + 2) {
		const double rho_inv = 1.0 / s[0], E = s[D + 1];
		double u[D], V2 = 0.0;
#pragma unroll
		for (int a = 0; a < D; ++a) { u[a] = s[1 + a] * rho_inv; V2 += u[a] * u[a]; }
		const double p = DPG_GM1_D * (E - 0.5 * s[0] * V2), Ep = E + p;
#pragma unroll
		for (int r = 0; r < D; ++r) {
			double W = 0.0, f0 = 0.0;
#pragma unroll
			for (int x = 0; x < D; ++x) { W += m[x][r] * u[x]; f0 += m[x][r] * s[1 + x]; }
			fr[r][0] = f0;
#pragma unroll
			for (int a = 0; a < D; ++a) fr[r][1 + a] = s[1 + a] * W + m[a][r] * p;
			fr[r][D + 1] = Ep * W;
		}
	} else {
#pragma unroll
		for (int r = 0; r < D; ++r) {
			double acc = 0.0;
#pragma unroll
			for (int x = 0; x < D; ++x) acc += m[x][r] * (b[x] * s[0]);
			fr[r][0] = acc;
		}
	}
}

// ------------------------------------------------------------------------------------------------------------
// ks_interp: traces and reference volume fluxes of a block of EB elements
// ------------------------------------------------------------------------------------------------------------
template <int D, int NV, int KS, int FMT, bool SLICED>
__global__ void __launch_bounds__(kThreads, 1)
ks_interp(const double* __restrict__ sol, GroupDev g, double* __restrict__ trace, double* __restrict__ xfr,
          int* __restrict__ colE, SplitArgs Acv, SplitArgs Acf, Plan P, int S, int EB, int n_c_pad, double bx,
          double by, double bz, int* err)
{
	extern __shared__ __align__(1024) uint8_t sm[];
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int n_s = g.n_s, n_c = g.n_c, n_fl = g.n_fl, n_fc = g.n_fc;
	const int e0 = blockIdx.x * EB, ne = min(EB, g.n_vol - e0), rows = ne * NV;
	const int nparts = SLICED ? S : 2, nacc = SLICED ? min(S, kAccSliced) : 1;
	constexpr int G = 4 * KS;             // groups of 8 K per solution column
	constexpr int ld_u = 32 * KS + 2;     // staged solution: +2 doubles keep the 16-byte reads conflict-free
	double* ST = (double*)(sm + P.off_st);
	int* colF = (int*)(sm + P.off_colF);
	Eng E;
	eng_init(E, sm, P, err, Acv, KS * nparts, Acf, KS * nparts);

	// 1. solution coefficients of the block (contiguous in memory) -> staging, column scales
	const double* src = sol + (size_t)e0 * NV * n_s;
	for (int i = tid; i < kRows * G; i += kThreads) {
		const int m = i / G, kg = i - m * G;   // G consecutive threads share a column
		double x[8];
		int e = -4000;
#pragma unroll
		for (int j = 0; j < 8; ++j) {
			const int k = 8 * kg + j;
			x[j] = (m < rows && k < n_s) ? src[(size_t)m * n_s + k] : 0.0;
			e = max(e, exp_bound(x[j]));
		}
#pragma unroll
		for (int j = 0; j < 4; ++j) *(double2*)(ST + m * ld_u + 8 * kg + 2 * j) = make_double2(x[2 * j], x[2 * j + 1]);
#pragma unroll
		for (int o = 1; o < G; o <<= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, o));
		if (kg == 0) colF[m] = col_exp_of(e, S);
	}
	__syncthreads();
	// 2. digits of all solution chunks (kept for both contractions)
	for (int i = tid; i < kRows * G; i += kThreads) {
		const int m = i & (kRows - 1), kg = i >> 7;
		double x[8];
#pragma unroll
		for (int j = 0; j < 4; ++j) {
			const double2 t = *(const double2*)(ST + m * ld_u + 8 * kg + 2 * j);
			x[2 * j] = t.x; x[2 * j + 1] = t.y;
		}
		store_digits8<FMT, SLICED>(E.dig + (kg >> 2) * P.chunk_bytes, P.part_bytes, m, 8 * (kg & 3), x, colF[m], S);
	}
	tc::fence_async_smem();
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();

	// 3. s_vc = Cv * U
	if (warp == 0) {
		const uint32_t idesc = tc::make_idesc(kRows, Acv.N_pad, FMT);
		for (int c = 0; c < KS; ++c)
			eng_issue_chunk<FMT, SLICED>(E, tc::smem_u32(E.dig + c * P.chunk_bytes), c * nparts, c == 0, S, Acv.N_pad, idesc);
		tc::mma_commit_elect(E.done);
		__syncwarp();
	}
	eng_wait_done(E, 0);
	const int ld_v = n_c_pad + 1;         // odd: the row-per-lane stores below are conflict-free
	const int m_t = 32 * (warp & 3) + lane;
	const uint32_t trow = E.tmem + ((uint32_t)(32 * (warp & 3)) << 16);
	for (int c8 = warp >> 2; c8 < Acv.N_pad / 8; c8 += 2) {
		double v8[8];
		combine8<SLICED>(trow, Acv.N_pad, 8 * c8, nacc, v8);
#pragma unroll
		for (int j = 0; j < 8; ++j) {
			const int node = 8 * c8 + j;
			if (node >= n_c) continue;
			double y = v8[j];
			if constexpr (SLICED) y = scale_out(y, Acv.row_exp[node], colF[m_t]);
			ST[m_t * ld_v + node] = y;
		}
	}
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();

	// 4. U_fc = Cf * U on the tensor pipe (same digits) while the volume fluxes are computed
	if (warp == 0) {
		const uint32_t idesc = tc::make_idesc(kRows, Acf.N_pad, FMT);
		for (int c = 0; c < KS; ++c)
			eng_issue_chunk<FMT, SLICED>(E, tc::smem_u32(E.dig + c * P.chunk_bytes), KS * nparts + c * nparts, c == 0, S,
			                             Acf.N_pad, idesc);
		tc::mma_commit_elect(E.done);
		__syncwarp();
	}

	// 5. reference volume fluxes -> global lift operand [element][variable][r * n_c_pad + node], exponent bounds
	const int KFR = D * n_c_pad;
	const double b[3] = {bx, by, bz};
	for (int el = warp; el < ne; el += kWarps) {
		const int e = e0 + el;
		double m[D][D];
#pragma unroll
		for (int x = 0; x < D; ++x)
#pragma unroll
			for (int r = 0; r < D; ++r) m[x][r] = g.met[(size_t)e * D * D + x + D * r];
		int emax[NV];
#pragma unroll
		for (int v = 0; v < NV; ++v) emax[v] = -4000;
		for (int c = lane; c < n_c_pad; c += 32) {
			double fr[D][NV];
			if (c < n_c) {
				double s[NV];
#pragma unroll
				for (int v = 0; v < NV; ++v) s[v] = ST[(el * NV + v) * ld_v + c];
				ref_flux<D, NV>(s, m, b, fr);
			} else {
#pragma unroll
				for (int r = 0; r < D; ++r)
#pragma unroll
					for (int v = 0; v < NV; ++v) fr[r][v] = 0.0;
			}
#pragma unroll
			for (int r = 0; r < D; ++r)
#pragma unroll
				for (int v = 0; v < NV; ++v) {
					xfr[((size_t)e * NV + v) * KFR + r * n_c_pad + c] = fr[r][v];
					emax[v] = max(emax[v], exp_bound(fr[r][v]));
				}
		}
#pragma unroll
		for (int v = 0; v < NV; ++v) {
			int ev = emax[v];
#pragma unroll
			for (int o = 16; o > 0; o >>= 1) ev = max(ev, __shfl_xor_sync(0xffffffffu, ev, o));
			if (lane == 0) colE[(size_t)e * NV + v] = ev;
		}
	}

	// 6. traces: TMEM -> shared staging (the digits are dead once the face contraction completed) -> the
	//    face-ordered trace buffer, one contiguous [NV][n_fc] run per (element, local face)
	eng_wait_done(E, 1);
	double* TS = (double*)E.dig;
	const int ld_t = Acf.N_pad + 1;
	const int nfq = n_fl * n_fc;
	for (int c8 = warp >> 2; c8 < Acf.N_pad / 8; c8 += 2) {
		double v8[8];
		combine8<SLICED>(trow, Acf.N_pad, 8 * c8, nacc, v8);
#pragma unroll
		for (int j = 0; j < 8; ++j) {
			const int fq = 8 * c8 + j;
			if (fq >= nfq) continue;
			double y = v8[j];
			if constexpr (SLICED) y = scale_out(y, Acf.row_exp[fq], colF[m_t]);
			TS[m_t * ld_t + fq] = y;
		}
	}
	__syncthreads();
	const int per_face = NV * n_fc;
	for (int i = tid; i < ne * n_fl * per_face; i += kThreads) {
		const int el = i / (n_fl * per_face), r = i - el * n_fl * per_face;
		const int lf = r / per_face, r2 = r - lf * per_face;
		const int v = r2 / n_fc, q = r2 - v * n_fc;
		const int vf = g.vol_face[(size_t)(e0 + el) * n_fl + lf];
		trace[((size_t)vf * NV + v) * n_fc + q] = TS[(el * NV + v) * ld_t + lf * n_fc + q];
	}
	eng_finish(E);
}

// ------------------------------------------------------------------------------------------------------------
// ks_face: numerical flux at every face node (as k_face of the FP64 form) and per-(face, variable) exponent bounds
// of the scaled flux.  32 / n_fc faces per warp, so a face's nodes are consecutive lanes of one warp.
// ------------------------------------------------------------------------------------------------------------
template <int D, int NV>
__global__ void __launch_bounds__(256) ks_face(const double* __restrict__ trace, FaceDev fd, double* __restrict__ nnf,
                                               int* __restrict__ face_exp, int num_flux, double bx, double by, double bz)
{
	const int n_fc = fd.n_fc, fpw = 32 / n_fc;
	const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
	const int f = gw * fpw + lane / n_fc, q = lane - (lane / n_fc) * n_fc;
	const bool active = lane < fpw * n_fc && f < fd.n_face;
	double nf[NV];
#pragma unroll
	for (int v = 0; v < NV; ++v) nf[v] = 0.0;
	if (active) {
		const int t = f * n_fc + q;
		const int qr = fd.nc[t];
		double WL[NV], WR[NV], n[D];
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
		for (int v = 0; v < NV; ++v) {
			nf[v] *= j;
			nnf[((size_t)f * NV + v) * n_fc + q] = nf[v];
		}
	}
#pragma unroll
	for (int v = 0; v < NV; ++v) {
		int e = active ? exp_bound(nf[v]) : -4000;
		for (int off = 1; off < n_fc; off <<= 1) {
			const int o = __shfl_down_sync(0xffffffffu, e, off);
			if (q + off < n_fc) e = max(e, o);
		}
		if (active && q == 0) face_exp[(size_t)f * NV + v] = e;
	}
}

// ------------------------------------------------------------------------------------------------------------
// ks_lift: rhs = L' * [nnf ; fr] of a block of EB elements, 1/detJ, RK stage update, ||rhs||_inf
// (L' = m_inv_ref [-tw0 | tw1] with K ordered face part first)
// ------------------------------------------------------------------------------------------------------------
template <int D, int NV, int KF>
__device__ __forceinline__ void lift_load(double (&xv)[2][8], int c, const double* __restrict__ nnf,
                                          const double* __restrict__ xfr, const GroupDev& g, int e0, int rows, int KFR)
{
	const int n_fl = g.n_fl, n_fc = g.n_fc, nfq = n_fl * n_fc;
#pragma unroll
	for (int j = 0; j < 2; ++j) {
		const int i = threadIdx.x + kThreads * j;
		const int m = i & (kRows - 1), kg = i >> 7;
		if (c < KF) {
			const int el = m / NV, v = m - el * NV;
#pragma unroll
			for (int jj = 0; jj < 8; ++jj) {
				const int fq = 32 * c + 8 * kg + jj;
				double x = 0.0;
				if (m < rows && fq < nfq) {
					const int lf = fq / n_fc, qq = fq - lf * n_fc;
					const int vf = g.vol_face[(size_t)(e0 + el) * n_fl + lf];
					const int f = vf >> 1;
					const int qs = (vf & 1) ? g.nc_inv[(size_t)f * n_fc + qq] : qq;
					x = nnf[((size_t)f * NV + v) * n_fc + qs];
					if (vf & 1) x = -x;
				}
				xv[j][jj] = x;
			}
		} else if (m < rows) {
			const double2* p = (const double2*)(xfr + ((size_t)e0 * NV + m) * KFR + 32 * (c - KF) + 8 * kg);
#pragma unroll
			for (int h = 0; h < 4; ++h) { const double2 t = p[h]; xv[j][2 * h] = t.x; xv[j][2 * h + 1] = t.y; }
		} else {
#pragma unroll
			for (int jj = 0; jj < 8; ++jj) xv[j][jj] = 0.0;
		}
	}
}

template <int D, int NV, int KF, int FMT, bool SLICED>
__global__ void __launch_bounds__(kThreads, 1)
ks_lift(double* __restrict__ sol, double* __restrict__ solp, double* __restrict__ rhs, const double* __restrict__ nnf,
        const int* __restrict__ face_exp, const double* __restrict__ xfr, const int* __restrict__ colE, GroupDev g,
        SplitArgs Al, Plan P, int S, int EB, int n_c_pad, const double* __restrict__ dt_ptr,
        unsigned long long* max_slot, int stage, int write_rhs, int* err)
{
	extern __shared__ __align__(1024) uint8_t sm[];
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int n_s = g.n_s, n_fl = g.n_fl;
	const int e0 = blockIdx.x * EB, ne = min(EB, g.n_vol - e0), rows = ne * NV;
	const int nparts = SLICED ? S : 2, nacc = SLICED ? min(S, kAccSliced) : 1;
	const int KFR = D * n_c_pad, KL = KF + KFR / 32;
	int* colF = (int*)(sm + P.off_colF);
	Eng E;
	eng_init(E, sm, P, err, Al, KL * nparts, Al, 0);

	// column scales from the two exponent bounds: the element's reference fluxes and its faces' fluxes
	for (int m = tid; m < kRows; m += kThreads) {
		int F = 0;
		if (m < rows) {
			const int el = m / NV, v = m - el * NV;
			int e = colE[(size_t)(e0 + el) * NV + v];
			for (int lf = 0; lf < n_fl; ++lf) {
				const int f = g.vol_face[(size_t)(e0 + el) * n_fl + lf] >> 1;
				e = max(e, face_exp[(size_t)f * NV + v]);
			}
			F = col_exp_of(e, S);
		}
		colF[m] = F;
	}
	__syncthreads();

	const uint32_t idesc = tc::make_idesc(kRows, Al.N_pad, FMT);
	double xv[2][8];
	lift_load<D, NV, KF>(xv, 0, nnf, xfr, g, e0, rows, KFR);
	for (int c = 0; c < KL; ++c) {
		uint8_t* xb = eng_begin_chunk(E);
#pragma unroll
		for (int j = 0; j < 2; ++j) {
			const int i = tid + kThreads * j;
			const int m = i & (kRows - 1), kg = i >> 7;
			store_digits8<FMT, SLICED>(xb, P.part_bytes, m, 8 * kg, xv[j], colF[m], S);
		}
		if (c + 1 < KL) lift_load<D, NV, KF>(xv, c + 1, nnf, xfr, g, e0, rows, KFR);   // in flight during the issue
		eng_end_chunk<FMT, SLICED>(E, c * nparts, c == 0, S, Al.N_pad, idesc);
	}
	eng_drain(E);

	// epilogue: TMEM -> shared staging -> coalesced pass over the block's contiguous [element][variable][node] range
	double* R = (double*)E.dig;
	const int ld_r = Al.N_pad + 1;
	{
		const int m = 32 * (warp & 3) + lane;
		const uint32_t trow = E.tmem + ((uint32_t)(32 * (warp & 3)) << 16);
		for (int c8 = warp >> 2; c8 < Al.N_pad / 8; c8 += 2) {
			double v8[8];
			combine8<SLICED>(trow, Al.N_pad, 8 * c8, nacc, v8);
#pragma unroll
			for (int j = 0; j < 8; ++j) {
				const int row = 8 * c8 + j;
				if (row >= n_s) continue;
				double y = v8[j];
				if constexpr (SLICED) y = scale_out(y, Al.row_exp[row], colF[m]);
				R[m * ld_r + row] = y;
			}
		}
	}
	tc::fence_before_sync();
	__syncthreads();
	const double dt = (stage >= 0 ? *dt_ptr : 0.0);
	double lmax = 0.0;
	const size_t base = (size_t)e0 * NV * n_s;
	for (int i = tid; i < rows * n_s; i += kThreads) {
		const int m = i / n_s, row = i - m * n_s;
		const double r = R[m * ld_r + row] * g.jinv[e0 + m / NV];
		lmax = fmax(lmax, fabs(r));
		if (isnan(r)) lmax = r;
		const size_t gi = base + i;
		if (write_rhs) rhs[gi] = r;
		if (stage >= 0) {
			const double u0 = sol[gi];
			if (stage == 0) { solp[gi] = u0; sol[gi] = u0 + dt * r; }
			else if (stage == 1) sol[gi] = (1.0 / 4.0) * (3.0 * solp[gi] + u0 + dt * r);
			else sol[gi] = (1.0 / 3.0) * (solp[gi] + 2.0 * u0 + 2.0 * dt * r);
		}
	}
	for (int off = 16; off > 0; off >>= 1) {
		const double other = __shfl_xor_sync(0xffffffffu, lmax, off);
		lmax = (isnan(other) || other > lmax) ? other : lmax;
	}
	if (lane == 0) atomicMax(max_slot, (unsigned long long)__double_as_longlong(fabs(lmax)));
	eng_finish(E);
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

// Slice an operator [N_op x K_real] (row-major, K column k placed at kmap[k] of the padded K) into device tiles of
// N_pad (a multiple of 16) rows x 32 K, [chunk][slice].
static int build_split_op(SplitOp& op, const std::vector<double>& Aop, int N_op, int K_real, const std::vector<int>& kmap,
                          int K_pad, int mode, int S, int es)
{
	op.N_op = N_op;
	op.N_pad = (N_op + 15) / 16 * 16;
	if (op.N_pad > 256) return DPG_ERR_UNSUPPORTED;
	op.K_pad = K_pad;
	op.n_chunks = K_pad / 32;
	op.S = (mode == DPG_PREC_BF16_SLICED ? S : 2);
	op.es = es;
	op.tile_bytes = (size_t)op.N_pad * 32 * es;
	std::vector<uint8_t> tiles(op.tile_bytes * op.S * op.n_chunks, 0);
	std::vector<int> rexp(op.N_pad, 0);
	for (int i = 0; i < N_op; ++i) {
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
	if (cudaMalloc(&op.row_exp, sizeof(int) * op.N_pad) != cudaSuccess) return DPG_ERR_CUDA;
	if (cudaMemcpy(op.row_exp, rexp.data(), sizeof(int) * op.N_pad, cudaMemcpyHostToDevice) != cudaSuccess)
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
	if (st->xfr) cudaFree(st->xfr);
	if (st->colE) cudaFree(st->colE);
	if (st->face_exp) cudaFree(st->face_exp);
	if (st->err) cudaFree(st->err);
	delete st;
	c->split = nullptr;
}

static SplitArgs args_of(const SplitOp& op) { return SplitArgs{op.tiles, op.row_exp, op.N_pad, (int)op.tile_bytes}; }

struct Kernels { void* interp; void* lift; };

template <int D, int NV, int KS, int KF, int FMT, bool SL>
static Kernels kernels_of() { return Kernels{(void*)ks_interp<D, NV, KS, FMT, SL>, (void*)ks_lift<D, NV, KF, FMT, SL>}; }

// The (d, NV, solution K chunks, face K chunks) combinations instantiated: Euler/advection on QUAD p1..4 and
// HEX p1..3.
#define DPG_SPLIT_CASES(X)  \
	X(3, 5, 2, 3)  /* HEX p3 Euler  */ \
	X(3, 5, 1, 2)  /* HEX p2 Euler  */ \
	X(3, 5, 1, 1)  /* HEX p1 Euler  */ \
	X(2, 4, 1, 1)  /* QUAD p1..4 Euler */ \
	X(2, 1, 1, 1)  /* QUAD advection */ \
	X(3, 1, 2, 3)  /* HEX p3 advection */ \
	X(3, 1, 1, 2)  /* HEX p2 advection */ \
	X(3, 1, 1, 1)  /* HEX p1 advection */

template <int FMT, bool SL>
static Kernels pick(int d, int nv, int ks, int kf)
{
#define DPG_PICK(D_, NV_, KS_, KF_) if (d == D_ && nv == NV_ && ks == KS_ && kf == KF_) return kernels_of<D_, NV_, KS_, KF_, FMT, SL>();
	DPG_SPLIT_CASES(DPG_PICK)
#undef DPG_PICK
	return Kernels{nullptr, nullptr};
}

static Kernels pick_all(int mode, int d, int nv, int ks, int kf)
{
	if (mode == DPG_PREC_BF16_SLICED) return pick<1, true>(d, nv, ks, kf);
	if (mode == DPG_PREC_BF16X3) return pick<1, false>(d, nv, ks, kf);
	return pick<2, false>(d, nv, ks, kf);
}

// Shared-memory plan: [ring | digit region | FP64 staging | column scales | barriers | TMEM slot].  The ring takes
// as many stages (2..kRingMax) as fit.
static int make_plan(Plan& P, int stage_bytes, int nparts, int es, int n_dig_chunks, int dig_min_bytes, int st_doubles)
{
	P.stage_bytes = (stage_bytes + 127) / 128 * 128;
	P.part_bytes = kRows * 32 * es;
	P.chunk_bytes = nparts * P.part_bytes;
	const int dig = std::max(n_dig_chunks * P.chunk_bytes, (dig_min_bytes + 127) / 128 * 128);
	auto total = [&](int nst) {
		return nst * P.stage_bytes + dig + 8 * st_doubles + 4 * kRows + 8 * (2 * nst + 6) + 16;
	};
	int nst = kRingMax;
	while (nst > 2 && total(nst) > kSmemMax) --nst;
	if (total(nst) > kSmemMax) return DPG_ERR_UNSUPPORTED;
	P.nst = nst;
	P.off_dig = nst * P.stage_bytes;
	P.off_st = P.off_dig + dig;
	P.off_colF = P.off_st + 8 * st_doubles;
	P.off_bars = P.off_colF + 4 * kRows;
	P.smem_bytes = std::max(total(nst), kSmemOneBlock);
	return DPG_OK;
}

int split_prepare(dpg_gpu_ctx* c)
{
	split_free(c);
	const GroupDev& g = c->g;
	if (!g.affine) return DPG_ERR_UNSUPPORTED;  // per-element m_inv on the split path: not provided
	if (c->fc.n_fc > 32) return DPG_ERR_UNSUPPORTED;
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
	const int KF = st->nf_pad / 32;
	const int KL = KF + d * st->n_c_pad / 32;
	Kernels kp = pick_all(st->mode, d, NV, KS, KF);
	if (!kp.interp) { split_free(c); return DPG_ERR_UNSUPPORTED; }

	// host copies of the FP64 operators (as uploaded for the FP64 form)
	std::vector<double> Cv((size_t)n_c * n_s), Cf((size_t)n_fl * n_fc * n_s), Lm((size_t)n_s * g.K);
	if (cudaMemcpy(Cv.data(), g.Cv, sizeof(double) * Cv.size(), cudaMemcpyDeviceToHost) ||
	    cudaMemcpy(Cf.data(), g.Cf, sizeof(double) * Cf.size(), cudaMemcpyDeviceToHost) ||
	    cudaMemcpy(Lm.data(), g.L, sizeof(double) * Lm.size(), cudaMemcpyDeviceToHost)) { split_free(c); return DPG_ERR_CUDA; }
	// K of the lift: the face part first, then the reference fluxes r-major with n_c_pad nodes each (the layout of
	// the global lift operand written by ks_interp)
	std::vector<int> kmap_s(n_s), kmap_l(g.K);
	for (int k = 0; k < n_s; ++k) kmap_s[k] = k;
	for (int r = 0; r < d; ++r)
		for (int cc = 0; cc < n_c; ++cc) kmap_l[r * n_c + cc] = st->nf_pad + r * st->n_c_pad + cc;
	for (int fq = 0; fq < n_fl * n_fc; ++fq) kmap_l[d * n_c + fq] = fq;
	int rc;
	if ((rc = build_split_op(st->cv, Cv, n_c, n_s, kmap_s, st->n_s_pad, st->mode, st->S, st->es))) { split_free(c); return rc; }
	if ((rc = build_split_op(st->cf, Cf, n_fl * n_fc, n_s, kmap_s, st->n_s_pad, st->mode, st->S, st->es))) { split_free(c); return rc; }
	if ((rc = build_split_op(st->lift, Lm, n_s, g.K, kmap_l, 32 * KL, st->mode, st->S, st->es))) { split_free(c); return rc; }
	const int nacc = (st->mode == DPG_PREC_BF16_SLICED ? std::min(st->S, kAccSliced) : 1);
	if (nacc * std::max(st->cv.N_pad, st->cf.N_pad) > 512 || nacc * st->lift.N_pad > 512) { split_free(c); return DPG_ERR_UNSUPPORTED; }

	// blocks: EB elements (EB * NV <= 128 data rows), as few whole waves of the SMs as possible, spread evenly
	int n_sm = 0;
	if (cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, c->dev) != cudaSuccess || n_sm < 1) n_sm = 1;
	const int eb_max = kRows / NV;
	const int waves = std::max(1, ((g.n_vol + eb_max - 1) / eb_max + n_sm - 1) / n_sm);
	st->EB = std::min(eb_max, (g.n_vol + waves * n_sm - 1) / (waves * n_sm));
	st->n_blocks = (g.n_vol + st->EB - 1) / st->EB;
	const int fpw = 32 / n_fc;
	st->n_face_warps = (c->fc.n_face + fpw - 1) / fpw;

	if (cudaMalloc(&st->err, sizeof(int)) != cudaSuccess || cudaMemset(st->err, 0, sizeof(int)) != cudaSuccess ||
	    cudaMalloc(&st->xfr, sizeof(double) * (size_t)g.n_vol * NV * d * st->n_c_pad) != cudaSuccess ||
	    cudaMalloc(&st->colE, sizeof(int) * (size_t)g.n_vol * NV) != cudaSuccess ||
	    cudaMalloc(&st->face_exp, sizeof(int) * (size_t)c->fc.n_face * NV) != cudaSuccess) {
		split_free(c);
		return DPG_ERR_CUDA;
	}
	const int nparts = st->S;
	const int ld_u = st->n_s_pad + 2, ld_v = st->n_c_pad + 1;
	if ((rc = make_plan(st->pi, (int)std::max(st->cv.tile_bytes, st->cf.tile_bytes), nparts, st->es, KS,
	                    8 * kRows * (st->cf.N_pad + 1), kRows * std::max(ld_u, ld_v)))) { split_free(c); return rc; }
	if ((rc = make_plan(st->pl, (int)st->lift.tile_bytes, nparts, st->es, 2, 8 * kRows * (st->lift.N_pad + 1), 0))) {
		split_free(c);
		return rc;
	}
	if (cudaFuncSetAttribute(kp.interp, cudaFuncAttributeMaxDynamicSharedMemorySize, st->pi.smem_bytes) ||
	    cudaFuncSetAttribute(kp.lift, cudaFuncAttributeMaxDynamicSharedMemorySize, st->pl.smem_bytes)) {
		split_free(c);
		return DPG_ERR_CUDA;
	}
	return DPG_OK;
}

template <int D, int NV, int KS, int KF, int FMT, bool SL>
static void launch_k(dpg_gpu_ctx* c, SplitState* st, int which, int stage, bool write_rhs, unsigned long long* max_slot)
{
	const GroupDev& g = c->g;
	if (which == 0) {
		ks_interp<D, NV, KS, FMT, SL><<<st->n_blocks, kThreads, st->pi.smem_bytes, c->stream>>>(
		    c->sol, g, c->trace, st->xfr, st->colE, args_of(st->cv), args_of(st->cf), st->pi, st->S, st->EB,
		    st->n_c_pad, c->b_adv[0], c->b_adv[1], c->b_adv[2], st->err);
	} else if (which == 1) {
		const int threads = 256, warps_per_block = threads / 32;
		ks_face<D, NV><<<(st->n_face_warps + warps_per_block - 1) / warps_per_block, threads, 0, c->stream>>>(
		    c->trace, c->fc, c->nnf, st->face_exp, c->num_flux, c->b_adv[0], c->b_adv[1], c->b_adv[2]);
	} else {
		ks_lift<D, NV, KF, FMT, SL><<<st->n_blocks, kThreads, st->pl.smem_bytes, c->stream>>>(
		    c->sol, c->solp, c->rhs, c->nnf, st->face_exp, st->xfr, st->colE, g, args_of(st->lift), st->pl, st->S,
		    st->EB, st->n_c_pad, c->ddt, max_slot, stage, write_rhs ? 1 : 0, st->err);
	}
}

template <int FMT, bool SL>
static int launch_sel(dpg_gpu_ctx* c, SplitState* st, int which, int stage, bool write_rhs, unsigned long long* max_slot)
{
	const int d = c->d, nv = c->n_var, ks = st->n_s_pad / 32, kf = st->nf_pad / 32;
#define DPG_LAUNCH(D_, NV_, KS_, KF_) \
	if (d == D_ && nv == NV_ && ks == KS_ && kf == KF_) { launch_k<D_, NV_, KS_, KF_, FMT, SL>(c, st, which, stage, write_rhs, max_slot); return DPG_OK; }
	DPG_SPLIT_CASES(DPG_LAUNCH)
#undef DPG_LAUNCH
	return DPG_ERR_UNSUPPORTED;
}

static int launch_any(dpg_gpu_ctx* c, int which, int stage, bool write_rhs, unsigned long long* max_slot)
{
	SplitState* st = (SplitState*)c->split;
	if (!st) return DPG_ERR_INVALID;
	int rc;
	if (st->mode == DPG_PREC_BF16_SLICED) rc = launch_sel<1, true>(c, st, which, stage, write_rhs, max_slot);
	else if (st->mode == DPG_PREC_BF16X3) rc = launch_sel<1, false>(c, st, which, stage, write_rhs, max_slot);
	else rc = launch_sel<2, false>(c, st, which, stage, write_rhs, max_slot);
	if (rc) return rc;
	return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

int split_launch_trace(dpg_gpu_ctx* c) { return launch_any(c, 0, -1, false, nullptr); }
int split_launch_face(dpg_gpu_ctx* c) { return launch_any(c, 1, -1, false, nullptr); }
int split_launch_volume(dpg_gpu_ctx* c, int stage, bool write_rhs, unsigned long long* max_slot)
{
	return launch_any(c, 2, stage, write_rhs, max_slot);
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
