// Split-precision residual kernels: the DG operator contractions on the tcgen05 tensor cores.
//
// Three precision modes share one kernel structure (DPG_PREC_*):
//   BF16_SLICED : every operand is scaled by a power of two per operator row / per data column (|value| 2^-E < 1/2)
//                 and cut into S signed 8-bit digits (the leading one in [-128, 128]); digit s is stored as the
//                 BF16 value d * 2^(-8s) (exact).  The digit products with level a+b < S are accumulated in FP32 in
//                 TMEM: one accumulator for each of the levels 0..3 and one for the levels >= 4.  Level sums are
//                 integers times 2^(-8L) below 2^24 in those units (exact) except in a contrived worst case of level
//                 3 at K = 288, where the FP32 rounding is 2^-48 of the leading level, like the tail accumulator's.
//                 The accumulators are combined in 64-bit integers and converted to FP64 once.  The error is
//                 ~ 2^(-8S) * K * max|row| * max|column|, i.e. FP64-like for S = 6..7.
//   BF16X3      : x = hi + lo in BF16, hi*hi + hi*lo + lo*hi in one FP32 accumulator (~1e-5 relative).
//   TF32X3      : the same with TF32 operands (kind::tf32, ~1e-7 relative).
// The pointwise physics (the reference volume flux and the numerical flux at the faces), which would be FP64-bound on
// this GPU (~2.6 FP64 lanes per clock per SM), runs in double-float arithmetic on the FP32 pipe (~2^-47 relative per
// operation); the lift operand, RK stages and norms stay in FP64.
//
// Shapes.  One tcgen05.mma (K = 16) occupies the tensor pipe for ~48-64 cycles whatever M <= 128 and N <= 128 are,
// so every contraction is laid out for M = 128: the data operand (A) has one row per (element, variable) of a
// block of EB elements (EB * NV <= 128), the operator slice (B) one row per operator row (N = 64 for the volume
// interpolation and the lift of HEX p=3, 96 for its face interpolation).  TMEM holds the accumulators
// [128 lanes = data rows][N columns] x 5 levels; one block per SM owns all 512 columns.  The issuing warp runs a
// fully unrolled stream of MMAs (the number of parts is a template parameter) whose descriptors differ by
// compile-time offsets: any scalar work between MMAs would leave the tensor pipe idle.
//
// Kernels of one residual (split path):
//   ks_interp : sol_coef -> digits (kept for both contractions) -> s_vc = Cv * U (TMEM) -> reference volume fluxes
//               (double-float, written as FP64) to global memory with a per-column exponent bound, while the tensor pipe runs
//               U_fc = Cf * U -> face traces in element order (FP32 pairs, straight from registers)
//   ks_face   : numerical flux per face node in double-float arithmetic (FP32 pairs, df64.cuh / flux_df.cuh) on the
//               traces, which ks_interp writes as FP32 pairs; the flux goes back to FP64, with a per-(face,
//               variable) exponent bound (split_ops.cu)
//   ks_lift   : digits of [face fluxes | reference volume fluxes] streamed chunk by chunk from global memory
//               (column scales known from the two exponent bounds), rhs = L' * X (TMEM), 1/detJ, ||rhs||_inf and
//               the SSP-RK3 stage update through a coalesced epilogue.
// Operator tiles [chunk][slice] are pre-sliced on the host in the shared-memory layout and streamed with
// cp.async.bulk (interpolation: a ring of slice tiles; lift: whole-chunk slots), completion is signalled by
// tcgen05.commit on mbarriers and every wait is bounded (a timeout sets an error flag read by the host).
#pragma once

#include <cstdint>

#include <cuda_bf16.h>

#include "dpg_gpu_internal.cuh"
#include "flux.cuh"
#include "flux_df.cuh"
#include "tc_sm100.cuh"

namespace dpg {
namespace split {

// 16 compute warps: every compute phase (digits, epilogues, pointwise fluxes) is latency-bound with one block per SM
// (the block owns all TMEM columns), so the warps per scheduler set its speed.  With the MMA-issuing warp and the
// operator-loading warp the block has 576 threads, 96 registers each.
constexpr int kCompute = 512;               // threads writing digits and running the epilogues (warps 0..15)
constexpr int kComputeWarps = kCompute / 32;
constexpr int kIssueWarp = kComputeWarps;       // warp 16 issues the MMAs
constexpr int kLoadWarp = kComputeWarps + 1;    // warp 17 streams the operator tiles into shared memory
constexpr int kBlockThreads = kCompute + 64;
constexpr int kRows = 128;      // data rows (element, variable) of one block: the MMA M
constexpr int kGroups = kCompute / kRows;   // K groups of 8 handled side by side per data row (thread = row, group)
constexpr int kItemsPerChunk = 4 / kGroups; // a 32-wide K chunk holds 4 groups of 8
constexpr int kColStride = kComputeWarps / 4;   // epilogues: warp w reads TMEM lanes 32 (w % 4).., columns 8 (w / 4) + 8 kColStride j
// share of the interpolation kernel's volume-flux items evaluated in FP64, in eighths (the rest in double-float
// arithmetic): the default of the block configuration, which the tile autotuner may change
constexpr int kFp64Eighths = 2;
static_assert(kCompute % kRows == 0 && 4 % kGroups == 0, "compute threads: a multiple of 128 dividing 512");
constexpr int kMaxS = 7;
constexpr int kColSlots = 8;    // exponent-bound slots per lift row: up to 6 local faces + the volume part, padded
constexpr int kAccSliced = 5;   // accumulators: levels 0, 1, 2, 3 and >= 4
// interpolation kernel: operator slice stages (a TF32 slice tile is twice as large)
__host__ __device__ constexpr int ring_stages(int fmt) { return fmt == 1 ? 7 : 3; }
constexpr int kSlotsL = 3;      // lift kernel: whole-chunk operator slots

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
	int stage_bytes;             // one operator stage (interpolation: one slice tile; lift: one chunk of slices)
	int off_dig, off_st, off_tab, off_colF, off_bars;
	int smem_bytes;
};

struct SplitState;

// Launchers of one (d, NV, chunk counts, mode) instantiation.
struct KernelTable {
	void (*interp)(dpg_gpu_ctx* c, const SplitState* st);
	void (*lift)(dpg_gpu_ctx* c, const SplitState* st, int stage, int write_rhs, unsigned long long* max_slot);
	const void* interp_fn;
	const void* lift_fn;
};

struct SplitState {
	int mode = 0, S = 0, fmt = 1, es = 2, nparts = 2;
	int n_s_pad = 0, n_c_pad = 0, nf_pad = 0;
	int EB = 0, n_blocks = 0, n_face_warps = 0;
	int fp64_eighths = kFp64Eighths;   // FP64 share of the volume-flux items
	int face_block_warps = 8;          // warps per block of the face kernel
	int eb_default = 0;                // elements per block chosen by the wave rule
	int KL = 0;                  // lift K chunks: KF face chunks, then d * KC volume chunks
	SplitOp cv, cf, lift;
	Plan pi{}, pl{};
	KernelTable kt{};
	double* xl = nullptr;        // [n_vol][NV][32 * KL] lift operand: scaled numerical fluxes of the element's face
	                             // nodes (K = local face * n_fc + node; right sides negated, in their own node order),
	                             // then the reference volume fluxes (K = 32 KF + r * n_c_pad + node); padding zero
	int* colE = nullptr;         // [n_vol][NV][kColSlots] exponent bounds of the parts of the element's row of xl:
	                             // slot lf per local face (written by the face kernel), slot n_fl for the reference
	                             // volume fluxes (the interpolation kernel); each slot has one writer, unused slots
	                             // stay at a very negative value
	int* fel = nullptr;          // [n_face][2] element * n_fl + local face of the face's two sides
	float2* nrm2 = nullptr;      // [n_face][n_fc][d] unit normals as double-floats
	float2* jf2 = nullptr;       // [n_face][n_fc] face Jacobians as double-floats
	float2 b2[3] = {};           // advection velocity as double-floats
	float2* met2 = nullptr;      // [n_vol][d*d] cofactor metrics as double-floats (m_ij at i + d*j)
	int* err = nullptr;
};

// Lookup of the instantiated kernels of a mode (split_inst_*.cu) by (d, NV, solution / face / volume-node K
// chunks); a null table when the combination is not instantiated.
KernelTable kernels_sliced4(int d, int nv, int ks, int kf, int kc);
KernelTable kernels_sliced5(int d, int nv, int ks, int kf, int kc);
KernelTable kernels_sliced6(int d, int nv, int ks, int kf, int kc);
KernelTable kernels_sliced7(int d, int nv, int ks, int kf, int kc);
KernelTable kernels_bf16x3(int d, int nv, int ks, int kf, int kc);
KernelTable kernels_tf32x3(int d, int nv, int ks, int kf, int kc);

// ------------------------------------------------------------------------------------------------------------
// digit / split helpers
// ------------------------------------------------------------------------------------------------------------
__device__ __forceinline__ int exp_bound(double x)
{
	const long long b = __double_as_longlong(x);
	const int be = (int)((b >> 52) & 0x7FF);
	return be == 0 ? -4000 : be - 1022;  // |x| < 2^e
}

// Column scale F (|x| 2^-F < 1/2) from the largest exponent bound of the column, clamped so that the digit shifts
// stay in range for tiny or huge columns.
__device__ __forceinline__ int col_exp_of(int emax, int S)
{
	const int F = emax < -3000 ? 0 : emax + 1;
	const int lo = 8 * S - 1000, hi = 8 * S + 1000;
	return F < lo ? lo : (F > hi ? hi : F);
}

// round(x * 2^sc) from the bits of x with integer operations only (the FP64 pipe is kept for the fluxes):
// x = +-mant * 2^(be - 1075), so the result is +-mant * 2^(be - 1075 + sc) (|result| < 2^(8S-1) by the choice of sc).
// Branch-free: a left shift by max(sh, 0) and a rounding right shift by min(max(-sh, 0), 63).
__device__ __forceinline__ long long scaled_mantissa(double x, int sc)
{
	const long long bits = __double_as_longlong(x);
	const int be = (int)((bits >> 52) & 0x7FF);
	const long long mant = (bits & 0xFFFFFFFFFFFFFll) | (1ll << 52);
	const int sh = be - 1075 + sc;
	const int rs = min(max(-sh, 0), 63);
	const long long half = rs > 0 ? (1ll << (rs - 1)) : 0ll;
	long long m = ((mant << max(sh, 0)) + half) >> rs;
	m = be == 0 ? 0ll : m;
	return bits < 0 ? -m : m;
}

// 128 in each of the S-1 low digit bytes: m + bias has the biased digits d_s + 128 in [0, 255] as its low bytes and
// the leading digit d_0 in [-128, 128] above them.
template <int S>
__host__ __device__ constexpr long long digit_bias()
{
	long long C = 0;
	for (int s = 0; s < S - 1; ++s) C |= 128ll << (8 * s);
	return C;
}

__host__ __device__ constexpr float pow2f(int e) { return e >= 0 ? (e == 0 ? 1.0f : 2.0f * pow2f(e - 1)) : 0.5f * pow2f(e + 1); }

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

// Digit s >= 1 (byte S-1-s of the biased integer) of 8 values as floats d * 2^(-8s), exactly: one byte permute
// places the byte u in the low mantissa bits under the exponent field 150 - 8s, i.e. the float
// 2^(23-8s) + u 2^(-8s), and one add removes 2^(23-8s) + 128 * 2^(-8s).  The leading digit (s = 0, 9 bits with
// its bias) is placed by an OR into the mantissa of 2^23.
template <int S, int s>
__device__ __forceinline__ uint4 digit_row(const uint32_t (&lo)[8], const uint32_t (&hi)[8], const uint32_t (&lead)[8])
{
	float f[8];
	if constexpr (s == 0) {
#pragma unroll
		for (int j = 0; j < 8; ++j) f[j] = __uint_as_float(0x4B000000u | lead[j]) - 8388736.0f;
	} else {
		constexpr int k = S - 1 - s;
		constexpr uint32_t K = (uint32_t)(150 - 8 * s) << 23;
		constexpr uint32_t sel = 0x7650u | (uint32_t)(k & 3);
		constexpr float sub = -8388736.0f * pow2f(-8 * s);
#pragma unroll
		for (int j = 0; j < 8; ++j) f[j] = __uint_as_float(__byte_perm(k < 4 ? lo[j] : hi[j], K, sel)) + sub;
	}
	return make_uint4(pack_bf16x2(f[0], f[1]), pack_bf16x2(f[2], f[3]), pack_bf16x2(f[4], f[5]), pack_bf16x2(f[6], f[7]));
}

template <int S, int s>
__device__ __forceinline__ void store_slices(uint8_t* dst, int part_bytes, const uint32_t (&lo)[8], const uint32_t (&hi)[8],
                                             const uint32_t (&lead)[8])
{
	if constexpr (s < S) {
		*(uint4*)(dst + s * part_bytes) = digit_row<S, s>(lo, hi, lead);
		store_slices<S, s + 1>(dst, part_bytes, lo, hi, lead);
	}
}

// Digits / split parts of 8 consecutive K values (kk0 .. kk0+7 of a 32-K chunk) of data row m, written as one
// 16-byte core-matrix row per part (two for TF32).  Eight consecutive threads taking eight consecutive rows of one
// K group fill one whole 128-byte core matrix (conflict-free).  F = column scale (sliced mode).
// Value access for the digit writers: FP64 values (the solution coefficients) or double-floats (the streamed lift
// operand, which the producing kernels keep as FP32 pairs).
__device__ __forceinline__ long long mantissa_of(double x, int sc) { return scaled_mantissa(x, sc); }
__device__ __forceinline__ long long mantissa_of(df::df64 x, int sc) { return df::scaled_mantissa(x, sc); }
__device__ __forceinline__ float float_of(double x) { return (float)x; }
__device__ __forceinline__ float float_of(df::df64 x) { return x.hi + x.lo; }

template <int FMT, int NP, bool SLICED, class T>
__device__ __forceinline__ void store_digits8(uint8_t* chunk, int m, int kk0, const T (&x)[8], int F)
{
	constexpr int es = (FMT == 1 ? 2 : 4);
	constexpr int part_bytes = kRows * 32 * es;
	if constexpr (SLICED) {
		const int sc = 8 * NP - F;
		uint32_t lo[8], hi[8], lead[8];
#pragma unroll
		for (int j = 0; j < 8; ++j) {
			const long long mm = mantissa_of(x[j], sc) + digit_bias<NP>();
			lo[j] = (uint32_t)mm;
			hi[j] = (uint32_t)((unsigned long long)mm >> 32);
			lead[j] = (uint32_t)((int)(mm >> (8 * (NP - 1))) + 128);
		}
		store_slices<NP, 0>(chunk + tc::kmajor_offset(m, kk0, 32, 2), part_bytes, lo, hi, lead);
	} else if constexpr (FMT == 1) {
		float hi[8], lo[8];
#pragma unroll
		for (int j = 0; j < 8; ++j) {
			const float xf = float_of(x[j]);
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
			const float xf = float_of(x[j]);
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
// MMA stream of one operator slice a against the data parts of one chunk: part b into accumulator min(a+b, 4)
// (sliced) or the three products hi*hi, hi*lo, lo*hi into one accumulator.  Issuing warp, all lanes.
// ------------------------------------------------------------------------------------------------------------
template <int FMT, int NP, bool SLICED, int a>
__device__ __forceinline__ void mma_slice(uint64_t xd0, uint64_t od, const uint32_t (&tacc)[kAccSliced], uint32_t idesc,
                                          bool first)
{
	constexpr int es = (FMT == 1 ? 2 : 4);
	constexpr uint32_t pstep = (uint32_t)(kRows * 32 * es) >> 4;
	constexpr int nb = SLICED ? NP - a : (a == 0 ? 2 : 1);
#pragma unroll
	for (int ks = 0; ks < es; ++ks) {
#pragma unroll
		for (int b = 0; b < nb; ++b) {
			const int L = SLICED ? (a + b < kAccSliced - 1 ? a + b : kAccSliced - 1) : 0;
			// the first product into accumulator L is (a = 0, b = L) (for the tail: (0, 4)); unsliced: (0, 0)
			const bool init_slot = ks == 0 && a == 0 && (SLICED ? b <= kAccSliced - 1 : b == 0);
			const uint32_t acc = (first && init_slot) ? 0u : 1u;
			const uint64_t dd = xd0 + (uint64_t)(b * pstep + 16 * ks);
			if constexpr (FMT == 1) tc::mma_bf16_elect(tacc[L], dd, od + 16 * ks, idesc, acc);
			else tc::mma_tf32_elect(tacc[L], dd, od + 16 * ks, idesc, acc);
		}
	}
}

template <int FMT, int NP, bool SLICED, int a>
struct SliceLoop {
	template <class PerSlice>
	__device__ __forceinline__ static void run(PerSlice& f)
	{
		if constexpr (a < NP) {
			f.template slice<a>();
			SliceLoop<FMT, NP, SLICED, a + 1>::run(f);
		}
	}
};

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
	asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void fail(int* err, int code) { atomicExch(err, code); }

// Barrier of the compute warps only (the issuing warp runs its own loop meanwhile).
__device__ __forceinline__ void compute_sync() { asm volatile("bar.sync 1, %0;" ::"n"(kCompute) : "memory"); }

// Issuing warp: bulk copy of `bytes` into shared memory completing on `bar` (one elected lane).
__device__ __forceinline__ void load_stage(uint8_t* dst, const uint8_t* src, uint32_t bytes, uint64_t* bar)
{
	if (tc::elect_one()) {
		tc::mbar_expect_tx(bar, bytes);
		tc::bulk_g2s(dst, src, bytes, bar);
	}
	__syncwarp();
}

// TMEM column addresses of the accumulators for a contraction with N_pad columns.
__device__ __forceinline__ void acc_addrs(uint32_t tmem, int N_pad, uint32_t (&tacc)[kAccSliced])
{
#pragma unroll
	for (int L = 0; L < kAccSliced; ++L) tacc[L] = tmem + (uint32_t)(L * N_pad);
}

// Eight accumulator columns c0..c0+7 of this thread's TMEM lane as double-floats, scaled by
// 2^(row_exp[c0 + j] + F - 16) in sliced mode (the operator row scale, the data column scale and 2^-16 of the two
// digit scalings).  Each level accumulator is an exact FP32 value (an integer times its 2^-8L), so the levels are
// summed with error-free FP32 additions (TwoSum): no conversion instruction, no FP64.  All lanes call (tcgen05.ld is
// warp-wide); `live` = a real data row.
template <bool SLICED, int NACC>
__device__ __forceinline__ void combine8_df(uint32_t trow, int N_pad, int c0, const int* __restrict__ row_exp, int F,
                                            bool live, df::df64 (&out)[8])
{
	if constexpr (SLICED) {
		float a[NACC][8];
#pragma unroll
		for (int L = 0; L < NACC; ++L) tc::tmem_ld8(trow + (uint32_t)(L * N_pad + c0), a[L]);
		tc::tmem_ld_wait();
		if (!live) return;
#pragma unroll
		for (int j = 0; j < 8; ++j) {
			df::df64 sj = df::mk(a[0][j]);
#pragma unroll
			for (int L = 1; L < NACC; ++L) sj = df::add_f(sj, a[L][j]);
			out[j] = df::scale_pow2(sj, row_exp[c0 + j] + F - 16);
		}
	} else {
		float a[8];
		tc::tmem_ld8(trow + (uint32_t)c0, a);
		tc::tmem_ld_wait();
		if (!live) return;
#pragma unroll
		for (int j = 0; j < 8; ++j) out[j] = df::mk(a[j]);
	}
}

// Eight accumulator columns combined exactly (the 64-bit level sum V in units of 2^-32: each level accumulator is an
// integer times 2^-8L below 2^25 in those units, converted by a 32-bit conversion) and returned as
// double-floats of V itself: V = V2 2^48 + V1 2^24 + V0 with three exactly convertible pieces, joined by TwoSum, so
// the error is ~2^-48 of V (an exact cancellation stays exact) and no FP64 instruction is used.  Not sliced: the
// single FP32 accumulator.  All lanes call (tcgen05.ld is warp-wide).
template <bool SLICED, int NACC>
__device__ __forceinline__ void combine8_exact_df(uint32_t trow, int N_pad, int c0, df::df64 (&out)[8])
{
	if constexpr (SLICED) {
		float a[NACC][8];
#pragma unroll
		for (int L = 0; L < NACC; ++L) tc::tmem_ld8(trow + (uint32_t)(L * N_pad + c0), a[L]);
		tc::tmem_ld_wait();
#pragma unroll
		for (int j = 0; j < 8; ++j) {
			long long V = 0;
#pragma unroll
			for (int L = 0; L < NACC; ++L)
				V += (long long)__float2int_rn(a[L][j] * __int_as_float((127 + 8 * L) << 23)) << (32 - 8 * L);
			const float f2 = (float)(int)(V >> 48) * 281474976710656.0f;            // 2^48
			const float f1 = (float)(int)((V >> 24) & 0xFFFFFF) * 16777216.0f;     // 2^24
			const float f0 = (float)(int)(V & 0xFFFFFF);
			out[j] = df::add_f(df::two_sum(f2, f1), f0);
		}
	} else {
		float a[8];
		tc::tmem_ld8(trow + (uint32_t)c0, a);
		tc::tmem_ld_wait();
#pragma unroll
		for (int j = 0; j < 8; ++j) out[j] = df::mk(a[j]);
	}
}


// Reference-space volume flux of one node in FP64, handed to emit(r, fr_r) one reference direction at a time (the
// formulas of the double-float version, flux_df.cuh ref_flux_rows; the direction loop stays rolled).
template <int D, int NV, class MCol, class Emit>
__device__ __forceinline__ void ref_flux_rows(const double* s, const MCol& mcol, const double* b, Emit&& emit)
{
	if constexpr (NV == D + 2) {
		const double rho_inv = 1.0 / s[0], E = s[D + 1];
		double u[D], V2 = 0.0;
#pragma unroll
		for (int a = 0; a < D; ++a) { u[a] = s[1 + a] * rho_inv; V2 += u[a] * u[a]; }
		const double p = DPG_GM1_D * (E - 0.5 * s[0] * V2), Ep = E + p;
#pragma unroll 1
		for (int r = 0; r < D; ++r) {
			double m[D];
#pragma unroll
			for (int x = 0; x < D; ++x) m[x] = mcol(x, r);
			double W = 0.0, f0 = 0.0;
#pragma unroll
			for (int x = 0; x < D; ++x) { W += m[x] * u[x]; f0 += m[x] * s[1 + x]; }
			double fr[NV];
			fr[0] = f0;
#pragma unroll
			for (int a = 0; a < D; ++a) fr[1 + a] = s[1 + a] * W + m[a] * p;
			fr[D + 1] = Ep * W;
			emit(r, fr);
		}
	} else {
#pragma unroll 1
		for (int r = 0; r < D; ++r) {
			double fr[NV];
			fr[0] = 0.0;
#pragma unroll
			for (int x = 0; x < D; ++x) fr[0] += mcol(x, r) * (b[x] * s[0]);
			emit(r, fr);
		}
	}
}

// ------------------------------------------------------------------------------------------------------------
// ks_interp: traces and reference volume fluxes of a block of EB elements.
// Operator tiles: Cv chunks 0..KS-1 then Cf chunks 0..KS-1, NP slice tiles each, through a ring of NST stages
// (tile t in stage t % NST).  The loading warp refills a stage as soon as the MMAs of its previous tile are done (one
// commit per tile on empty[stage]); the issuing warp waits for each tile on full[stage].  (Refills by the issuing
// warp itself come late: it runs ahead of the tensor pipe, so a stage is rarely free when it looks.)
// ------------------------------------------------------------------------------------------------------------
template <int NST>
struct InterpRing {
	uint8_t* ring;
	int stage_bytes;
	uint64_t* full;      // [NST]
	uint64_t* empty;     // [NST]
	const uint8_t* src0;
	const uint8_t* src1;
	int tb0, tb1, T0, T;
	int* err;

	// loading warp: every tile in order, each once its stage is free (bounded waits)
	__device__ __forceinline__ void produce()
	{
		for (int t = 0; t < T; ++t) {
			const int st = t % NST;
			if (t >= NST && !tc::mbar_wait(&empty[st], (uint32_t)((t / NST - 1) & 1))) { fail(err, 1); return; }
			const uint8_t* src = t < T0 ? src0 + (size_t)t * tb0 : src1 + (size_t)(t - T0) * tb1;
			load_stage(ring + (size_t)st * stage_bytes, src, (uint32_t)(t < T0 ? tb0 : tb1), &full[st]);
		}
	}
};

template <int FMT, int NP, bool SLICED, int NST>
struct InterpChunk {
	InterpRing<NST>& R;
	uint64_t xd0;
	const uint32_t (&tacc)[kAccSliced];
	uint32_t idesc;
	int g0;
	bool first;
	template <int a>
	__device__ __forceinline__ void slice()
	{
		const int g = g0 + a, st = g % NST;
		if (!tc::mbar_wait(&R.full[st], (uint32_t)((g / NST) & 1))) fail(R.err, 3);
		tc::fence_after_sync();
		const uint64_t od = tc::make_sdesc(tc::smem_u32(R.ring + (size_t)st * R.stage_bytes), 128, 32 * (FMT == 1 ? 2 : 4) / 16 * 128);
		mma_slice<FMT, NP, SLICED, a>(xd0, od, tacc, idesc, first);
		tc::mma_commit_elect(&R.empty[st]);
	}
};

template <int D, int NV, int KS, int KF, int KC, int FMT, int NP, bool SLICED>
__global__ void __launch_bounds__(kBlockThreads, 1)
ks_interp(const double* __restrict__ sol, GroupDev g, const float2* __restrict__ met2, float2* __restrict__ trace,
          double* __restrict__ xl, int* __restrict__ colE, SplitArgs Acv, SplitArgs Acf, Plan P, int EB,
          int fp64_eighths, float2 bx, float2 by, float2 bz, double bxd, double byd, double bzd, int* err)
{
	extern __shared__ __align__(1024) uint8_t sm[];
	constexpr int es = (FMT == 1 ? 2 : 4);
	constexpr int chunk_bytes = NP * kRows * 32 * es;
	constexpr int NACC = SLICED ? (NP < kAccSliced ? NP : kAccSliced) : 1;
	constexpr int G = 4 * KS;                 // groups of 8 K per solution column
	constexpr int n_c_pad = 32 * KC;
	constexpr int ld_v = n_c_pad + 1;         // odd: the row-per-lane stores of s_vc are conflict-free
	constexpr int NST = ring_stages(FMT);
	constexpr uint32_t sbo = 32 * es / 16 * 128;
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int n_s = g.n_s, n_c = g.n_c, n_fl = g.n_fl, n_fc = g.n_fc;
	const int e0 = blockIdx.x * EB, ne = min(EB, g.n_vol - e0), rows = ne * NV;
	uint8_t* dig = sm + P.off_dig;
	double* SV = (double*)(sm + P.off_st);
	float2* SV2 = (float2*)SV;                // s_vc as double-floats (after the Cv contraction)
	int* colF = (int*)(sm + P.off_colF);
	int* emx = colF + kRows;                  // exponent bounds of the block's reference fluxes per data row
	int* qctr = emx + kRows;                  // next double-float volume-flux item
	uint64_t* bars = (uint64_t*)(sm + P.off_bars);
	uint64_t* done = bars + 2 * NST;         // a contraction done (tcgen05.commit)
	uint64_t* ready = bars + 2 * NST + 1;    // [KS + 1]: digits of chunk c written (c < KS) / Cv accumulators read
	uint32_t* slot = (uint32_t*)(bars + 2 * NST + 1 + KS + 1);

	if (tid < kRows) { colF[tid] = -4000; emx[tid] = -4000; }
	if (tid == 0) *qctr = 0;
	if (warp == 0) { tc::tmem_alloc(slot, 512u); tc::tmem_relinquish(); }
	if (tid == 0) {
		for (int i = 0; i < NST; ++i) { tc::mbar_init(&bars[i], 1); tc::mbar_init(&bars[NST + i], 1); }
		tc::mbar_init(done, 1);
		for (int i = 0; i <= KS; ++i) tc::mbar_init(&ready[i], kCompute);
		tc::fence_mbar_init();
	}
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	const uint32_t tmem = *slot;

	InterpRing<NST> R{sm, P.stage_bytes, bars, bars + NST, Acv.tiles, Acf.tiles, Acv.tile_bytes, Acf.tile_bytes,
	                  KS * NP, 2 * KS * NP, err};
	if (warp == kLoadWarp) {
		R.produce();
	} else if (warp == kIssueWarp) {
		// issuing warp: Cv contraction once the digits are written, Cf contraction once the Cv accumulators were read
		// one rolled loop over the chunks of both contractions: a single copy of the unrolled MMA stream of a chunk
		// (straight-line streams for every chunk are instruction-fetch bound, each runs once per block)
#pragma unroll 1
		for (int q = 0; q < 2 * KS; ++q) {
			const int k = q >= KS ? 1 : 0, c = q - k * KS;
			const int n_pad = k == 0 ? Acv.N_pad : Acf.N_pad;
			// Cv chunk c starts as soon as its digits are written; the Cf contraction reuses the Cv accumulator
			// columns, so it waits until they were read
			if (!tc::mbar_wait(&ready[k == 0 ? c : KS], 0)) fail(err, 6);
			tc::fence_after_sync();
			uint32_t tacc[kAccSliced];
			acc_addrs(tmem, n_pad, tacc);
			const uint32_t idesc = tc::make_idesc(kRows, n_pad, FMT);
			InterpChunk<FMT, NP, SLICED, NST> ch{R, tc::make_sdesc(tc::smem_u32(dig + c * chunk_bytes), 128, sbo), tacc,
			                                     idesc, q * NP, c == 0};
			SliceLoop<FMT, NP, SLICED, 0>::run(ch);
			if (c == KS - 1) tc::mma_commit_elect(done);
			__syncwarp();
		}
	} else {
		// 1. solution coefficients of the block (contiguous in memory) into registers: thread = data row
		//    m = tid & 127, K groups kg = (tid >> 7) + kGroups j; column exponent bounds by shared-memory max
		//    (staged in shared memory so that the digit loop below stays rolled: its unrolled code would be fetched
		//    once per block, which costs more than the loop)
		constexpr int NJ = G / kGroups;
		constexpr int ld_u = 32 * KS + 2;     // +2 doubles: the 16-byte reads of consecutive rows hit distinct banks
		const int m_r = tid & (kRows - 1), kg0 = tid >> 7;
		double* ST = SV;                      // the s_vc staging is free until the Cv contraction completed
		{
			// every load issued before any is used (one memory round trip); 16-byte loads when the rows are
			// 16-byte aligned (n_s even)
			const double* src = sol + ((size_t)e0 * NV + m_r) * n_s;
			double x[NJ][8];
			if ((n_s & 1) == 0 && m_r < rows) {
#pragma unroll
				for (int j = 0; j < NJ; ++j)
#pragma unroll
					for (int h = 0; h < 4; ++h) {
						const int k = 8 * (kg0 + kGroups * j) + 2 * h;
						const double2 t = k < n_s ? *(const double2*)(src + k) : make_double2(0.0, 0.0);
						x[j][2 * h] = t.x; x[j][2 * h + 1] = t.y;
					}
			} else {
#pragma unroll
				for (int j = 0; j < NJ; ++j)
#pragma unroll
					for (int jj = 0; jj < 8; ++jj) {
						const int k = 8 * (kg0 + kGroups * j) + jj;
						x[j][jj] = (m_r < rows && k < n_s) ? src[k] : 0.0;
					}
			}
			int e = -4000;
#pragma unroll
			for (int j = 0; j < NJ; ++j) {
#pragma unroll
				for (int jj = 0; jj < 8; ++jj) e = max(e, exp_bound(x[j][jj]));
#pragma unroll
				for (int h = 0; h < 4; ++h)
					*(double2*)(ST + m_r * ld_u + 8 * (kg0 + kGroups * j) + 2 * h) = make_double2(x[j][2 * h], x[j][2 * h + 1]);
			}
			atomicMax(&colF[m_r], e);
		}
		compute_sync();
		const int F_r = col_exp_of(colF[m_r], NP);
		// 2. digits of all solution chunks (kept for both contractions)
#pragma unroll 1
		for (int j = 0; j < NJ; ++j) {
			const int kg = kg0 + kGroups * j;
			double x[8];
#pragma unroll
			for (int h = 0; h < 4; ++h) {
				const double2 t = *(const double2*)(ST + m_r * ld_u + 8 * kg + 2 * h);
				x[2 * h] = t.x; x[2 * h + 1] = t.y;
			}
			store_digits8<FMT, NP, SLICED>(dig + (kg >> 2) * chunk_bytes, m_r, 8 * (kg & 3), x, F_r);
			if ((j + 1) % kItemsPerChunk == 0) {   // the thread's last item of chunk j / kItemsPerChunk: publish it
				tc::fence_async_smem();
				mbar_arrive(&ready[j / kItemsPerChunk]);
			}
		}
		compute_sync();   // every thread has read colF
		if (tid < kRows) colF[tid] = F_r;
		compute_sync();

		// 3. s_vc = Cv * U (accumulators) -> staging
		if (!tc::mbar_wait(done, 0)) fail(err, 5);
		tc::fence_after_sync();
		const int m_t = 32 * (warp & 3) + lane;
		const uint32_t trow = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
		for (int c8 = warp >> 2; c8 < Acv.N_pad / 8; c8 += kColStride) {
			df::df64 v8[8];
			combine8_df<SLICED, NACC>(trow, Acv.N_pad, 8 * c8, Acv.row_exp, colF[m_t], m_t < rows, v8);
			if (m_t >= rows) continue;
#pragma unroll
			for (int j = 0; j < 8; ++j) {
				const int node = 8 * c8 + j;
				if (node < n_c) SV2[m_t * ld_v + node] = df::to2(v8[j]);
			}
		}
		// 4. the Cf contraction (same digits, same accumulator columns) starts once every thread read its Cv columns
		tc::fence_before_sync();
		mbar_arrive(&ready[KS]);
		compute_sync();

		// 5. reference volume fluxes -> global lift operand [element][variable][32 KF + r * n_c_pad + node], exponent
		//    bounds.
		//    Work items (element, 32-node chunk), split between the two arithmetic pipes, which run side by side: the
		//    first fp64_eighths / 8 of the items in FP64 on warps 0..7 (FP64-pipe bound, few issue slots), the
		//    rest in double-float arithmetic on the FP32 pipe, taken from a shared counter by warps 8..15 and by
		//    warps 0..7 once their FP64 items are done.  The results are written as doubles; the exponent bounds
		//    meet in shared memory.
		{
			constexpr int LDX = 32 * (KF + D * KC);   // row of the lift operand
			const df::df64 b2[3] = {df::from2(bx), df::from2(by), df::from2(bz)};
			const double bd[3] = {bxd, byd, bzd};
			// FP64 items: the share rounded down to whole rounds of the FP64 warps (a second FP64 item on one warp
			// would outlast everything else: an FP64 item takes ~1.5x a double-float one at this pipe balance)
			constexpr int W64 = kComputeWarps / 2;
			const int n_items = ne * KC, n64 = (n_items * fp64_eighths / 8) / W64 * W64;
			const bool fp64w = warp < kComputeWarps / 2;
			int it = fp64w ? warp : n_items;   // warps 0..7: the FP64 items warp, warp + 8, .. first
#pragma unroll 1
			for (;;) {   // rolled: one copy of each flux code
				if (!(fp64w && it < n64)) {   // then double-float items from the shared counter, as they come
					int t = 0;
					if (lane == 0) t = atomicAdd(qctr, 1);
					it = n64 + __shfl_sync(0xffffffffu, t, 0);
					if (it >= n_items) break;
				}
				const bool fp64 = it < n64;   // the arithmetic of an item depends on its index only
				const int el = it / KC, jc = it - el * KC;
				const int e = e0 + el, c = 32 * jc + lane;
				int emax[NV];
#pragma unroll
				for (int v = 0; v < NV; ++v) emax[v] = -4000;
				double* dst = xl + (size_t)e * NV * LDX + 32 * KF + c;
				const bool live = c < n_c;
				if (fp64) {
					double sv[NV];
#pragma unroll
					for (int v = 0; v < NV; ++v) sv[v] = live ? df::to_double(df::from2(SV2[(el * NV + v) * ld_v + c])) : 1.0;
					const double* me = g.met + (size_t)e * D * D;
					ref_flux_rows<D, NV>(sv, [&](int x, int r) { return me[x + D * r]; }, bd, [&](int r, const double (&fr)[NV]) {
#pragma unroll
						for (int v = 0; v < NV; ++v) {
							const double y = live ? fr[v] : 0.0;   // padding nodes: zero (finite) lift operand
							dst[(size_t)v * LDX + r * n_c_pad] = y;
							emax[v] = max(emax[v], exp_bound(y));
						}
					});
				} else {
					df::df64 sv[NV];
#pragma unroll
					for (int v = 0; v < NV; ++v) sv[v] = live ? df::from2(SV2[(el * NV + v) * ld_v + c]) : df::mk(1.f);
					const float2* me = met2 + (size_t)e * D * D;
					df::ref_flux_rows<D, NV>(sv, [&](int x, int r) { return df::from2(me[x + D * r]); }, b2,
					                         [&](int r, const df::df64 (&fr)[NV]) {
#pragma unroll
						for (int v = 0; v < NV; ++v) {
							const df::df64 y = live ? fr[v] : df::mk(0.f);
							dst[(size_t)v * LDX + r * n_c_pad] = df::to_double(y);
							emax[v] = max(emax[v], df::exp_bound(y));
						}
					});
				}
#pragma unroll
				for (int v = 0; v < NV; ++v) {
					int ev = emax[v];
#pragma unroll
					for (int o = 16; o > 0; o >>= 1) ev = max(ev, __shfl_xor_sync(0xffffffffu, ev, o));
					if (lane == 0) atomicMax(&emx[el * NV + v], ev);
				}
				if (fp64) it += W64;
			}
		}

		// 6. traces: TMEM -> the element-ordered trace buffer [element][variable][local face * n_fc + node] as FP32
		//    pairs, straight from registers: 8 consecutive face nodes (64 bytes) per thread and column block (the
		//    face kernel gathers both sides of a face through its static side table)
		if (!tc::mbar_wait(done, 1)) fail(err, 5);
		tc::fence_after_sync();
		const int nfq = n_fl * n_fc;   // odd for triangles of even order: rows then start on 8-byte boundaries only
		float2* trow_g = trace + ((size_t)e0 * NV + m_t) * nfq;
		const bool row16 = ((reinterpret_cast<uintptr_t>(trow_g) & 15u) == 0);   // 16-byte stores allowed
		for (int c8 = warp >> 2; c8 < Acf.N_pad / 8; c8 += kColStride) {
			df::df64 v8[8];
			combine8_df<SLICED, NACC>(trow, Acf.N_pad, 8 * c8, Acf.row_exp, colF[m_t], m_t < rows, v8);
			if (m_t >= rows) continue;
			if (row16 && 8 * c8 + 8 <= nfq) {
				float4* d4 = (float4*)(trow_g + 8 * c8);
#pragma unroll
				for (int h = 0; h < 4; ++h)
					d4[h] = make_float4(v8[2 * h].hi, v8[2 * h].lo, v8[2 * h + 1].hi, v8[2 * h + 1].lo);
			} else {
#pragma unroll
				for (int j = 0; j < 8; ++j)
					if (8 * c8 + j < nfq) trow_g[8 * c8 + j] = df::to2(v8[j]);
			}
		}
		compute_sync();   // every volume-flux item done: the exponent bounds are complete
		if (tid < rows) colE[((size_t)e0 * NV + tid) * kColSlots + g.n_fl] = emx[tid];
	}
	tc::fence_before_sync();
	__syncthreads();
	if (warp == 0) tc::tmem_dealloc(tmem, 512u);
}

// ------------------------------------------------------------------------------------------------------------
// ks_lift: rhs = L' * X of a block of EB elements (X = [face fluxes | reference volume fluxes], the lift operand
// rows), 1/detJ, RK stage update, ||rhs||_inf (L' = m_inv_ref [-tw0 | tw1] with K ordered face part first).
// The data digits go to TMEM and the MMAs read them from there (A operand in TMEM: an MMA then reads only the
// operator slice from shared memory, 32 instead of 48 cycles at N = 64).  TMEM: the kAccSliced accumulators in
// columns 0..kDigCol-1, then a ring of HS slots of half-chunks (16 K values x NP parts): half-chunk H (chunk H / 2,
// K 16 (H % 2)..) in slot H % HS; HS = as many as fit, at most 4 (with 4 each thread half owns two slots).  Operator chunks go to kSlotsL whole-chunk shared-memory
// slots (chunk c in slot c % kSlotsL), loaded by the loading warp.
// ------------------------------------------------------------------------------------------------------------
constexpr int kMaxHalfSlots = 4;
constexpr uint32_t kDigCol = 320;   // first TMEM column of the digit slots (5 accumulators of N <= 64 below it)

// TMEM columns of one data part of a half-chunk (16 K values: 8 columns of BF16 pairs, 16 of TF32).
template <int FMT>
__host__ __device__ constexpr int half_part_cols() { return FMT == 1 ? 8 : 16; }
// half-chunk slots beside the accumulators (S = 7 BF16: 3; S = 6: 4)
template <int FMT, int NP>
__host__ __device__ constexpr int half_slots()
{
	return (512 - (int)kDigCol) / (NP * half_part_cols<FMT>()) < kMaxHalfSlots
	           ? (512 - (int)kDigCol) / (NP * half_part_cols<FMT>()) : kMaxHalfSlots;
}

// MMA stream of operator slice a against the data parts of one half-chunk in TMEM (A operand) (the products and
// accumulator levels of mma_slice).
template <int FMT, int NP, bool SLICED, int a>
__device__ __forceinline__ void mma_slice_ts(uint32_t xa0, uint64_t od, const uint32_t (&tacc)[kAccSliced], uint32_t idesc,
                                             bool first)
{
	constexpr int KSH = (FMT == 1 ? 1 : 2);   // MMA K steps of a half-chunk (K 16 per BF16 MMA, 8 per TF32 MMA)
	constexpr int pc = half_part_cols<FMT>();
	constexpr int nb = SLICED ? NP - a : (a == 0 ? 2 : 1);
#pragma unroll
	for (int ks = 0; ks < KSH; ++ks) {
#pragma unroll
		for (int b = 0; b < nb; ++b) {
			const int L = SLICED ? (a + b < kAccSliced - 1 ? a + b : kAccSliced - 1) : 0;
			const bool init_slot = ks == 0 && a == 0 && (SLICED ? b <= kAccSliced - 1 : b == 0);
			const uint32_t acc = (first && init_slot) ? 0u : 1u;
			const uint32_t xa = xa0 + (uint32_t)(b * pc + 8 * ks);
			if constexpr (FMT == 1) tc::mma_bf16_ts_elect(tacc[L], xa, od + 16 * ks, idesc, acc);
			else tc::mma_tf32_ts_elect(tacc[L], xa, od + 16 * ks, idesc, acc);
		}
	}
}

template <int FMT, int NP, bool SLICED>
struct LiftHalf {
	uint32_t xa0;         // TMEM address of part 0 of the half-chunk's slot
	uint64_t od;          // slice 0 of the chunk's operator slot at the half's first K step (slice a at a * tile_bytes)
	const uint32_t (&tacc)[kAccSliced];
	uint32_t idesc;
	bool first;
	int tile_bytes;
	template <int a>
	__device__ __forceinline__ void slice()
	{
		mma_slice_ts<FMT, NP, SLICED, a>(xa0, od + (uint64_t)(((uint32_t)a * (uint32_t)tile_bytes) >> 4), tacc, idesc, first);
	}
};

template <int S, int s>
__device__ __forceinline__ void store_slices_tmem(uint32_t ta, const uint32_t (&lo)[8], const uint32_t (&hi)[8],
                                                  const uint32_t (&lead)[8])
{
	if constexpr (s < S) {
		tc::tmem_st4(ta + (uint32_t)(s * half_part_cols<1>()), digit_row<S, s>(lo, hi, lead));
		store_slices_tmem<S, s + 1>(ta, lo, hi, lead);
	}
}

// Digits / split parts of 8 consecutive K values of this thread's data row into TMEM: ta = the thread's lane and the
// column of its values in part 0 (parts half_part_cols apart).  Asynchronous: tmem_st_wait before handing over.
template <int FMT, int NP, bool SLICED>
__device__ __forceinline__ void store_digits8_tmem(uint32_t ta, const double (&x)[8], int F)
{
	constexpr int pc = half_part_cols<FMT>();
	if constexpr (SLICED) {
		const int sc = 8 * NP - F;
		uint32_t lo[8], hi[8], lead[8];
#pragma unroll
		for (int j = 0; j < 8; ++j) {
			const long long mm = scaled_mantissa(x[j], sc) + digit_bias<NP>();
			lo[j] = (uint32_t)mm;
			hi[j] = (uint32_t)((unsigned long long)mm >> 32);
			lead[j] = (uint32_t)((int)(mm >> (8 * (NP - 1))) + 128);
		}
		store_slices_tmem<NP, 0>(ta, lo, hi, lead);
	} else if constexpr (FMT == 1) {
		float h[8], l[8];
#pragma unroll
		for (int j = 0; j < 8; ++j) {
			const float xf = (float)x[j];
			h[j] = __bfloat162float(__float2bfloat16_rn(xf));
			l[j] = xf - h[j];
		}
		tc::tmem_st4(ta, make_uint4(pack_bf16x2(h[0], h[1]), pack_bf16x2(h[2], h[3]), pack_bf16x2(h[4], h[5]), pack_bf16x2(h[6], h[7])));
		tc::tmem_st4(ta + pc, make_uint4(pack_bf16x2(l[0], l[1]), pack_bf16x2(l[2], l[3]), pack_bf16x2(l[4], l[5]), pack_bf16x2(l[6], l[7])));
	} else {
		uint32_t h[8], l[8];
#pragma unroll
		for (int j = 0; j < 8; ++j) {
			const float xf = (float)x[j];
			h[j] = tf32_bits(xf);
			l[j] = tf32_bits(xf - __uint_as_float(h[j]));
		}
		tc::tmem_st8(ta, h);
		tc::tmem_st8(ta + pc, l);
	}
}

template <int D, int NV, int KF, int KC, int FMT, int NP, bool SLICED>
__global__ void __launch_bounds__(kBlockThreads, 1)
ks_lift(double* __restrict__ sol, double* __restrict__ solp, double* __restrict__ rhs, const double* __restrict__ xl,
        const int* __restrict__ colE, GroupDev g,
        SplitArgs Al, Plan P, int EB, const double* __restrict__ dt_ptr, unsigned long long* max_slot, int stage,
        int write_rhs, int* err)
{
	static_assert(kItemsPerChunk == 1 && kGroups == 4, "one K group of 8 per thread and chunk: threads 256 h.. write half h");
	extern __shared__ __align__(1024) uint8_t sm[];
	constexpr int es = (FMT == 1 ? 2 : 4);
	constexpr int NACC = SLICED ? (NP < kAccSliced ? NP : kAccSliced) : 1;
	constexpr int KL = KF + D * KC;
	constexpr int LDX = 32 * KL;
	constexpr int KSH = es / 2;                          // MMA K steps per half-chunk
	constexpr int pc = half_part_cols<FMT>();
	constexpr uint32_t slot_cols = (uint32_t)(NP * pc);
	constexpr uint32_t sbo = 32 * es / 16 * 128;
	constexpr int HS = half_slots<FMT, NP>();
	static_assert(HS >= 3 && kDigCol + HS * NP * half_part_cols<FMT>() <= 512, "TMEM columns");
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int n_s = g.n_s;
	const int e0 = blockIdx.x * EB, ne = min(EB, g.n_vol - e0), rows = ne * NV;
	int* colF = (int*)(sm + P.off_colF);
	uint64_t* bars = (uint64_t*)(sm + P.off_bars);
	uint64_t* full = bars;                       // [kSlotsL] operator chunk landed
	uint64_t* odone = bars + kSlotsL;            // [kSlotsL] MMAs of chunk c done: operator slot c % kSlotsL free
	uint64_t* hready = bars + 2 * kSlotsL;       // [HS] digits of half-chunk H written (256 threads)
	uint64_t* hdone = hready + HS;       // [HS] MMAs of half-chunk H done: its TMEM slot free
	uint64_t* fin = hdone + HS;          // all MMAs done
	uint32_t* slot = (uint32_t*)(fin + 1);
	const uint32_t op_bytes = (uint32_t)(NP * Al.tile_bytes);

	if (warp == 0) { tc::tmem_alloc(slot, 512u); tc::tmem_relinquish(); }
	if (tid == 0) {
		for (int i = 0; i < kSlotsL; ++i) { tc::mbar_init(&full[i], 1); tc::mbar_init(&odone[i], 1); }
		for (int i = 0; i < HS; ++i) { tc::mbar_init(&hready[i], kCompute / 2); tc::mbar_init(&hdone[i], 1); }
		tc::mbar_init(fin, 1);
		tc::fence_mbar_init();
	}
	tc::fence_before_sync();
	__syncthreads();
	tc::fence_after_sync();
	const uint32_t tmem = *slot;

	if (warp == kLoadWarp) {
		// loading warp: operator chunk n into slot n % kSlotsL once chunk n - kSlotsL's MMAs are done
		for (int n = 0; n < KL; ++n) {
			const int sl = n % kSlotsL;
			if (n >= kSlotsL && !tc::mbar_wait(&odone[sl], (uint32_t)((n / kSlotsL - 1) & 1))) { fail(err, 1); break; }
			load_stage(sm + (size_t)sl * P.stage_bytes, Al.tiles + (size_t)n * op_bytes, op_bytes, &full[sl]);
		}
	} else if (warp == kIssueWarp) {
		// issuing warp: one MMA stream per half-chunk
		uint32_t tacc[kAccSliced];
		acc_addrs(tmem, Al.N_pad, tacc);
		const uint32_t idesc = tc::make_idesc(kRows, Al.N_pad, FMT);
#pragma unroll 1
		for (int H = 0; H < 2 * KL; ++H) {
			const int c = H >> 1, h = H & 1, s = H % HS;
			if (h == 0 && !tc::mbar_wait(&full[c % kSlotsL], (uint32_t)((c / kSlotsL) & 1))) fail(err, 3);
			if (!tc::mbar_wait(&hready[s], (uint32_t)((H / HS) & 1))) fail(err, 6);
			tc::fence_after_sync();
			LiftHalf<FMT, NP, SLICED> ch{tmem + kDigCol + (uint32_t)s * slot_cols,
			                             tc::make_sdesc(tc::smem_u32(sm + (size_t)(c % kSlotsL) * P.stage_bytes), 128, sbo) +
			                                 (uint64_t)(16 * KSH * h),
			                             tacc, idesc, H == 0, Al.tile_bytes};
			SliceLoop<FMT, NP, SLICED, 0>::run(ch);
			tc::mma_commit_elect(&hdone[s]);
			if (h == 1) tc::mma_commit_elect(&odone[c % kSlotsL]);
			__syncwarp();
		}
		tc::mma_commit_elect(fin);
		__syncwarp();
	} else {
		// column scales from the exponent bounds of the rows: the largest of the row's face parts and volume part
		if (tid < kRows) {
			int m = -4000;
			if (tid < rows) {   // the row's 8 slots in two 16-byte loads
				const int4* ce = reinterpret_cast<const int4*>(colE + ((size_t)e0 * NV + tid) * kColSlots);
				const int4 a = ce[0], b = ce[1];
				m = max(max(max(a.x, a.y), max(a.z, a.w)), max(max(b.x, b.y), max(b.z, b.w)));
			}
			colF[tid] = tid < rows ? col_exp_of(m, NP) : 0;
		}
		compute_sync();

		// thread items: data row m_r, K group kg0 = tid >> 7 of each chunk, i.e. half h_r = kg0 >> 1 (threads
		// 256 h_r ..) at K offset 8 (kg0 & 1) within it; the raw values of a chunk are loaded two chunks ahead of
		// its digits (registers), so the global latency is covered
		const int m_r = tid & (kRows - 1), kg0 = tid >> 7, h_r = kg0 >> 1;
		const int F_r = colF[m_r];
		const double* xrow = xl + ((size_t)e0 * NV + m_r) * LDX;   // the block's rows are contiguous
		const uint32_t ta0 = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + kDigCol + (uint32_t)((kg0 & 1) * (pc / 2));
		auto load_chunk = [&](int c, double (&xv)[8]) {
			if (m_r >= rows) {
#pragma unroll
				for (int jj = 0; jj < 8; ++jj) xv[jj] = 0.0;
			} else {
				const double2* p = (const double2*)(xrow + 32 * c + 8 * kg0);
#pragma unroll
				for (int h = 0; h < 4; ++h) { const double2 t2 = p[h]; xv[2 * h] = t2.x; xv[2 * h + 1] = t2.y; }
			}
		};
		// three register sets in rotation, the loop unrolled by three: chunk c + 3 is loaded into the set of chunk c
		// right after its digits are written, so every load has two chunks of digit work to land in (a register move
		// of a set would wait for its pending loads, i.e. shorten that distance to one chunk)
		auto digits = [&](int c, const double (&xv)[8]) {
			const int H = 2 * c + h_r, s = H % HS;
			// the slot is free once half-chunk H - HS's MMAs are done
			if (H >= HS && !tc::mbar_wait(&hdone[s], (uint32_t)(((H - HS) / HS) & 1))) fail(err, 2);
			tc::fence_after_sync();
			store_digits8_tmem<FMT, NP, SLICED>(ta0 + (uint32_t)s * slot_cols, xv, F_r);
			tc::tmem_st_wait();
			tc::fence_before_sync();
			mbar_arrive(&hready[s]);
		};
		double x0[8], x1[8], x2[8];
		load_chunk(0, x0);
		if (KL > 1) load_chunk(1, x1);
		if (KL > 2) load_chunk(2, x2);
#pragma unroll 1
		for (int c = 0; c < KL; c += 3) {
			digits(c, x0);
			if (c + 3 < KL) load_chunk(c + 3, x0);
			if (c + 1 < KL) {
				digits(c + 1, x1);
				if (c + 4 < KL) load_chunk(c + 4, x1);
			}
			if (c + 2 < KL) {
				digits(c + 2, x2);
				if (c + 5 < KL) load_chunk(c + 5, x2);
			}
		}
		// epilogue, fused: each thread owns data row m (its TMEM lane) and the 8-node column blocks c8 = warp / 4 +
		// kColStride j; per block the accumulators are combined exactly, scaled (row, column, 1/detJ) in double-float
		// arithmetic and the rhs / RK stage written, 64 contiguous bytes per row.  The state rows of the first block are loaded before the wait for
		// the last MMAs, so their latency overlaps the tensor pipe's tail.
		const int m = 32 * (warp & 3) + lane;
		const bool live = m < rows;
		const uint32_t trow = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
		const double dt = (stage >= 0 ? *dt_ptr : 0.0);
		const df::df64 jv = df::from2(df::split_double(live ? g.jinv[e0 + m / NV] : 0.0));
		const int Fm = colF[m];
		const size_t rbase = ((size_t)e0 * NV + m) * n_s;   // the row's first node
		double u0[8], up[8];
		auto load_state = [&](int c8) {
#pragma unroll
			for (int j = 0; j < 8; ++j) {
				const int node = 8 * c8 + j;
				const bool in = live && node < n_s;
				u0[j] = (in && stage >= 0) ? sol[rbase + node] : 0.0;
				up[j] = (in && stage >= 1) ? solp[rbase + node] : 0.0;
			}
		};
		int c8 = warp >> 2;
		if (c8 < Al.N_pad / 8) load_state(c8);
		if (!tc::mbar_wait(fin, 0)) fail(err, 4);
		tc::fence_after_sync();
		unsigned long long lmax = 0;   // max |rhs| as IEEE bits (NaN patterns order above +inf)
#pragma unroll 1
		for (; c8 < Al.N_pad / 8; c8 += kColStride) {
			df::df64 v8[8];
			combine8_exact_df<SLICED, NACC>(trow, Al.N_pad, 8 * c8, v8);
#pragma unroll
			for (int j = 0; j < 8; ++j) {
				const int node = 8 * c8 + j;
				if (!live || node >= n_s) continue;
				df::df64 y = v8[j];
				if constexpr (SLICED) y = df::scale_pow2(y, Al.row_exp[node] + Fm - 48);
				// the residual in double-float (~2^-47 relative): it enters the state only through dt * r, so the
				// stage update below (FP64, the only FP64 instructions here) keeps the state's full precision
				const double r = df::to_double(df::mul(y, jv));
				const unsigned long long ab = (unsigned long long)__double_as_longlong(r) & 0x7FFFFFFFFFFFFFFFull;
				lmax = ab > lmax ? ab : lmax;
				const size_t gi = rbase + node;
				if (write_rhs) rhs[gi] = r;
				if (stage == 0) { solp[gi] = u0[j]; sol[gi] = u0[j] + dt * r; }
				else if (stage == 1) sol[gi] = (1.0 / 4.0) * (3.0 * up[j] + u0[j] + dt * r);
				else if (stage == 2) sol[gi] = (1.0 / 3.0) * (up[j] + 2.0 * u0[j] + 2.0 * dt * r);
			}
			if (c8 + kColStride < Al.N_pad / 8) load_state(c8 + kColStride);
		}
		for (int off = 16; off > 0; off >>= 1) {
			const unsigned long long o = __shfl_xor_sync(0xffffffffu, lmax, off);
			lmax = o > lmax ? o : lmax;
		}
		if (lane == 0) atomicMax(max_slot, lmax);
	}
	tc::fence_before_sync();
	__syncthreads();
	if (warp == 0) tc::tmem_dealloc(tmem, 512u);
}

// ------------------------------------------------------------------------------------------------------------
// launchers
// ------------------------------------------------------------------------------------------------------------
__host__ inline SplitArgs args_of(const SplitOp& op) { return SplitArgs{op.tiles, op.row_exp, op.N_pad, (int)op.tile_bytes}; }

template <int D, int NV, int KS, int KF, int KC, int FMT, int NP, bool SLICED>
void launch_interp(dpg_gpu_ctx* c, const SplitState* st)
{
	ks_interp<D, NV, KS, KF, KC, FMT, NP, SLICED><<<st->n_blocks, kBlockThreads, st->pi.smem_bytes, c->stream>>>(
	    c->sol, c->g, st->met2, (float2*)c->trace, st->xl, st->colE, args_of(st->cv), args_of(st->cf), st->pi,
	    st->EB, st->fp64_eighths, st->b2[0], st->b2[1], st->b2[2], c->b_adv[0], c->b_adv[1], c->b_adv[2], st->err);
}

template <int D, int NV, int KS, int KF, int KC, int FMT, int NP, bool SLICED>
void launch_lift(dpg_gpu_ctx* c, const SplitState* st, int stage, int write_rhs, unsigned long long* max_slot)
{
	ks_lift<D, NV, KF, KC, FMT, NP, SLICED><<<st->n_blocks, kBlockThreads, st->pl.smem_bytes, c->stream>>>(
	    c->sol, c->solp, c->rhs, st->xl, st->colE, c->g, args_of(st->lift), st->pl, st->EB,
	    c->ddt, max_slot, stage, write_rhs, st->err);
}

// Each (mode, shape) instantiation lives in exactly one translation unit (split_inst_*.cu): a kernel registered by
// two units can receive its shared-memory opt-in in one module and be launched from the other.
template <int D, int NV, int KS, int KF, int KC, int FMT, int NP, bool SLICED>
KernelTable table_of()
{
	return KernelTable{launch_interp<D, NV, KS, KF, KC, FMT, NP, SLICED>, launch_lift<D, NV, KS, KF, KC, FMT, NP, SLICED>,
	                   (const void*)ks_interp<D, NV, KS, KF, KC, FMT, NP, SLICED>,
	                   (const void*)ks_lift<D, NV, KF, KC, FMT, NP, SLICED>};
}

// The (d, NV, solution K chunks, face K chunks, volume-node chunks) combinations instantiated: Euler/advection on
// QUAD p1..4 and HEX p1..3.
#define DPG_SPLIT_CASES(X)  \
	X(3, 5, 2, 3, 2)  /* HEX p3 Euler  */ \
	X(3, 5, 1, 2, 1)  /* HEX p2 Euler  */ \
	X(3, 5, 1, 1, 1)  /* HEX p1 Euler  */ \
	X(2, 4, 1, 1, 1)  /* QUAD p1..4 Euler */ \
	X(2, 1, 1, 1, 1)  /* QUAD advection; TRI p1..4 advection */ \
	X(3, 1, 2, 3, 2)  /* HEX p3 advection */ \
	X(3, 1, 1, 2, 1)  /* HEX p2 advection; TET p3 advection */ \
	X(3, 1, 1, 1, 1)  /* HEX p1 advection; TET p1, p2 advection */

} // namespace split
} // namespace dpg
