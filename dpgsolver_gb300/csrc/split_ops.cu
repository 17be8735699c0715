// Host side of the split-precision path: operator slicing, shared-memory plans and block shapes, kernel
// selection, the face kernel (mode-independent) and the launches.  The contraction kernels are in
// split_kernels.cuh, instantiated per mode in split_inst_*.cu.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <vector>

#include "split_kernels.cuh"

namespace dpg {
namespace split {

constexpr int kSmemMax = 227 * 1024;
constexpr int kSmemOneBlock = 116 * 1024;   // requests at least this much: one block per SM (512 TMEM columns)

// ------------------------------------------------------------------------------------------------------------
// ks_face: numerical flux at every face node (the formulas of k_face of the FP64 form, in double-float arithmetic
// on traces -- element-ordered, gathered through the side table -- and geometry held as FP32 pairs), scaled by the
// face Jacobian and stored in FP64 straight into the lift operand rows of the face's two elements (the right one
// negated, at its own node nc[q]), with the exponent bound of the face's part of each row in that part's own slot.
// 32 / n_fc faces per warp, so a face's nodes are consecutive lanes of one warp.
// ------------------------------------------------------------------------------------------------------------
template <int D, int NV>
__global__ void __launch_bounds__(256, 4) ks_face(const float2* __restrict__ trace, FaceDev fd, const float2* __restrict__ nrm2,
                                               const float2* __restrict__ jf2, const int* __restrict__ fel, int n_fl,
                                               double* __restrict__ xl, int ldx, int* __restrict__ colE, int num_flux,
                                               float2 bx, float2 by, float2 bz)
{
	using df::df64;
	const int n_fc = fd.n_fc, fpw = 32 / n_fc;
	const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
	const int f = gw * fpw + lane / n_fc, q = lane - (lane / n_fc) * n_fc;
	const bool active = lane < fpw * n_fc && f < fd.n_face;
	df64 nf[NV];
	double nfd[NV];
#pragma unroll
	for (int v = 0; v < NV; ++v) { nf[v] = df::mk(0.f); nfd[v] = 0.0; }
	int elf[2] = {0, 0};
	if (active) {
		const int t = f * n_fc + q;
		const int qr = fd.nc[t];
		elf[0] = fel[2 * f]; elf[1] = fel[2 * f + 1];
		// traces in element order [element][variable][local face * n_fc + node]; the right side at its node qr
		const int nfq = n_fl * n_fc;
		const int eL0 = elf[0] / n_fl, eR0 = elf[1] / n_fl;
		const float2* tL = trace + (size_t)eL0 * NV * nfq + (elf[0] - eL0 * n_fl) * n_fc + q;
		const float2* tR = trace + (size_t)eR0 * NV * nfq + (elf[1] - eR0 * n_fl) * n_fc + qr;
		df64 WL[NV], WR[NV], n[D];
#pragma unroll
		for (int v = 0; v < NV; ++v) {
			WL[v] = df::from2(tL[(size_t)v * nfq]);
			WR[v] = df::from2(tR[(size_t)v * nfq]);
		}
#pragma unroll
		for (int a = 0; a < D; ++a) n[a] = df::from2(nrm2[(size_t)t * D + a]);
		if constexpr (NV == D + 2) {
			if (num_flux == DPG_NUM_FLUX_ROE_PIKE) df::numflux_roe_pike<D>(WL, WR, n, nf);
			else                                   df::numflux_lax_friedrichs<D>(WL, WR, n, nf);
		} else {
			const df64 b[3] = {df::from2(bx), df::from2(by), df::from2(bz)};
			nf[0] = df::numflux_upwind<D>(b, WL[0], WR[0], n);
		}
		const df64 j = df::from2(jf2[t]);
		// rows of the lift operand: element * NV + v; K = local face * n_fc + node
		const int eL = elf[0] / n_fl, lfL = elf[0] - eL * n_fl, eR = elf[1] / n_fl, lfR = elf[1] - eR * n_fl;
		double* dL = xl + (size_t)eL * NV * ldx + lfL * n_fc + q;
		double* dR = xl + (size_t)eR * NV * ldx + lfR * n_fc + qr;
#pragma unroll
		for (int v = 0; v < NV; ++v) {
			nfd[v] = df::to_double(df::mul(nf[v], j));
			dL[(size_t)v * ldx] = nfd[v];
			dR[(size_t)v * ldx] = -nfd[v];
		}
	}
#pragma unroll
	for (int v = 0; v < NV; ++v) {
		int e = active ? exp_bound(nfd[v]) : -4000;
		for (int off = 1; off < n_fc; off <<= 1) {
			const int o = __shfl_down_sync(0xffffffffu, e, off);
			if (q + off < n_fc) e = max(e, o);
		}
		if (active && q == 0) {   // the face's slot in each side's row: one writer per slot, no atomics
			const int eL = elf[0] / n_fl, eR = elf[1] / n_fl;
			colE[((size_t)eL * NV + v) * kColSlots + (elf[0] - eL * n_fl)] = e;
			colE[((size_t)eR * NV + v) * kColSlots + (elf[1] - eR * n_fl)] = e;
		}
	}
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

static void free_state(SplitState* st)
{
	free_op(st->cv); free_op(st->cf); free_op(st->lift);
	if (st->xl) cudaFree(st->xl);
	if (st->colE) cudaFree(st->colE);
	if (st->fel) cudaFree(st->fel);
	if (st->met2) cudaFree(st->met2);
	if (st->nrm2) cudaFree(st->nrm2);
	if (st->jf2) cudaFree(st->jf2);
	if (st->err) cudaFree(st->err);
	delete st;
}

static KernelTable lookup(int mode, int S, int d, int nv, int ks, int kf, int kc)
{
	if (mode == DPG_PREC_BF16X3) return kernels_bf16x3(d, nv, ks, kf, kc);
	if (mode == DPG_PREC_TF32X3) return kernels_tf32x3(d, nv, ks, kf, kc);
	switch (S) {
	case 4: return kernels_sliced4(d, nv, ks, kf, kc);
	case 5: return kernels_sliced5(d, nv, ks, kf, kc);
	case 6: return kernels_sliced6(d, nv, ks, kf, kc);
	case 7: return kernels_sliced7(d, nv, ks, kf, kc);
	default: return KernelTable{nullptr, nullptr, nullptr, nullptr};
	}
}

static int align128(int b) { return (b + 127) / 128 * 128; }

} // namespace split

using namespace split;

void split_free(dpg_gpu_ctx* c)
{
	SplitState* st = (SplitState*)c->split;
	if (!st) return;
	free_state(st);
	c->split = nullptr;
}

int split_prepare(dpg_gpu_ctx* c)
{
	split_free(c);
	const GroupDev& g = c->g;
	if (!g.affine) return DPG_ERR_UNSUPPORTED;  // per-element m_inv on the split path: not provided
	if (c->fc.n_fc > 32 || g.n_fl + 1 > kColSlots) return DPG_ERR_UNSUPPORTED;
	SplitState* st = new SplitState();
	c->split = st;
	st->mode = c->prec_mode;
	st->S = (st->mode == DPG_PREC_BF16_SLICED ? c->n_slices : 2);
	if (st->mode == DPG_PREC_BF16_SLICED && (st->S < 2 || st->S > kMaxS)) { split_free(c); return DPG_ERR_INVALID; }
	st->nparts = st->S;
	st->fmt = (st->mode == DPG_PREC_TF32X3 ? 2 : 1);
	st->es = (st->fmt == 1 ? 2 : 4);
	const int d = c->d, NV = c->n_var;
	const int n_s = g.n_s, n_c = g.n_c, n_fl = g.n_fl, n_fc = g.n_fc;
	st->n_s_pad = (n_s + 31) / 32 * 32;
	st->n_c_pad = (n_c + 31) / 32 * 32;
	st->nf_pad = (n_fl * n_fc + 31) / 32 * 32;
	const int KS = st->n_s_pad / 32, KF = st->nf_pad / 32, KC = st->n_c_pad / 32;
	const int KL = KF + d * KC;
	st->KL = KL;
	st->kt = lookup(st->mode, st->S, d, NV, KS, KF, KC);
	if (!st->kt.interp) { split_free(c); return DPG_ERR_UNSUPPORTED; }

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
	if (nacc * std::max(st->cv.N_pad, st->cf.N_pad) > 512 || nacc * st->lift.N_pad > (int)kDigCol) { split_free(c); return DPG_ERR_UNSUPPORTED; }

	// shared-memory plans
	const int chunk_bytes = st->nparts * kRows * 32 * st->es;
	Plan& pi = st->pi;
	pi.stage_bytes = align128((int)std::max(st->cv.tile_bytes, st->cf.tile_bytes));
	const int nst_i = ring_stages(st->fmt);
	pi.off_dig = nst_i * pi.stage_bytes;
	pi.off_st = pi.off_dig + align128(KS * chunk_bytes);
	pi.off_tab = pi.off_st + align128(8 * kRows * std::max(st->n_c_pad + 1, st->n_s_pad + 2));   // s_vc or staged U
	pi.off_colF = pi.off_tab;
	pi.off_bars = pi.off_colF + 8 * kRows + 16;   // colF, the reference-flux exponent bounds, the item counter
	pi.smem_bytes = std::max(pi.off_bars + 8 * (2 * nst_i + 2 + KS) + 16, kSmemOneBlock);
	Plan& pl = st->pl;
	pl.stage_bytes = align128(st->nparts * (int)st->lift.tile_bytes);
	pl.off_dig = kSlotsL * pl.stage_bytes;
	pl.off_tab = pl.off_dig;   // digits live in TMEM; the epilogue writes from registers
	pl.off_colF = pl.off_tab;
	if (pi.smem_bytes > kSmemMax || pl.off_colF + 4 * kRows + 8 * (2 * kSlotsL + 2 * kMaxHalfSlots + 1) + 16 > kSmemMax) {
		split_free(c);
		return DPG_ERR_UNSUPPORTED;
	}

	// blocks: EB elements (EB * NV <= 128 data rows), as few whole waves of the SMs as possible, spread evenly
	int n_sm = 0;
	if (cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, c->dev) != cudaSuccess || n_sm < 1) n_sm = 1;
	st->EB = st->eb_default = wave_rule_eb(g.n_vol, NV, n_sm, 0);
	st->n_blocks = (g.n_vol + st->EB - 1) / st->EB;
	pl.off_bars = pl.off_colF + 4 * kRows;
	pl.smem_bytes = std::max(pl.off_bars + 8 * (2 * kSlotsL + 2 * kMaxHalfSlots + 1) + 16, kSmemOneBlock);
	const int fpw = 32 / n_fc;
	st->n_face_warps = (c->fc.n_face + fpw - 1) / fpw;

	const size_t n_xl = (size_t)g.n_vol * NV * 32 * KL;
	if (cudaMalloc(&st->err, sizeof(int)) != cudaSuccess || cudaMemset(st->err, 0, sizeof(int)) != cudaSuccess ||
	    cudaMalloc(&st->xl, sizeof(double) * n_xl) != cudaSuccess ||
	    cudaMemset(st->xl, 0, sizeof(double) * n_xl) != cudaSuccess ||   // padding columns stay zero
	    cudaMalloc(&st->colE, sizeof(int) * (size_t)g.n_vol * NV * kColSlots) != cudaSuccess ||
	    cudaMemset(st->colE, 0x80, sizeof(int) * (size_t)g.n_vol * NV * kColSlots) != cudaSuccess) {   // 0x80808080 < 0
		split_free(c);
		return DPG_ERR_CUDA;
	}
	// the two (element, local face) sides of every face, static for the mesh (every face has two: periodic meshes)
	{
		const size_t n_vf = (size_t)g.n_vol * n_fl;
		std::vector<int> vf(n_vf), fel((size_t)c->fc.n_face * 2, -1);
		if (cudaMemcpy(vf.data(), g.vol_face, sizeof(int) * n_vf, cudaMemcpyDeviceToHost)) { split_free(c); return DPG_ERR_CUDA; }
		for (size_t i = 0; i < n_vf; ++i) fel[(size_t)vf[i]] = (int)i;   // vol_face = (face << 1) | side
		for (int x : fel)
			if (x < 0) { split_free(c); return DPG_ERR_UNSUPPORTED; }
		if (cudaMalloc(&st->fel, sizeof(int) * fel.size()) ||
		    cudaMemcpy(st->fel, fel.data(), sizeof(int) * fel.size(), cudaMemcpyHostToDevice)) { split_free(c); return DPG_ERR_CUDA; }
	}
	// face geometry and the advection velocity as double-floats for the double-float face kernel
	{
		const size_t n_nrm = (size_t)c->fc.n_face * n_fc * d, n_jf = (size_t)c->fc.n_face * n_fc;
		std::vector<double> hn(n_nrm), hj(n_jf);
		if (cudaMemcpy(hn.data(), c->fc.nrm, sizeof(double) * n_nrm, cudaMemcpyDeviceToHost) ||
		    cudaMemcpy(hj.data(), c->fc.jf, sizeof(double) * n_jf, cudaMemcpyDeviceToHost)) { split_free(c); return DPG_ERR_CUDA; }
		std::vector<float2> n2(n_nrm), j2(n_jf);
		for (size_t i = 0; i < n_nrm; ++i) n2[i] = df::split_double(hn[i]);
		for (size_t i = 0; i < n_jf; ++i) j2[i] = df::split_double(hj[i]);
		if (cudaMalloc(&st->nrm2, sizeof(float2) * n_nrm) || cudaMalloc(&st->jf2, sizeof(float2) * n_jf) ||
		    cudaMemcpy(st->nrm2, n2.data(), sizeof(float2) * n_nrm, cudaMemcpyHostToDevice) ||
		    cudaMemcpy(st->jf2, j2.data(), sizeof(float2) * n_jf, cudaMemcpyHostToDevice)) { split_free(c); return DPG_ERR_CUDA; }
		for (int a = 0; a < 3; ++a) st->b2[a] = df::split_double(c->b_adv[a]);
		const size_t n_met = (size_t)g.n_vol * d * d;   // affine geometry (checked above): one metric per element
		std::vector<double> hm(n_met);
		if (cudaMemcpy(hm.data(), g.met, sizeof(double) * n_met, cudaMemcpyDeviceToHost)) { split_free(c); return DPG_ERR_CUDA; }
		std::vector<float2> m2(n_met);
		for (size_t i = 0; i < n_met; ++i) m2[i] = df::split_double(hm[i]);
		if (cudaMalloc(&st->met2, sizeof(float2) * n_met) ||
		    cudaMemcpy(st->met2, m2.data(), sizeof(float2) * n_met, cudaMemcpyHostToDevice)) { split_free(c); return DPG_ERR_CUDA; }
	}
	if (cudaFuncSetAttribute(st->kt.interp_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, pi.smem_bytes) ||
	    cudaFuncSetAttribute(st->kt.lift_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, pl.smem_bytes)) {
		split_free(c);
		return DPG_ERR_CUDA;
	}
	return DPG_OK;
}

template <int D, int NV>
static void launch_face_k(dpg_gpu_ctx* c, const SplitState* st)
{
	const int warps_per_block = st->face_block_warps, threads = 32 * warps_per_block;
	ks_face<D, NV><<<(st->n_face_warps + warps_per_block - 1) / warps_per_block, threads, 0, c->stream>>>(
	    (const float2*)c->trace, c->fc, st->nrm2, st->jf2, st->fel, c->g.n_fl, st->xl, 32 * st->KL, st->colE,
	    c->num_flux, st->b2[0], st->b2[1], st->b2[2]);
}

int split_launch_trace(dpg_gpu_ctx* c)
{
	SplitState* st = (SplitState*)c->split;
	if (!st) return DPG_ERR_INVALID;
	st->kt.interp(c, st);
	return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

int split_launch_face(dpg_gpu_ctx* c)
{
	SplitState* st = (SplitState*)c->split;
	if (!st) return DPG_ERR_INVALID;
	if (c->d == 3 && c->n_var == 5) launch_face_k<3, 5>(c, st);
	else if (c->d == 2 && c->n_var == 4) launch_face_k<2, 4>(c, st);
	else if (c->d == 3 && c->n_var == 1) launch_face_k<3, 1>(c, st);
	else if (c->d == 2 && c->n_var == 1) launch_face_k<2, 1>(c, st);
	else return DPG_ERR_UNSUPPORTED;
	return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

int split_launch_volume(dpg_gpu_ctx* c, int stage, bool write_rhs, unsigned long long* max_slot)
{
	SplitState* st = (SplitState*)c->split;
	if (!st) return DPG_ERR_INVALID;
	st->kt.lift(c, st, stage, write_rhs ? 1 : 0, max_slot);
	return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

int wave_rule_eb(int n_vol, int NV, int n_sm, int extra_waves)
{
	const int eb_max = kRows / NV;
	const int waves = std::max(1, ((n_vol + eb_max - 1) / eb_max + n_sm - 1) / n_sm) + extra_waves;
	return std::max(1, std::min(eb_max, (n_vol + waves * n_sm - 1) / (waves * n_sm)));
}

int split_get_tiles(dpg_gpu_ctx* c, TileConfig* t)
{
	const SplitState* st = (const SplitState*)c->split;
	if (!st) return DPG_ERR_INVALID;
	t->elems_per_block = st->EB;
	t->fp64_share_eighths = st->fp64_eighths;
	t->face_block_warps = st->face_block_warps;
	return DPG_OK;
}

int split_set_tiles(dpg_gpu_ctx* c, const TileConfig& t)
{
	SplitState* st = (SplitState*)c->split;
	if (!st) return DPG_ERR_INVALID;
	const int w = t.face_block_warps;
	if (t.elems_per_block < 1 || t.elems_per_block * c->n_var > kRows || t.fp64_share_eighths < 0 ||
	    t.fp64_share_eighths > 8 || !(w == 1 || w == 2 || w == 4 || w == 8))   // ks_face: at most 256 threads
		return DPG_ERR_INVALID;
	st->EB = t.elems_per_block;
	st->n_blocks = (c->g.n_vol + st->EB - 1) / st->EB;
	st->fp64_eighths = t.fp64_share_eighths;
	st->face_block_warps = w;
	return DPG_OK;
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
