// Fluxes of the split path in double-float arithmetic (df64.cuh): the numerical fluxes Roe-Pike, Lax-Friedrichs and
// upwind, and the reference-space volume flux.  Same formulas and operation order as the FP64 versions (flux.cuh and
// the FP64 form's volume kernel), evaluated on the FP32 pipe.  Sums use the one-TwoSum addition: its error is
// ~2^-47 of the larger operand, the forward-error behaviour of FP64 arithmetic at 48 bits (a difference of nearly
// equal operands is as accurate as the operands are); the results agree with FP64 to ~1e-14 of the flux scale.
#pragma once

#include "df64.cuh"

namespace dpg {
namespace df {

// gamma - 1 and gamma as double-floats (0.4 and 1.4 are not FP32 numbers)
__device__ __forceinline__ df64 gm1() { return df64{0.4f, (float)(0.4 - (double)0.4f)}; }
__device__ __forceinline__ df64 gam() { return df64{1.4f, (float)(1.4 - (double)1.4f)}; }

__device__ __forceinline__ df64 min_abs(df64 a, df64 b) { return abs_less(a, b) ? absd(a) : absd(b); }
__device__ __forceinline__ df64 max_abs(df64 a, df64 b) { return abs_less(b, a) ? absd(a) : absd(b); }

// Roe-Pike flux (the formula of flux.cuh numflux_roe_pike, with the entropy fix of min/max_abs_real).
template <int D>
__device__ __forceinline__ void numflux_roe_pike(const df64* WL, const df64* WR, const df64* n, df64* nF)
{
	df64 uL[D], uR[D];
	const df64 rhoL = WL[0], rhoR = WR[0], EL = WL[D + 1], ER = WR[D + 1];
	const df64 rhoL_inv = rcp(rhoL), rhoR_inv = rcp(rhoR);
	df64 V2L = mk(0.f), V2R = mk(0.f), VnL = mk(0.f), VnR = mk(0.f);
#pragma unroll
	for (int a = 0; a < D; ++a) {
		uL[a] = mul(WL[1 + a], rhoL_inv); uR[a] = mul(WR[1 + a], rhoR_inv);
		V2L = add_s(V2L, mul(uL[a], uL[a])); V2R = add_s(V2R, mul(uR[a], uR[a]));
		VnL = add_s(VnL, mul(n[a], uL[a]));  VnR = add_s(VnR, mul(n[a], uR[a]));
	}
	const df64 pL = mul(gm1(), sub_s(EL, scale(mul(rhoL, V2L), 0.5f))), HL = mul(add_s(EL, pL), rhoL_inv);
	const df64 pR = mul(gm1(), sub_s(ER, scale(mul(rhoR, V2R), 0.5f))), HR = mul(add_s(ER, pR), rhoR_inv);
	const df64 r = sqrt(mul(rhoR, rhoL_inv)), rP1_inv = rcp(add_s(r, mk(1.f))), rho = mul(r, rhoL);
	df64 u[D], Vn = mk(0.f), V2 = mk(0.f);
#pragma unroll
	for (int a = 0; a < D; ++a) {
		u[a] = mul(add_s(mul(r, uR[a]), uL[a]), rP1_inv);
		Vn = add_s(Vn, mul(n[a], u[a]));
		V2 = add_s(V2, mul(u[a], u[a]));
	}
	const df64 H = mul(add_s(mul(r, HR), HL), rP1_inv);
	const df64 c2 = mul(gm1(), sub_s(H, scale(V2, 0.5f))), c = sqrt(c2), c_inv = rcp(c);
	const df64 l1 = min_abs(sub_s(VnL, c), sub_s(Vn, c)), l5 = max_abs(add_s(VnR, c), add_s(Vn, c)), l234 = absd(Vn);
	const df64 drho = sub_s(rhoR, rhoL), dE = sub_s(ER, EL), dp = sub_s(pR, pL), dVn = sub_s(VnR, VnL);
	const df64 lc1 = sub_s(scale(add_s(l5, l1), 0.5f), l234), lc2 = scale(sub_s(l5, l1), 0.5f);
	const df64 dpc = mul(dp, c_inv), rdv = mul(rho, dVn);
	const df64 disInter1 = mul(add_s(mul(lc1, dpc), mul(lc2, rdv)), c_inv);
	const df64 disInter2 = add_s(mul(lc1, rdv), mul(lc2, dpc));
	const df64 rhoVnL = mul(rhoL, VnL), rhoVnR = mul(rhoR, VnR), pLR = add_s(pL, pR);
	nF[0] = scale(sub_s(add_s(rhoVnL, rhoVnR), add_s(mul(l234, drho), disInter1)), 0.5f);
#pragma unroll
	for (int a = 0; a < D; ++a) {
		const df64 drhou = sub_s(mul(rhoR, uR[a]), mul(rhoL, uL[a]));
		const df64 cen = add_s(add_s(mul(rhoVnL, uL[a]), mul(rhoVnR, uR[a])), mul(n[a], pLR));
		const df64 dis = add_s(add_s(mul(l234, drhou), mul(disInter1, u[a])), mul(disInter2, n[a]));
		nF[1 + a] = scale(sub_s(cen, dis), 0.5f);
	}
	const df64 cenE = add_s(mul(VnL, add_s(EL, pL)), mul(VnR, add_s(ER, pR)));
	const df64 disE = add_s(add_s(mul(l234, dE), mul(disInter1, H)), mul(disInter2, Vn));
	nF[D + 1] = scale(sub_s(cenE, disE), 0.5f);
}

// Euler physical flux f[x][eq] (for the Lax-Friedrichs flux).
template <int D>
__device__ __forceinline__ void flux_euler(const df64* s, df64 (&f)[D][D + 2])
{
	const df64 rho_inv = rcp(s[0]), E = s[D + 1];
	df64 uvw[D], V2 = mk(0.f);
#pragma unroll
	for (int a = 0; a < D; ++a) { uvw[a] = mul(s[1 + a], rho_inv); V2 = add_s(V2, mul(uvw[a], uvw[a])); }
	const df64 p = mul(gm1(), sub_s(E, scale(mul(s[0], V2), 0.5f))), Ep = add_s(E, p);
#pragma unroll
	for (int x = 0; x < D; ++x) {
		f[x][0] = s[1 + x];
#pragma unroll
		for (int a = 0; a < D; ++a) f[x][1 + a] = a == x ? add_s(mul(s[1 + a], uvw[x]), p) : mul(s[1 + a], uvw[x]);
		f[x][D + 1] = mul(Ep, uvw[x]);
	}
}

// Lax-Friedrichs flux (the formula of flux.cuh numflux_lax_friedrichs).
template <int D>
__device__ __forceinline__ void numflux_lax_friedrichs(const df64* WL, const df64* WR, const df64* n, df64* nF)
{
	df64 fl[D][D + 2], fr[D][D + 2];
	df64 V2L = mk(0.f), V2R = mk(0.f);
	const df64 iL = rcp(WL[0]), iR = rcp(WR[0]);
#pragma unroll
	for (int a = 0; a < D; ++a) {
		const df64 ul = mul(WL[1 + a], iL), ur = mul(WR[1 + a], iR);
		V2L = add_s(V2L, mul(ul, ul)); V2R = add_s(V2R, mul(ur, ur));
	}
	const df64 pL = mul(gm1(), sub_s(WL[D + 1], scale(mul(WL[0], V2L), 0.5f)));
	const df64 pR = mul(gm1(), sub_s(WR[D + 1], scale(mul(WR[0], V2R), 0.5f)));
	const df64 maxlL = add_s(sqrt(V2L), sqrt(mul(mul(gam(), pL), iL)));
	const df64 maxlR = add_s(sqrt(V2R), sqrt(mul(mul(gam(), pR), iR)));
	const df64 maxV = abs_less(maxlR, maxlL) ? maxlL : maxlR;
	flux_euler<D>(WL, fl);
	flux_euler<D>(WR, fr);
#pragma unroll
	for (int eq = 0; eq < D + 2; ++eq) {
		df64 s = mk(0.f);
#pragma unroll
		for (int x = 0; x < D; ++x) s = add_s(s, mul(n[x], add_s(fl[x][eq], fr[x][eq])));
		nF[eq] = scale(add_s(s, mul(maxV, sub_s(WL[eq], WR[eq]))), 0.5f);
	}
}

// Upwind flux of linear advection (the formula of flux.cuh numflux_upwind).
template <int D>
__device__ __forceinline__ df64 numflux_upwind(const df64* b, df64 wl, df64 wr, const df64* n)
{
	df64 bn = mk(0.f);
#pragma unroll
	for (int a = 0; a < D; ++a) bn = add_s(bn, mul(b[a], n[a]));
	const bool left = bn.hi > 2.220446049250313e-16f || (bn.hi == 2.220446049250313e-16f && bn.lo > 0.f);
	return mul(bn, left ? wl : wr);
}

// Reference-space volume flux fr[r][eq] = sum_x m[x][r] f[x][eq] (m_xr = detJ dr/dx, the cofactor metrics) of one
// node, handed to emit(r, fr_r) one reference direction at a time: the per-node quantities (1/rho, velocity,
// pressure) are formed once and the direction loop stays rolled (one copy of its code; the metric column m[.][r] is
// read by mcol(x, r)).  Euler: the contraction is taken through W_r = sum_x m[x][r] u_x.  Sums use the sloppy
// addition: each flux is accurate to ~2^-46 of its largest term, below the resolution of the row-scaled digits it
// feeds.
template <int D, int NV, class MCol, class Emit>
__device__ __forceinline__ void ref_flux_rows(const df64* s, const MCol& mcol, const df64* b, Emit&& emit)
{
	if constexpr (NV == D + 2) {
		const df64 rho_inv = rcp(s[0]), E = s[D + 1];
		df64 u[D];
#pragma unroll
		for (int a = 0; a < D; ++a) u[a] = mul(s[1 + a], rho_inv);
		df64 V2 = mul(u[0], u[0]);
#pragma unroll
		for (int a = 1; a < D; ++a) V2 = add_s(V2, mul(u[a], u[a]));
		const df64 p = mul(gm1(), add_s(E, scale(mul(s[0], V2), -0.5f))), Ep = add_s(E, p);
#pragma unroll 1
		for (int r = 0; r < D; ++r) {
			df64 m[D];
#pragma unroll
			for (int x = 0; x < D; ++x) m[x] = mcol(x, r);
			df64 W = mul(m[0], u[0]), f0 = mul(m[0], s[1]);
#pragma unroll
			for (int x = 1; x < D; ++x) { W = add_s(W, mul(m[x], u[x])); f0 = add_s(f0, mul(m[x], s[1 + x])); }
			df64 fr[NV];
			fr[0] = f0;
#pragma unroll
			for (int a = 0; a < D; ++a) fr[1 + a] = add_s(mul(s[1 + a], W), mul(m[a], p));
			fr[D + 1] = mul(Ep, W);
			emit(r, fr);
		}
	} else {
#pragma unroll 1
		for (int r = 0; r < D; ++r) {
			df64 fr[NV];
			fr[0] = mul(mcol(0, r), mul(b[0], s[0]));
#pragma unroll
			for (int x = 1; x < D; ++x) fr[0] = add_s(fr[0], mul(mcol(x, r), mul(b[x], s[0])));
			emit(r, fr);
		}
	}
}

} // namespace df
} // namespace dpg
