// Pointwise physics on the device: Euler physical flux, Roe-Pike and Lax-Friedrichs numerical fluxes, upwind
// advection flux.  FP64, one node per thread.
//
// Follows compute_Flux_T_euler (flux_euler_T.c:71-143, f at :259-298), compute_Numerical_Flux_T_euler_roe_pike
// (numerical_flux_euler_T.c:470-..., entropy fix from min/max_abs_real_T, math_functions_T.c:222-236),
// compute_Numerical_Flux_T_euler_lax_friedrichs (numerical_flux_euler_T.c:60-...) and
// compute_Numerical_Flux_T_advection_upwind (numerical_flux_advection_T.c:39-75).  The operation order of each
// formula is the reference's (up to taking repeated divisors as one reciprocal), so that FP64 results agree with
// the CPU oracle to rounding.
//
// The flux functions are templated on the scalar type: double (the residual) or dual (dual.cuh: the tangent of the
// linearisation); the double instantiations are the FP64 formulas above, operation for operation.
#pragma once

#include "dual.cuh"

#define DPG_GM1_D   0.4
#define DPG_GAMMA_D 1.4

namespace dpg {

// f[x][eq] for the state s (conservative), D = 2 or 3, NEQ = D+2.
template <int D, class T>
__device__ __forceinline__ void flux_euler(const T* s, T f[D][D + 2])
{
	const T rho = s[0], rho_inv = 1.0 / rho, E = s[D + 1];
	T uvw[D], V2 = 0.0;
#pragma unroll
	for (int a = 0; a < D; ++a) { uvw[a] = rho_inv * s[1 + a]; V2 += uvw[a] * uvw[a]; }
	const T p = DPG_GM1_D * (E - 0.5 * rho * V2);
#pragma unroll
	for (int x = 0; x < D; ++x) {
		f[x][0] = s[1 + x];
#pragma unroll
		for (int a = 0; a < D; ++a) f[x][1 + a] = s[1 + a] * uvw[x] + (a == x ? p : T(0.0));
		f[x][D + 1] = (E + p) * uvw[x];
	}
}

// |x|, min(|a|, |b|) and max(|a|, |b|) on the integer pipe: magnitudes of finite doubles order like their bit
// patterns with the sign cleared (the FP64 pipe is the bound of the face kernels).
__device__ __forceinline__ unsigned long long abs_bits(double x) { return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull; }
__device__ __forceinline__ double abs_i(double x) { return __longlong_as_double((long long)abs_bits(x)); }
__device__ __forceinline__ double min_abs_real(double a, double b)
{
	const unsigned long long ua = abs_bits(a), ub = abs_bits(b);
	return __longlong_as_double((long long)(ua < ub ? ua : ub));
}
__device__ __forceinline__ double max_abs_real(double a, double b)
{
	const unsigned long long ua = abs_bits(a), ub = abs_bits(b);
	return __longlong_as_double((long long)(ua > ub ? ua : ub));
}

// Same formula as the reference; the divisions by rP1 and c are taken once as reciprocals (4 FP64 divisions and
// 2 square roots per node instead of 9 and 2: the GB300 FP64 pipe is the bound of this kernel).  Results differ
// from the reference's operation order by rounding only.
template <int D, class T>
__device__ __forceinline__ void numflux_roe_pike(const T* WL, const T* WR, const double* n, T* nF)
{
	T uL[D], uR[D];
	const T rhoL = WL[0], rhoR = WR[0], EL = WL[D + 1], ER = WR[D + 1];
	const T rhoL_inv = 1.0 / rhoL, rhoR_inv = 1.0 / rhoR;
	T V2L = 0.0, V2R = 0.0, VnL = 0.0, VnR = 0.0;
#pragma unroll
	for (int a = 0; a < D; ++a) {
		uL[a] = WL[1 + a] * rhoL_inv; uR[a] = WR[1 + a] * rhoR_inv;
		V2L += uL[a] * uL[a]; V2R += uR[a] * uR[a];
		VnL += n[a] * uL[a];  VnR += n[a] * uR[a];
	}
	const T pL = DPG_GM1_D * (EL - 0.5 * rhoL * V2L), HL = (EL + pL) * rhoL_inv;
	const T pR = DPG_GM1_D * (ER - 0.5 * rhoR * V2R), HR = (ER + pR) * rhoR_inv;
	const T r = sqrt(rhoR * rhoL_inv), rP1_inv = 1.0 / (r + 1.0), rho = r * rhoL;
	T u[D], Vn = 0.0, V2 = 0.0;
#pragma unroll
	for (int a = 0; a < D; ++a) { u[a] = (r * uR[a] + uL[a]) * rP1_inv; Vn += n[a] * u[a]; V2 += u[a] * u[a]; }
	const T H = (r * HR + HL) * rP1_inv, c2 = DPG_GM1_D * (H - 0.5 * V2), c = sqrt(c2), c_inv = 1.0 / c;
	const T l1 = min_abs_real(VnL - c, Vn - c), l5 = max_abs_real(VnR + c, Vn + c), l234 = abs_i(Vn);
	const T drho = rhoR - rhoL, dE = ER - EL, dp = pR - pL, dVn = VnR - VnL;
	const T lc1 = 0.5 * (l5 + l1) - l234, lc2 = 0.5 * (l5 - l1);
	const T disInter1 = (lc1 * dp * c_inv + lc2 * rho * dVn) * c_inv, disInter2 = lc1 * rho * dVn + lc2 * dp * c_inv;
	const T rhoVnL = rhoL * VnL, rhoVnR = rhoR * VnR, pLR = pL + pR;
	nF[0] = 0.5 * ((rhoVnL + rhoVnR) - (l234 * drho + disInter1));
#pragma unroll
	for (int a = 0; a < D; ++a) {
		const T drhou = rhoR * uR[a] - rhoL * uL[a];
		nF[1 + a] = 0.5 * ((rhoVnL * uL[a] + rhoVnR * uR[a] + n[a] * pLR) - (l234 * drhou + disInter1 * u[a] + disInter2 * n[a]));
	}
	nF[D + 1] = 0.5 * ((VnL * (EL + pL) + VnR * (ER + pR)) - (l234 * dE + disInter1 * H + disInter2 * Vn));
}

template <int D, class T>
__device__ __forceinline__ void numflux_lax_friedrichs(const T* WL, const T* WR, const double* n, T* nF)
{
	T fl[D][D + 2], fr[D][D + 2];
	T V2L = 0.0, V2R = 0.0;
#pragma unroll
	for (int a = 0; a < D; ++a) {
		const T ul = WL[1 + a] / WL[0], ur = WR[1 + a] / WR[0];
		V2L += ul * ul; V2R += ur * ur;
	}
	const T pL = DPG_GM1_D * (WL[D + 1] - 0.5 * WL[0] * V2L), pR = DPG_GM1_D * (WR[D + 1] - 0.5 * WR[0] * V2R);
	const T maxlL = sqrt(V2L) + sqrt(DPG_GAMMA_D * pL / WL[0]), maxlR = sqrt(V2R) + sqrt(DPG_GAMMA_D * pR / WR[0]);
	const T maxV = (maxlL > maxlR ? maxlL : maxlR);
	flux_euler<D>(WL, fl);
	flux_euler<D>(WR, fr);
#pragma unroll
	for (int eq = 0; eq < D + 2; ++eq) {
		T s = 0.0;
#pragma unroll
		for (int x = 0; x < D; ++x) s += n[x] * (fl[x][eq] + fr[x][eq]);
		nF[eq] = 0.5 * (s + maxV * (WL[eq] - WR[eq]));
	}
}

template <int D, class T>
__device__ __forceinline__ T numflux_upwind(const double* b, T wl, T wr, const double* n)
{
	double bn = 0.0;
#pragma unroll
	for (int a = 0; a < D; ++a) bn += b[a] * n[a];
	return (bn > 2.220446049250313e-16 ? bn * wl : bn * wr);
}

} // namespace dpg
