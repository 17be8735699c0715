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
#include "dpg_simulation.h"

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

// Second-order (viscous) flux of the Navier-Stokes equations, f[x][eq], with the reference's sign (it is added to
// the inviscid flux: compute_Flux_T_navier_stokes subtracts the viscous stresses, flux_navier_stokes_T.c:170-245,
// 1000-1040): constant viscosity mu, Prandtl number Pr, g[x][var] the gradient of the conservative variables.
//   du_i/dx = (d rho u_i/dx - u_i d rho/dx) / rho;  tau_ij = mu (du_j/dx_i + du_i/dx_j) - (2/3) mu div(V) delta_ij;
//   dTs/dx = (dE/dx rho - E drho/dx) / rho^2 - V . dV/dx  (Ts = p / (rho (gamma - 1)));
//   f[x] = -(0, tau[0][x], .., tau[d-1][x], gamma/Pr mu dTs/dx + sum_j u_j tau[x][j]).
template <int D, class T>
__device__ __forceinline__ void flux_viscous(double mu, double Pr, const T* s, const T (*g)[D + 2], T f[D][D + 2])
{
	const T rho_inv = 1.0 / s[0], E = s[D + 1];
	T u[D], du[D][D];
#pragma unroll
	for (int a = 0; a < D; ++a) u[a] = s[1 + a] * rho_inv;
#pragma unroll
	for (int i = 0; i < D; ++i)
#pragma unroll
		for (int x = 0; x < D; ++x) du[i][x] = rho_inv * (g[x][1 + i] - g[x][0] * u[i]);
	T divV = 0.0;
#pragma unroll
	for (int a = 0; a < D; ++a) divV += du[a][a];
	T tau[D][D];
#pragma unroll
	for (int i = 0; i < D; ++i)
#pragma unroll
		for (int j = 0; j < D; ++j)
			tau[i][j] = (i == j) ? mu * 2.0 * (du[i][i] - divV / 3.0) : mu * (du[j][i] + du[i][j]);
#pragma unroll
	for (int x = 0; x < D; ++x) {
		T dV2 = 0.0, w = 0.0;
#pragma unroll
		for (int a = 0; a < D; ++a) { dV2 += u[a] * du[a][x]; w += u[a] * tau[x][a]; }
		const T dTs = rho_inv * rho_inv * (g[x][D + 1] * s[0] - E * g[x][0]) - 0.5 * (2.0 * dV2);
		f[x][0] = T(0.0);
#pragma unroll
		for (int i = 0; i < D; ++i) f[x][1 + i] = -tau[i][x];
		f[x][D + 1] = -(DPG_GAMMA_D / Pr * mu * dTs + w);
	}
}

// Parameters of the boundary states.
struct BcParams {
	double omega, rho_b, E_b;      // BC_NOSLIP_ALL_ROTATING: wall angular velocity, imposed density and total energy
	double ext[5];                 // BC_RIEMANN: external primitive state rho, u, v, w, p
};

// Boundary state s_b from the interior trace s_l at a face node with unit normal n and position x (the reference's
// constructor_Boundary_Value_T_* of boundary_euler_T.c:99-180,494-530 and boundary_navier_stokes_T.c:198-330):
// slip wall (momentum mirrored), Riemann invariants against the external state, no-slip with all variables imposed
// (2 s_wall - s_l, rotating wall velocity omega x r) and no-slip with adiabatic flux (momentum negated).
template <int D, class T>
__device__ __forceinline__ void boundary_state(int bc, const T* sl, const double* n, const double* x, const BcParams& bp, T* sb)
{
	if (bc == DPG_BC_SLIPWALL) {
		T rvn = 0.0;
#pragma unroll
		for (int a = 0; a < D; ++a) rvn += n[a] * sl[1 + a];
		sb[0] = sl[0]; sb[D + 1] = sl[D + 1];
#pragma unroll
		for (int a = 0; a < D; ++a) sb[1 + a] = sl[1 + a] - 2.0 * rvn * n[a];
	} else if (bc == DPG_BC_RIEMANN) {
		T wl[D + 2], w[D + 2];
		double wr[D + 2];
		wl[0] = sl[0];
		T V2l = 0.0;
#pragma unroll
		for (int a = 0; a < D; ++a) { wl[1 + a] = sl[1 + a] / sl[0]; V2l += wl[1 + a] * wl[1 + a]; }
		wl[D + 1] = DPG_GM1_D * (sl[D + 1] - 0.5 * sl[0] * V2l);
		wr[0] = bp.ext[0];
#pragma unroll
		for (int a = 0; a < D; ++a) wr[1 + a] = bp.ext[1 + a];
		wr[D + 1] = bp.ext[4];
		const T cl = sqrt(DPG_GAMMA_D * wl[D + 1] / wl[0]);
		const double cr = ::sqrt(DPG_GAMMA_D * wr[D + 1] / wr[0]);
		T vnl = 0.0;
		double vnr = 0.0;
#pragma unroll
		for (int a = 0; a < D; ++a) { vnl += n[a] * wl[1 + a]; vnr += n[a] * wr[1 + a]; }
		const T Rl = vnl + 2.0 / DPG_GM1_D * cl;
		const double Rr = vnr - 2.0 / DPG_GM1_D * cr;
		const T vn = 0.5 * (Rl + Rr), c = 0.25 * DPG_GM1_D * (Rl - Rr);
		if (value_of(fabs(vn)) >= value_of(fabs(c))) {          // supersonic: all from outside (inflow) or inside
			if (value_of(vn) < 0.0) {
#pragma unroll
				for (int k = 0; k < D + 2; ++k) w[k] = T(wr[k]);
			} else {
#pragma unroll
				for (int k = 0; k < D + 2; ++k) w[k] = wl[k];
			}
		} else if (value_of(vn) < 0.0) {                        // subsonic inflow: entropy, tangential velocity outside
			const double ent = wr[D + 1] / ::pow(wr[0], DPG_GAMMA_D);
			w[0] = pow(1.0 / DPG_GAMMA_D * c * c / ent, 1.0 / DPG_GM1_D);
#pragma unroll
			for (int a = 0; a < D; ++a) w[1 + a] = (wr[1 + a] - vnr * n[a]) + vn * n[a];
			w[D + 1] = 1.0 / DPG_GAMMA_D * c * c * w[0];
		} else {                                                 // subsonic outflow: entropy, tangential velocity inside
			const T ent = wl[D + 1] / pow(wl[0], DPG_GAMMA_D);
			w[0] = pow(1.0 / DPG_GAMMA_D * c * c / ent, 1.0 / DPG_GM1_D);
#pragma unroll
			for (int a = 0; a < D; ++a) w[1 + a] = (wl[1 + a] - vnl * n[a]) + vn * n[a];
			w[D + 1] = 1.0 / DPG_GAMMA_D * c * c * w[0];
		}
		sb[0] = w[0];
		T V2 = 0.0;
#pragma unroll
		for (int a = 0; a < D; ++a) { sb[1 + a] = w[0] * w[1 + a]; V2 += w[1 + a] * w[1 + a]; }
		sb[D + 1] = w[D + 1] / DPG_GM1_D + 0.5 * w[0] * V2;
	} else if (bc == DPG_BC_NOSLIP_ALL_ROTATING) {
		const double r = ::sqrt(x[0] * x[0] + x[1] * x[1]), th = ::atan2(x[1], x[0]), vt = bp.omega * r;
		const double uw[3] = {-::sin(th) * vt, ::cos(th) * vt, 0.0};
		sb[0] = -sl[0] + 2.0 * bp.rho_b;
#pragma unroll
		for (int a = 0; a < D; ++a) sb[1 + a] = -sl[1 + a] + 2.0 * bp.rho_b * uw[a];
		sb[D + 1] = -sl[D + 1] + 2.0 * bp.E_b;
	} else {   // DPG_BC_NOSLIP_ADIABATIC
		sb[0] = sl[0]; sb[D + 1] = sl[D + 1];
#pragma unroll
		for (int a = 0; a < D; ++a) sb[1 + a] = -sl[1 + a];
	}
}

} // namespace dpg
