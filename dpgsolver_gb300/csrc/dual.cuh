// Forward-mode tangent numbers for the linearisation of the residual: a value v and its directional derivative d
// along one direction of the state.  Propagated through the flux formulas of flux.cuh (templated on the scalar
// type), they give the exact Jacobian-vector products of the numerical and physical fluxes -- the products the
// reference forms from its analytic flux Jacobians (df_ds, dnnf_ds: compute_volume_rlhs_T.c:179-220,
// compute_face_rlhs_T.c:163-220; Roe-Pike / Lax-Friedrichs Jacobians in numerical_flux_euler_T.c) -- without
// forming the Jacobian matrices.  Branches (the entropy fix's min/max of |lambda|, the Lax-Friedrichs max wave
// speed) follow the value, as the analytic Jacobians do.
#pragma once

#include <cmath>

namespace dpg {

struct dual {
	double v, d;
	__host__ __device__ dual(double x = 0.0, double dx = 0.0) : v(x), d(dx) {}
};

__device__ __forceinline__ dual operator+(dual a, dual b) { return dual(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ dual operator-(dual a, dual b) { return dual(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ dual operator-(dual a) { return dual(-a.v, -a.d); }
__device__ __forceinline__ dual operator*(dual a, dual b) { return dual(a.v * b.v, a.d * b.v + a.v * b.d); }
__device__ __forceinline__ dual operator/(dual a, dual b)
{
	const double q = a.v / b.v;
	return dual(q, (a.d - q * b.d) / b.v);
}
__device__ __forceinline__ dual operator+(dual a, double b) { return dual(a.v + b, a.d); }
__device__ __forceinline__ dual operator+(double a, dual b) { return dual(a + b.v, b.d); }
__device__ __forceinline__ dual operator-(dual a, double b) { return dual(a.v - b, a.d); }
__device__ __forceinline__ dual operator-(double a, dual b) { return dual(a - b.v, -b.d); }
__device__ __forceinline__ dual operator*(dual a, double b) { return dual(a.v * b, a.d * b); }
__device__ __forceinline__ dual operator*(double a, dual b) { return dual(a * b.v, a * b.d); }
__device__ __forceinline__ dual operator/(dual a, double b) { return dual(a.v / b, a.d / b); }
__device__ __forceinline__ dual operator/(double a, dual b)
{
	const double q = a / b.v;
	return dual(q, -q * b.d / b.v);
}
__device__ __forceinline__ dual& operator+=(dual& a, dual b) { a = a + b; return a; }
__device__ __forceinline__ bool operator>(dual a, dual b) { return a.v > b.v; }

using ::sqrt;   // sqrt(double) stays visible next to the dual overload inside namespace dpg
__device__ __forceinline__ dual sqrt(dual a)
{
	const double s = ::sqrt(a.v);
	return dual(s, s > 0.0 ? a.d / (2.0 * s) : 0.0);
}
using ::pow;
__device__ __forceinline__ dual pow(dual a, double e)
{
	const double p = ::pow(a.v, e);
	return dual(p, a.v != 0.0 ? e * p / a.v * a.d : 0.0);
}
using ::fabs;
__device__ __forceinline__ dual fabs(dual a) { return a.v < 0.0 ? -a : a; }
__device__ __forceinline__ bool operator<(dual a, double b) { return a.v < b; }
__device__ __forceinline__ bool operator>=(dual a, dual b) { return a.v >= b.v; }
__device__ __forceinline__ double value_of(dual a) { return a.v; }
__device__ __forceinline__ double value_of(double a) { return a; }

// |x|, min(|a|, |b|), max(|a|, |b|) with the branches of the FP64 versions (flux.cuh): ties pick b
__device__ __forceinline__ dual abs_i(dual a) { return a.v < 0.0 ? -a : a; }
__device__ __forceinline__ dual min_abs_real(dual a, dual b) { return fabs(a.v) < fabs(b.v) ? abs_i(a) : abs_i(b); }
__device__ __forceinline__ dual max_abs_real(dual a, dual b) { return fabs(a.v) > fabs(b.v) ? abs_i(a) : abs_i(b); }

} // namespace dpg
