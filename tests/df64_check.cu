// GPU check of the double-float layer of the split path (df64.cuh, flux_df.cuh) against FP64 on seeded random
// inputs: the conversion to FP64 (bit-exact), reciprocal, square root, product and sums (relative bounds, operands
// within 2^+-40), and the Roe-Pike / Lax-Friedrichs numerical fluxes against the FP64 formulas of flux.cuh (bounded
// relative to the flux scale of each node).  Built and run by tests/test_gpu_df64.py; prints one line per check and
// exits 1 if any bound is missed.
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <vector>

#include "df64.cuh"
#include "flux.cuh"
#include "flux_df.cuh"

using dpg::df::df64;

namespace {

struct Rng {   // 64-bit LCG (Knuth's MMIX constants), top 53 bits as a uniform double in [0, 1)
	uint64_t s;
	double u() { s = s * 6364136223846793005ull + 1442695040888963407ull; return (double)(s >> 11) * (1.0 / 9007199254740992.0); }
	double in(double a, double b) { return a + (b - a) * u(); }
};

__device__ df64 load(const float2* p, int i) { return dpg::df::from2(p[i]); }

// one value per thread: out[6i + k] for the six primitive checks of pair (x_i, y_i)
__global__ void k_prims(int n, const float2* x, const float2* y, double* out)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	using namespace dpg::df;
	const df64 a = load(x, i), b = load(y, i);
	out[6 * i + 0] = to_double(a);
	out[6 * i + 1] = to_double(rcp(b));
	out[6 * i + 2] = to_double(sqrt(absd(b)));
	out[6 * i + 3] = to_double(mul(a, b));
	out[6 * i + 4] = to_double(add(a, b));
	out[6 * i + 5] = to_double(add_s(absd(a), absd(b)));
}

// numerical flux of node i in FP64 (from the doubles) and in double-float (from their FP32-pair splits)
template <int D>
__global__ void k_flux(int n, int roe, const double* WL, const double* WR, const double* nrm, double* f64, double* fdf)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	constexpr int NV = D + 2;
	double wl[NV], wr[NV], nn[D], nf[NV];
	df64 dl[NV], dr[NV], dn[D], df[NV];
	for (int v = 0; v < NV; ++v) {
		wl[v] = WL[NV * i + v]; wr[v] = WR[NV * i + v];
		dl[v] = dpg::df::from2(dpg::df::split_double(wl[v])); dr[v] = dpg::df::from2(dpg::df::split_double(wr[v]));
	}
	for (int a = 0; a < D; ++a) { nn[a] = nrm[D * i + a]; dn[a] = dpg::df::from2(dpg::df::split_double(nn[a])); }
	if (roe) { dpg::numflux_roe_pike<D>(wl, wr, nn, nf); dpg::df::numflux_roe_pike<D>(dl, dr, dn, df); }
	else { dpg::numflux_lax_friedrichs<D>(wl, wr, nn, nf); dpg::df::numflux_lax_friedrichs<D>(dl, dr, dn, df); }
	for (int v = 0; v < NV; ++v) { f64[NV * i + v] = nf[v]; fdf[NV * i + v] = dpg::df::to_double(df[v]); }
}

float2 split(double v) { return dpg::df::split_double(v); }

int report(const char* name, double err, double bound)
{
	const bool ok = err <= bound;
	std::printf("check %-28s max_err %.3e bound %.1e %s\n", name, err, bound, ok ? "ok" : "FAIL");
	return ok ? 0 : 1;
}

template <int D>
int flux_checks(Rng& r, int n, int roe)
{
	constexpr int NV = D + 2;
	std::vector<double> wl(NV * n), wr(NV * n), nrm(D * n);
	auto state = [&](double* w) {   // rho in [0.5, 2], |u| <= 0.6, p in [0.5, 2]
		const double rho = r.in(0.5, 2.0), p = r.in(0.5, 2.0);
		double V2 = 0.0;
		w[0] = rho;
		for (int a = 0; a < D; ++a) { const double u = r.in(-0.6, 0.6); w[1 + a] = rho * u; V2 += u * u; }
		w[D + 1] = p / 0.4 + 0.5 * rho * V2;
	};
	for (int i = 0; i < n; ++i) {
		state(&wl[NV * i]);
		if (i % 4 == 0) for (int v = 0; v < NV; ++v) wr[NV * i + v] = wl[NV * i + v];   // equal states
		else state(&wr[NV * i]);
		double s = 0.0;
		for (int a = 0; a < D; ++a) { nrm[D * i + a] = r.in(-1.0, 1.0); s += nrm[D * i + a] * nrm[D * i + a]; }
		s = std::sqrt(s);
		for (int a = 0; a < D; ++a) nrm[D * i + a] /= s;
	}
	double *dWL, *dWR, *dN, *dF, *dG;
	cudaMalloc(&dWL, sizeof(double) * NV * n); cudaMalloc(&dWR, sizeof(double) * NV * n);
	cudaMalloc(&dN, sizeof(double) * D * n); cudaMalloc(&dF, sizeof(double) * NV * n); cudaMalloc(&dG, sizeof(double) * NV * n);
	cudaMemcpy(dWL, wl.data(), sizeof(double) * NV * n, cudaMemcpyHostToDevice);
	cudaMemcpy(dWR, wr.data(), sizeof(double) * NV * n, cudaMemcpyHostToDevice);
	cudaMemcpy(dN, nrm.data(), sizeof(double) * D * n, cudaMemcpyHostToDevice);
	k_flux<D><<<(n + 127) / 128, 128>>>(n, roe, dWL, dWR, dN, dF, dG);
	std::vector<double> f(NV * n), g(NV * n);
	const cudaError_t e = cudaDeviceSynchronize();
	cudaMemcpy(f.data(), dF, sizeof(double) * NV * n, cudaMemcpyDeviceToHost);
	cudaMemcpy(g.data(), dG, sizeof(double) * NV * n, cudaMemcpyDeviceToHost);
	cudaFree(dWL); cudaFree(dWR); cudaFree(dN); cudaFree(dF); cudaFree(dG);
	if (e != cudaSuccess) { std::printf("cuda error %s\n", cudaGetErrorString(e)); return 1; }
	double err = 0.0;
	for (int i = 0; i < n; ++i) {
		double scale = 0.0;   // the flux scale of the node: its largest component
		for (int v = 0; v < NV; ++v) scale = std::fmax(scale, std::fabs(f[NV * i + v]));
		for (int v = 0; v < NV; ++v) err = std::fmax(err, std::fabs(g[NV * i + v] - f[NV * i + v]) / scale);
	}
	char name[64];
	std::snprintf(name, sizeof name, "%s flux %dD", roe ? "Roe-Pike" : "Lax-Friedrichs", D);
	return report(name, err, 3e-13);   // ~2^-41.6 of the flux scale (FP32 alone: ~1e-6)
}

} // namespace

int main()
{
	Rng r{12345};
	const int n = 1 << 18;
	std::vector<double> xs(n), ys(n);
	std::vector<float2> xh(n), yh(n);
	for (int i = 0; i < n; ++i) {
		// magnitudes 2^-40 .. 2^40, both signs (products stay where the trailing FP32 word is normal: the
		// double-float format keeps its 48 bits for |x| >= 2^-102); every fourth pair of equal exponents
		const int ex = (int)(r.u() * 80) - 40, ey = (i % 4 == 0) ? ex : (int)(r.u() * 80) - 40;
		xs[i] = std::ldexp(r.in(1.0, 2.0), ex) * (r.u() < 0.5 ? -1.0 : 1.0);
		ys[i] = std::ldexp(r.in(1.0, 2.0), ey) * (r.u() < 0.5 ? -1.0 : 1.0);
		xh[i] = split(xs[i]); yh[i] = split(ys[i]);
	}
	float2 *dx, *dy; double* dout;
	cudaMalloc(&dx, sizeof(float2) * n); cudaMalloc(&dy, sizeof(float2) * n); cudaMalloc(&dout, sizeof(double) * 6 * n);
	cudaMemcpy(dx, xh.data(), sizeof(float2) * n, cudaMemcpyHostToDevice);
	cudaMemcpy(dy, yh.data(), sizeof(float2) * n, cudaMemcpyHostToDevice);
	k_prims<<<(n + 255) / 256, 256>>>(n, dx, dy, dout);
	std::vector<double> out(6 * (size_t)n);
	const cudaError_t e = cudaDeviceSynchronize();
	cudaMemcpy(out.data(), dout, sizeof(double) * 6 * n, cudaMemcpyDeviceToHost);
	cudaFree(dx); cudaFree(dy); cudaFree(dout);
	if (e != cudaSuccess) { std::printf("cuda error %s\n", cudaGetErrorString(e)); return 1; }
	long mism = 0;
	double e_rcp = 0, e_sqrt = 0, e_mul = 0, e_add = 0, e_adds = 0;
	for (int i = 0; i < n; ++i) {
		const double a = (double)xh[i].x + (double)xh[i].y, b = (double)yh[i].x + (double)yh[i].y;   // exact
		if (out[6 * i] != a) ++mism;
		e_rcp = std::fmax(e_rcp, std::fabs(out[6 * i + 1] * b - 1.0));
		const double sb = std::sqrt(std::fabs(b));
		e_sqrt = std::fmax(e_sqrt, std::fabs(out[6 * i + 2] - sb) / sb);
		e_mul = std::fmax(e_mul, std::fabs(out[6 * i + 3] - a * b) / std::fabs(a * b));
		// sums: reference a + b in FP64 (error 2^-53 of the result), bound relative to the larger operand
		const double big = std::fmax(std::fabs(a), std::fabs(b));
		e_add = std::fmax(e_add, std::fabs(out[6 * i + 4] - (a + b)) / big);
		e_adds = std::fmax(e_adds, std::fabs(out[6 * i + 5] - (std::fabs(a) + std::fabs(b))) / big);
	}
	int bad = 0;
	bad += report("to_double (mismatches)", (double)mism, 0.0);
	bad += report("rcp (relative)", e_rcp, std::ldexp(1.0, -44));
	bad += report("sqrt (relative)", e_sqrt, std::ldexp(1.0, -44));
	bad += report("mul (relative)", e_mul, std::ldexp(1.0, -44));
	bad += report("add (rel. to larger operand)", e_add, std::ldexp(1.0, -45));
	bad += report("add_s (rel. to larger operand)", e_adds, std::ldexp(1.0, -45));
	bad += flux_checks<3>(r, 1 << 16, 1);
	bad += flux_checks<3>(r, 1 << 16, 0);
	bad += flux_checks<2>(r, 1 << 16, 1);
	bad += flux_checks<2>(r, 1 << 16, 0);
	std::printf("%s\n", bad ? "FAILED" : "all checks passed");
	return bad ? 1 : 0;
}
