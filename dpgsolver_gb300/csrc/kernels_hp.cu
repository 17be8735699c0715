// Mixed orders (hp meshes) in the FP64 form of the DG residual: volumes grouped by order, three launches per
// residual as in kernels_fp64.cu, each launch covering every group.
//
//   k_hp_trace  : per volume, the trace of every local face at the cubature of the face's order p_f (the larger
//                 order of its two volumes, compute_face_reference_order, face_solver.c:123-132), through the
//                 volume basis' operator cv0_vs_fc[p_f][p] (get_operator__cv0_vs_fc_T, compute_face_rlhs_T.c:67-80).
//   k_hp_face   : per face node, the numerical flux with the left normal, scaled by jacobian_det_fc.
//   k_hp_volume : per volume, volume flux, the face fluxes of its local faces gathered in local-face order (right
//                 sides reordered and negated), one lift contraction over [tw1 | -tw0[p_f(0)] | -tw0[p_f(1)] | ...]
//                 (m_inv_ref folded in for affine groups), the mass-matrix inverse, ||rhs||_inf and the SSP-RK3 stage.
// The operands of a volume block are those of its group, the face operators those of (group, p_f).  A block
// processes E_b volumes of one group; the grid is the concatenation of the groups' blocks.  The per-face arrays
// (traces, fluxes, normals, node correspondence) are packed by face at the face-node offsets of the host data
// model (face_geo_off).  With a single order the sums run in the order of the single-group kernels.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "dpg_gpu_internal.cuh"
#include "flux.cuh"

namespace dpg {

constexpr int kHpMaxGroups = DPG_P_MAX;

struct HpGroup {
	int p, n_vol, n_s, n_c, E_b, blk0;     // blk0: first block of the group in every launch
	int affine;                            // every volume affine: Lv, Lf carry m_inv_ref, scale by 1 / detJ
	const int* vols;                       // [n_vol] volume indices
	const double* Cv;                      // [n_c x n_s]
	const double* Lv;                      // [n_s x d n_c]
	const double* Cf[DPG_P_MAX + 1];       // by face order: [n_fl][n_fc(p_f) x n_s]
	const double* Lf[DPG_P_MAX + 1];       // by face order: [n_s x n_fl n_fc(p_f)], negated
	const double* minv;                    // non-affine groups: [n_vol][n_s x n_s] in group order
	const double* met;                     // affine: [n_vol][d d]; else [n_vol][d d][n_c], group order
	const double* jinv;                    // affine: [n_vol]
};

struct HpDev {
	int n_groups, n_fl, n_blocks, nfc_max;
	int n_fc[DPG_P_MAX + 1];               // face cubature nodes by order
	const HpGroup* grp;                    // [n_groups] (device copy)
	const int64_t* dof_off;                // [n_vol + 1]
	const int* vol_face;                   // [n_vol][n_fl]: (face << 1) | side
	const int* face_p;                     // [n_face]
	const int64_t* fnode_off;              // [n_face + 1]
	const int* node_face;                  // [n_fnode]
	const int* nc;                         // [n_fnode] right node of each left node
	const int* nc_inv;                     // [n_fnode]
	const double* nrm;                     // [n_fnode][d]
	const double* jf;                      // [n_fnode]
	int64_t n_fnode;
};

struct HpState {
	HpDev dev{};
	std::vector<HpGroup> host_groups;
	HpGroup* d_groups = nullptr;
	std::vector<void*> allocs;
	double* trace = nullptr;               // [2 n_var n_fnode]
	double* nnf = nullptr;                 // [n_var n_fnode]
	size_t smem_trace = 0, smem_volume = 0;
	int blocks = 0;
};

__device__ __forceinline__ int hp_group_of(const HpDev& h, int blk)
{
	int g = 0;
	while (g + 1 < h.n_groups && h.grp[g + 1].blk0 <= blk) ++g;
	return g;
}

__device__ __forceinline__ void hp_atomic_max_abs(unsigned long long* slot, double v)
{
	atomicMax(slot, (unsigned long long)__double_as_longlong(fabs(v)));
}

template <int NV>
__global__ void __launch_bounds__(256) k_hp_trace(const double* __restrict__ sol, HpDev h, double* __restrict__ trace)
{
	extern __shared__ double sm[];
	const HpGroup& G = h.grp[hp_group_of(h, blockIdx.x)];
	const int n_s = G.n_s, n_fl = h.n_fl, nfm = h.nfc_max;
	const int e0 = (blockIdx.x - G.blk0) * G.E_b;
	const int ne = min(G.E_b, G.n_vol - e0);
	double* sU = sm;   // [ne][NV][n_s]
	for (int i = threadIdx.x; i < ne * NV * n_s; i += blockDim.x) {
		const int e = i / (NV * n_s), r = i - e * NV * n_s;
		sU[i] = sol[h.dof_off[G.vols[e0 + e]] + r];
	}
	__syncthreads();
	const int per_e = n_fl * NV * nfm;
	for (int o = threadIdx.x; o < ne * per_e; o += blockDim.x) {
		const int e = o / per_e, r = o - e * per_e;
		const int lf = r / (NV * nfm), r2 = r - lf * NV * nfm;
		const int var = r2 / nfm, q = r2 - var * nfm;
		const int vf = h.vol_face[(size_t)G.vols[e0 + e] * n_fl + lf];
		const int f = vf >> 1, side = vf & 1;
		const int pf = h.face_p[f], n_fc = h.n_fc[pf];
		if (q >= n_fc) continue;
		const double* op = G.Cf[pf] + (size_t)(lf * n_fc + q) * n_s;
		const double* u = sU + (e * NV + var) * n_s;
		double acc = 0.0;
		for (int s = 0; s < n_s; ++s) acc = fma(__ldg(op + s), u[s], acc);
		trace[2 * NV * h.fnode_off[f] + (size_t)(side * NV + var) * n_fc + q] = acc;
	}
}

template <int D, int NV>
__global__ void __launch_bounds__(128) k_hp_face(const double* __restrict__ trace, HpDev h, double* __restrict__ nnf,
                                                 int num_flux, double bx, double by, double bz)
{
	const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= h.n_fnode) return;
	const int f = h.node_face[t];
	const int64_t off = h.fnode_off[f];
	const int n_fc = (int)(h.fnode_off[f + 1] - off), q = (int)(t - off);
	const int qr = h.nc[t];
	double WL[NV], WR[NV], n[D], nf[NV];
#pragma unroll
	for (int v = 0; v < NV; ++v) {
		WL[v] = trace[2 * NV * off + (size_t)v * n_fc + q];
		WR[v] = trace[2 * NV * off + (size_t)(NV + v) * n_fc + qr];
	}
#pragma unroll
	for (int a = 0; a < D; ++a) n[a] = h.nrm[t * D + a];
	if constexpr (NV == D + 2) {
		if (num_flux == DPG_NUM_FLUX_ROE_PIKE) numflux_roe_pike<D>(WL, WR, n, nf);
		else                                   numflux_lax_friedrichs<D>(WL, WR, n, nf);
	} else {
		const double b[3] = {bx, by, bz};
		nf[0] = numflux_upwind<D>(b, WL[0], WR[0], n);
	}
	const double j = h.jf[t];
#pragma unroll
	for (int v = 0; v < NV; ++v) nnf[NV * off + (size_t)v * n_fc + q] = nf[v] * j;
}

// stage < 0: residual only.  stage 0..2: SSP-RK3 stage update (solp holds the step's initial state).
template <int D, int NV>
__global__ void __launch_bounds__(256) k_hp_volume(double* __restrict__ sol, double* __restrict__ solp,
                                                   double* __restrict__ rhs, const double* __restrict__ nnf, HpDev h,
                                                   const double* __restrict__ dt_ptr, unsigned long long* max_slot,
                                                   int stage, int write_rhs, double bx, double by, double bz)
{
	extern __shared__ double sm[];
	const HpGroup& G = h.grp[hp_group_of(h, blockIdx.x)];
	const int n_s = G.n_s, n_c = G.n_c, n_fl = h.n_fl, E_b = G.E_b;
	const int Kmax = D * n_c + n_fl * h.nfc_max;
	const int e0 = (blockIdx.x - G.blk0) * E_b;
	const int ne = min(E_b, G.n_vol - e0);
	double* sU = sm;                                    // [E_b][NV][n_s]
	double* sS = sU + (size_t)E_b * NV * n_s;           // [E_b][NV][max(n_c, n_s)]
	double* sX = sS + (size_t)E_b * NV * max(n_c, n_s); // [E_b][NV][Kmax]
	for (int i = threadIdx.x; i < ne * NV * n_s; i += blockDim.x) {
		const int e = i / (NV * n_s), r = i - e * NV * n_s;
		sU[i] = sol[h.dof_off[G.vols[e0 + e]] + r];
	}
	__syncthreads();
	// 1. s_vc = cv0_vs_vc sol_coef
	for (int o = threadIdx.x; o < ne * NV * n_c; o += blockDim.x) {
		const int ev = o / n_c, c = o - ev * n_c;
		const double* op = G.Cv + (size_t)c * n_s;
		const double* u = sU + (size_t)ev * n_s;
		double acc = 0.0;
		for (int s = 0; s < n_s; ++s) acc = fma(__ldg(op + s), u[s], acc);
		sS[(size_t)ev * n_c + c] = acc;
	}
	// 2. face fluxes of the local faces, in the volume's own node order (negated on right sides), packed after the
	//    volume part: local face lf at D n_c + sum_{lf' < lf} n_fc(lf')
	for (int o = threadIdx.x; o < ne * n_fl * h.nfc_max; o += blockDim.x) {
		const int e = o / (n_fl * h.nfc_max), r = o - e * n_fl * h.nfc_max;
		const int lf = r / h.nfc_max, q = r - lf * h.nfc_max;
		const int vol = G.vols[e0 + e];
		const int vf = h.vol_face[(size_t)vol * n_fl + lf];
		const int f = vf >> 1, side = vf & 1;
		const int n_fc = h.n_fc[h.face_p[f]];
		if (q >= n_fc) continue;
		int k0 = D * n_c;
		for (int l = 0; l < lf; ++l) k0 += h.n_fc[h.face_p[h.vol_face[(size_t)vol * n_fl + l] >> 1]];
		const int64_t off = h.fnode_off[f];
		const int qs = side ? h.nc_inv[off + q] : q;
		const double sgn = side ? -1.0 : 1.0;
#pragma unroll
		for (int v = 0; v < NV; ++v)
			sX[((size_t)e * NV + v) * Kmax + k0 + q] = sgn * nnf[NV * off + (size_t)v * n_fc + qs];
	}
	__syncthreads();
	// 3. physical flux and reference flux fr[eq][r][c] = sum_x m_{x r} f[x][eq]
	for (int o = threadIdx.x; o < ne * n_c; o += blockDim.x) {
		const int e = o / n_c, c = o - e * n_c;
		double s[NV];
#pragma unroll
		for (int v = 0; v < NV; ++v) s[v] = sS[((size_t)e * NV + v) * n_c + c];
		double m[D][D];
		const size_t ve = (size_t)(e0 + e);
#pragma unroll
		for (int x = 0; x < D; ++x)
#pragma unroll
			for (int r = 0; r < D; ++r)
				m[x][r] = G.affine ? G.met[ve * D * D + x + D * r] : G.met[(ve * D * D + x + D * r) * n_c + c];
		if constexpr (NV == D + 2) {
			double f[D][D + 2];
			flux_euler<D>(s, f);
#pragma unroll
			for (int eq = 0; eq < NV; ++eq)
#pragma unroll
				for (int r = 0; r < D; ++r) {
					double acc = 0.0;
#pragma unroll
					for (int x = 0; x < D; ++x) acc += m[x][r] * f[x][eq];
					sX[((size_t)e * NV + eq) * Kmax + r * n_c + c] = acc;
				}
		} else {
			const double b[3] = {bx, by, bz};
#pragma unroll
			for (int r = 0; r < D; ++r) {
				double acc = 0.0;
#pragma unroll
				for (int x = 0; x < D; ++x) acc += m[x][r] * (b[x] * s[0]);
				sX[(size_t)e * Kmax + r * n_c + c] = acc;
			}
		}
	}
	__syncthreads();
	// 4. lift: R_i = sum_k Lv[i][k] X[k] + sum_lf sum_q Lf[p_f(lf)][i][lf n_fc + q] X[k0(lf) + q], one accumulator
	double* sR = sS;
	for (int o = threadIdx.x; o < ne * NV * n_s; o += blockDim.x) {
		const int ev = o / n_s, i = o - ev * n_s, e = ev / NV;
		const int vol = G.vols[e0 + e];
		const double* x = sX + (size_t)ev * Kmax;
		const double* lv = G.Lv + (size_t)i * D * n_c;
		double acc = 0.0;
		for (int k = 0; k < D * n_c; ++k) acc = fma(__ldg(lv + k), x[k], acc);
		int k0 = D * n_c;
		for (int lf = 0; lf < n_fl; ++lf) {
			const int pf = h.face_p[h.vol_face[(size_t)vol * n_fl + lf] >> 1];
			const int n_fc = h.n_fc[pf];
			const double* lfp = G.Lf[pf] + (size_t)i * n_fl * n_fc + lf * n_fc;
			for (int q = 0; q < n_fc; ++q) acc = fma(__ldg(lfp + q), x[k0 + q], acc);
			k0 += n_fc;
		}
		sR[o] = acc;
	}
	__syncthreads();
	// 5. mass-matrix inverse, RK stage, norm
	const double dt = (stage >= 0 ? *dt_ptr : 0.0);
	double lmax = 0.0;
	for (int o = threadIdx.x; o < ne * NV * n_s; o += blockDim.x) {
		const int ev = o / n_s, i = o - ev * n_s, e = ev / NV;
		double r;
		if (G.affine) {
			r = sR[o] * G.jinv[e0 + e];
		} else {
			const double* mi = G.minv + (size_t)(e0 + e) * n_s * n_s + (size_t)i * n_s;
			const double* x = sR + (size_t)ev * n_s;
			double acc = 0.0;
			for (int j = 0; j < n_s; ++j) acc = fma(mi[j], x[j], acc);
			r = acc;
		}
		lmax = fmax(lmax, fabs(r));
		if (isnan(r)) lmax = r;
		const size_t gi = (size_t)h.dof_off[G.vols[e0 + e]] + (size_t)(ev - e * NV) * n_s + i;
		if (write_rhs) rhs[gi] = r;
		if (stage == 0) { const double s0 = sU[o]; solp[gi] = s0; sol[gi] = s0 + dt * r; }
		else if (stage == 1) sol[gi] = (1.0 / 4.0) * (3.0 * solp[gi] + sU[o] + dt * r);
		else if (stage == 2) sol[gi] = (1.0 / 3.0) * (solp[gi] + 2.0 * sU[o] + 2.0 * dt * r);
	}
	for (int off = 16; off > 0; off >>= 1) {
		const double other = __shfl_xor_sync(0xffffffffu, lmax, off);
		lmax = (isnan(other) || other > lmax) ? other : lmax;
	}
	if ((threadIdx.x & 31) == 0) hp_atomic_max_abs(max_slot, lmax);
}

// ------------------------------------------------------------------------------------------------------------
// host
// ------------------------------------------------------------------------------------------------------------
template <typename T>
static int hp_upload(HpState* s, T** dst, const T* src, size_t n)
{
	void* p = nullptr;
	if (cudaMalloc(&p, (n ? n : 1) * sizeof(T)) != cudaSuccess) return DPG_ERR_CUDA;
	s->allocs.push_back(p);
	if (n && src && cudaMemcpy(p, src, n * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) return DPG_ERR_CUDA;
	*dst = (T*)p;
	return DPG_OK;
}

void hp_free(dpg_gpu_ctx* c)
{
	HpState* s = (HpState*)c->hp;
	if (!s) return;
	for (void* p : s->allocs) cudaFree(p);
	delete s;
	c->hp = nullptr;
}

template <int D, int NV>
static int hp_set_smem(HpState* s)
{
	if (cudaFuncSetAttribute(k_hp_trace<NV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->smem_trace) ||
	    cudaFuncSetAttribute(k_hp_volume<D, NV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s->smem_volume))
		return DPG_ERR_CUDA;
	return DPG_OK;
}

int hp_prepare(dpg_gpu_ctx* c, const struct dpg_sim* sim)
{
	const int d = sim->d, NV = sim->n_var, n_vol = sim->n_vol, n_face = sim->n_face;
	const int n_fl = sim->ops[0].n_fl;
	if (sim->n_ops > kHpMaxGroups || !sim->face_p) return DPG_ERR_UNSUPPORTED;
	HpState* s = new HpState();
	c->hp = s;
	HpDev& h = s->dev;
	h.n_fl = n_fl;
	for (int k = 0; k < sim->n_ops; ++k) h.n_fc[sim->ops[k].p] = sim->ops[k].n_fc;
	h.nfc_max = 0;
	for (int k = 0; k < sim->n_ops; ++k) h.nfc_max = std::max(h.nfc_max, sim->ops[k].n_fc);
	int rc;
	// groups: the volumes of each order present, in volume order
	std::vector<std::vector<int>> members(sim->n_ops);
	for (int v = 0; v < n_vol; ++v) members[sim->vol_ops[v]].push_back(v);
	size_t smem_t = 0, smem_v = 0;
	int blocks = 0;
	for (int k = 0; k < sim->n_ops; ++k) {
		if (members[k].empty()) continue;
		const dpg_element_ops& o = sim->ops[k];
		HpGroup G{};
		G.p = o.p; G.n_vol = (int)members[k].size(); G.n_s = o.n_s; G.n_c = o.n_c;
		const int Kmax = d * o.n_c + n_fl * h.nfc_max;
		const size_t per_v = (size_t)NV * (o.n_s + std::max(o.n_c, o.n_s) + Kmax) * sizeof(double);
		G.E_b = std::max(1, std::min(16, (int)((96 * 1024) / per_v)));
		const size_t per_t = (size_t)NV * o.n_s * sizeof(double);
		smem_t = std::max(smem_t, G.E_b * per_t);
		smem_v = std::max(smem_v, G.E_b * per_v);
		G.blk0 = blocks;
		blocks += (G.n_vol + G.E_b - 1) / G.E_b;
		G.affine = 1;
		for (int v : members[k]) G.affine &= sim->vol_affine[v];
		if ((rc = hp_upload(s, (int**)&G.vols, members[k].data(), members[k].size()))) return rc;
		if ((rc = hp_upload(s, (double**)&G.Cv, o.cv0_vs_vc, (size_t)o.n_c * o.n_s))) return rc;
		// lift operators [tw1 | -tw0[p_f]] row by row, times m_inv_ref for an affine group (the sums of the
		// single-group lift operator)
		auto premul = [&](std::vector<double>& L, int K) {
			if (!G.affine) return;
			std::vector<double> Lm((size_t)o.n_s * K);
			for (int i = 0; i < o.n_s; ++i)
				for (int kk = 0; kk < K; ++kk) {
					double acc = 0.0;
					for (int j = 0; j < o.n_s; ++j) acc += o.m_inv_ref[(size_t)i * o.n_s + j] * L[(size_t)j * K + kk];
					Lm[(size_t)i * K + kk] = acc;
				}
			L.swap(Lm);
		};
		{
			const int K = d * o.n_c;
			std::vector<double> L((size_t)o.n_s * K);
			for (int i = 0; i < o.n_s; ++i)
				for (int r = 0; r < d; ++r)
					for (int cc = 0; cc < o.n_c; ++cc)
						L[(size_t)i * K + r * o.n_c + cc] = o.tw1_vt_vc[((size_t)r * o.n_s + i) * o.n_c + cc];
			premul(L, K);
			if ((rc = hp_upload(s, (double**)&G.Lv, L.data(), L.size()))) return rc;
		}
		for (int pf = o.p; pf <= DPG_P_MAX; ++pf) {
			const double* cf = dpg_face_cv0(&o, pf);
			const double* tw = dpg_face_tw0(&o, pf);
			if (!cf || !tw) continue;
			const int n_fc = h.n_fc[pf];
			const int K = n_fl * n_fc;
			std::vector<double> L((size_t)o.n_s * K);
			for (int i = 0; i < o.n_s; ++i)
				for (int lf = 0; lf < n_fl; ++lf)
					for (int q = 0; q < n_fc; ++q)
						L[(size_t)i * K + lf * n_fc + q] = -tw[((size_t)lf * o.n_s + i) * n_fc + q];
			premul(L, K);
			if ((rc = hp_upload(s, (double**)&G.Cf[pf], cf, (size_t)n_fl * n_fc * o.n_s))) return rc;
			if ((rc = hp_upload(s, (double**)&G.Lf[pf], L.data(), L.size()))) return rc;
		}
		// geometry in group order
		std::vector<double> met, jinv, minv;
		for (int v : members[k]) {
			const double* m = &sim->metrics_vc[(size_t)sim->vol_geo_off[v] * d * d];
			if (G.affine) {
				for (int kk = 0; kk < d * d; ++kk) met.push_back(m[(size_t)o.n_c * kk]);
				jinv.push_back(1.0 / sim->jacobian_det_vc[sim->vol_geo_off[v]]);
			} else {
				met.insert(met.end(), m, m + (size_t)o.n_c * d * d);
				if (sim->vol_minv_off[v + 1] > sim->vol_minv_off[v]) {
					minv.insert(minv.end(), &sim->m_inv[sim->vol_minv_off[v]], &sim->m_inv[sim->vol_minv_off[v]] + (size_t)o.n_s * o.n_s);
				} else {
					const double jd = sim->jacobian_det_vc[sim->vol_geo_off[v]];
					for (int kk = 0; kk < o.n_s * o.n_s; ++kk) minv.push_back(o.m_inv_ref[kk] / jd);
				}
			}
		}
		if ((rc = hp_upload(s, (double**)&G.met, met.data(), met.size()))) return rc;
		if (G.affine) { if ((rc = hp_upload(s, (double**)&G.jinv, jinv.data(), jinv.size()))) return rc; }
		else if ((rc = hp_upload(s, (double**)&G.minv, minv.data(), minv.size()))) return rc;
		s->host_groups.push_back(G);
	}
	h.n_groups = (int)s->host_groups.size();
	h.n_blocks = blocks;
	s->blocks = blocks;
	s->smem_trace = smem_t;
	s->smem_volume = smem_v;
	if ((rc = hp_upload(s, &s->d_groups, s->host_groups.data(), s->host_groups.size()))) return rc;
	h.grp = s->d_groups;
	// volumes and faces
	std::vector<int> vf((size_t)n_vol * n_fl);
	for (int v = 0; v < n_vol; ++v)
		for (int lf = 0; lf < n_fl; ++lf)
			vf[(size_t)v * n_fl + lf] = (sim->vol_face[v * DPG_NFL_MAX + lf] << 1) | sim->vol_face_side[v * DPG_NFL_MAX + lf];
	const int64_t n_fnode = sim->face_geo_off[n_face];
	h.n_fnode = n_fnode;
	std::vector<int> node_face((size_t)n_fnode), ncinv((size_t)n_fnode);
	for (int f = 0; f < n_face; ++f) {
		const int64_t off = sim->face_geo_off[f];
		for (int q = 0; q < sim->face_nfc[f]; ++q) {
			node_face[off + q] = f;
			ncinv[off + sim->nc_fc[off + q]] = q;
		}
	}
	if ((rc = hp_upload(s, (int64_t**)&h.dof_off, sim->vol_dof_off, (size_t)n_vol + 1))) return rc;
	if ((rc = hp_upload(s, (int**)&h.vol_face, vf.data(), vf.size()))) return rc;
	if ((rc = hp_upload(s, (int**)&h.face_p, sim->face_p, (size_t)n_face))) return rc;
	if ((rc = hp_upload(s, (int64_t**)&h.fnode_off, sim->face_geo_off, (size_t)n_face + 1))) return rc;
	if ((rc = hp_upload(s, (int**)&h.node_face, node_face.data(), node_face.size()))) return rc;
	if ((rc = hp_upload(s, (int**)&h.nc, sim->nc_fc, (size_t)n_fnode))) return rc;
	if ((rc = hp_upload(s, (int**)&h.nc_inv, ncinv.data(), ncinv.size()))) return rc;
	if ((rc = hp_upload(s, (double**)&h.nrm, sim->normals_fc, (size_t)n_fnode * d))) return rc;
	if ((rc = hp_upload(s, (double**)&h.jf, sim->jacobian_det_fc, (size_t)n_fnode))) return rc;
	if ((rc = hp_upload(s, &s->trace, (const double*)nullptr, (size_t)2 * NV * n_fnode))) return rc;
	if ((rc = hp_upload(s, &s->nnf, (const double*)nullptr, (size_t)NV * n_fnode))) return rc;
	if (d == 2 && NV == 1) return hp_set_smem<2, 1>(s);
	if (d == 3 && NV == 1) return hp_set_smem<3, 1>(s);
	if (d == 2 && NV == 4) return hp_set_smem<2, 4>(s);
	if (d == 3 && NV == 5) return hp_set_smem<3, 5>(s);
	return DPG_ERR_UNSUPPORTED;
}

template <int D, int NV>
static int hp_launch(dpg_gpu_ctx* c, int which, int stage, bool write_rhs, unsigned long long* max_slot)
{
	HpState* s = (HpState*)c->hp;
	const HpDev& h = s->dev;
	if (which == 0) {
		k_hp_trace<NV><<<s->blocks, 256, s->smem_trace, c->stream>>>(c->sol, h, s->trace);
	} else if (which == 1) {
		const int64_t n = h.n_fnode;
		k_hp_face<D, NV><<<(unsigned)((n + 127) / 128), 128, 0, c->stream>>>(s->trace, h, s->nnf, c->num_flux,
		                                                                 c->b_adv[0], c->b_adv[1], c->b_adv[2]);
	} else {
		k_hp_volume<D, NV><<<s->blocks, 256, s->smem_volume, c->stream>>>(c->sol, c->solp, c->rhs, s->nnf, h, c->ddt,
		                                                                  max_slot, stage, write_rhs ? 1 : 0,
		                                                                  c->b_adv[0], c->b_adv[1], c->b_adv[2]);
	}
	return cudaGetLastError() == cudaSuccess ? DPG_OK : DPG_ERR_CUDA;
}

int hp_launch_part(dpg_gpu_ctx* c, int which, int stage, bool write_rhs, unsigned long long* max_slot)
{
	if (c->d == 2 && c->n_var == 1) return hp_launch<2, 1>(c, which, stage, write_rhs, max_slot);
	if (c->d == 3 && c->n_var == 1) return hp_launch<3, 1>(c, which, stage, write_rhs, max_slot);
	if (c->d == 2 && c->n_var == 4) return hp_launch<2, 4>(c, which, stage, write_rhs, max_slot);
	if (c->d == 3 && c->n_var == 5) return hp_launch<3, 5>(c, which, stage, write_rhs, max_slot);
	return DPG_ERR_UNSUPPORTED;
}

int hp_residual(dpg_gpu_ctx* c, int stage, bool write_rhs, unsigned long long* max_slot)
{
	int rc;
	if ((rc = hp_launch_part(c, 0, stage, write_rhs, max_slot))) return rc;
	if ((rc = hp_launch_part(c, 1, stage, write_rhs, max_slot))) return rc;
	return hp_launch_part(c, 2, stage, write_rhs, max_slot);
}

} // namespace dpg
