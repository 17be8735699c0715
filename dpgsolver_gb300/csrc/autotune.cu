// Tile shapes of the split-precision residual: get / set and the autotuner (declared in include/dpg_gb300.h).
//
// The tunable block configuration is the number of elements per block of the interpolation and lift kernels (the
// data rows of each 128-row tensor-core tile and, with one block per SM, how many waves the grid takes), the share
// of volume-flux work items given to the FP64 pipe, and the face kernel's block size.  The tuner times whole
// residual evaluations -- the three kernels back to back, as an RK stage runs them -- because the configurations
// trade between kernels (a smaller block shortens the tail wave of both tensor-core kernels but wastes tile rows).
// Search: one coordinate at a time from the wave-rule default, a candidate replacing the running best only when it
// is faster by more than 1 %, so that timing noise between near-equal candidates leaves the default in place.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "dpg_gpu_internal.cuh"

namespace {

struct TuneKey {
	std::string device;
	int sms, d, n_var, n_s, n_vol, n_face, mode, slices;
	bool operator<(const TuneKey& o) const
	{
		return std::tie(device, sms, d, n_var, n_s, n_vol, n_face, mode, slices) <
		       std::tie(o.device, o.sms, o.d, o.n_var, o.n_s, o.n_vol, o.n_face, o.mode, o.slices);
	}
};

struct TuneEntry {
	dpg_tile_config cfg;
	double ms;
};

std::mutex g_mu;
std::map<TuneKey, TuneEntry> g_cache;

#define TK(call)                                                                                            \
	do {                                                                                                    \
		cudaError_t err_ = (call);                                                                          \
		if (err_ != cudaSuccess) {                                                                          \
			fprintf(stderr, "dpg_gb300: %s failed: %s (%s:%d)\n", #call, cudaGetErrorString(err_), __FILE__, \
			        __LINE__);                                                                              \
			return DPG_ERR_CUDA;                                                                            \
		}                                                                                                   \
	} while (0)

struct Events {
	cudaEvent_t a = nullptr, b = nullptr;
	~Events()
	{
		if (a) cudaEventDestroy(a);
		if (b) cudaEventDestroy(b);
	}
};

// Time per residual (ms) of configuration t: one untimed evaluation, then the best of three batches of n_rep.
int time_config(dpg_gpu_ctx* c, const dpg_tile_config& t, int n_rep, unsigned long long* slot, Events& ev, double* ms)
{
	int rc = dpg::split_set_tiles(c, t);
	if (rc) return rc;
	if ((rc = dpg::enqueue_residual_raw(c, slot))) return rc;
	double best = INFINITY;
	for (int b = 0; b < 3; ++b) {
		TK(cudaEventRecord(ev.a, c->stream));
		for (int r = 0; r < n_rep; ++r)
			if ((rc = dpg::enqueue_residual_raw(c, slot))) return rc;
		TK(cudaEventRecord(ev.b, c->stream));
		TK(cudaEventSynchronize(ev.b));
		float f = 0.f;
		TK(cudaEventElapsedTime(&f, ev.a, ev.b));
		best = std::fmin(best, (double)f / n_rep);
	}
	if (dpg::split_error(c)) return DPG_ERR_TIMEOUT;
	*ms = best;
	return DPG_OK;
}

int tune(dpg_gpu_ctx* c, int n_rep, dpg_tile_config* best, double* best_ms)
{
	int n_sm = 1;
	if (cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, c->dev) != cudaSuccess || n_sm < 1) n_sm = 1;
	const int n_vol = c->g.n_vol, NV = c->n_var, eb_max = 128 / NV;
	Events ev;
	TK(cudaEventCreate(&ev.a));
	TK(cudaEventCreate(&ev.b));
	unsigned long long* slot = c->dmax + dpg::kMaxStages;
	TK(cudaMemsetAsync(slot, 0, sizeof *slot, c->stream));

	dpg_tile_config cur{};
	int rc = dpg::split_get_tiles(c, &cur);
	if (rc) return rc;
	cur.elems_per_block = dpg::wave_rule_eb(n_vol, NV, n_sm, 0);   // start from the defaults
	cur.fp64_share_eighths = 2;
	cur.face_block_warps = 8;
	double cur_ms = 0.0;
	if ((rc = time_config(c, cur, n_rep, slot, ev, &cur_ms))) return rc;
	auto consider = [&](dpg_tile_config t) -> int {
		if (t.elems_per_block == cur.elems_per_block && t.fp64_share_eighths == cur.fp64_share_eighths &&
		    t.face_block_warps == cur.face_block_warps)
			return DPG_OK;
		double ms = 0.0;
		const int r = time_config(c, t, n_rep, slot, ev, &ms);
		if (r) return r;
		if (ms < 0.99 * cur_ms) { cur = t; cur_ms = ms; }
		return DPG_OK;
	};
	// 1. elements per block
	std::vector<int> ebs = {dpg::wave_rule_eb(n_vol, NV, n_sm, 1), dpg::wave_rule_eb(n_vol, NV, n_sm, 2), eb_max};
	const dpg_tile_config base = cur;
	for (int eb : ebs) {
		dpg_tile_config t = base;
		t.elems_per_block = eb;
		if ((rc = consider(t))) return rc;
	}
	// 2. FP64 share of the volume-flux items
	const dpg_tile_config base2 = cur;
	for (int s = 0; s <= 4; ++s) {
		dpg_tile_config t = base2;
		t.fp64_share_eighths = s;
		if ((rc = consider(t))) return rc;
	}
	// 3. face kernel block size
	const dpg_tile_config base3 = cur;
	for (int w : {2, 4, 8}) {
		dpg_tile_config t = base3;
		t.face_block_warps = w;
		if ((rc = consider(t))) return rc;
	}
	if ((rc = dpg::split_set_tiles(c, cur))) return rc;
	*best = cur;
	*best_ms = cur_ms;
	return DPG_OK;
}

} // namespace

extern "C" int dpg_gpu_get_tiles(dpg_gpu_ctx* c, dpg_tile_config* out)
{
	if (!c || !out) return DPG_ERR_INVALID;
	return dpg::split_get_tiles(c, out);
}

extern "C" int dpg_gpu_set_tiles(dpg_gpu_ctx* c, const dpg_tile_config* cfg)
{
	if (!c || !cfg) return DPG_ERR_INVALID;
	const int rc = dpg::split_set_tiles(c, *cfg);
	if (rc == DPG_OK) dpg::invalidate_step_graph(c);   // the captured step holds the launch shapes
	return rc;
}

extern "C" int dpg_gpu_autotune(dpg_gpu_ctx* c, int n_rep, int force, dpg_tile_config* best, double* best_ms)
{
	if (!c || n_rep < 1) return DPG_ERR_INVALID;
	if (c->prec_mode == DPG_PREC_FP64 || !c->split) return DPG_ERR_UNSUPPORTED;
	cudaDeviceProp prop;
	TK(cudaGetDeviceProperties(&prop, c->dev));
	const TuneKey key{prop.name, prop.multiProcessorCount, c->d, c->n_var, c->g.n_s, c->g.n_vol, c->fc.n_face,
	                  c->prec_mode, c->prec_mode == DPG_PREC_BF16_SLICED ? c->n_slices : 0};
	TuneEntry e{};
	bool hit = false;
	if (!force) {
		std::lock_guard<std::mutex> lk(g_mu);
		auto it = g_cache.find(key);
		if (it != g_cache.end()) { e = it->second; hit = true; }
	}
	dpg_tile_config prev{};
	int rc = dpg::split_get_tiles(c, &prev);
	if (rc) return rc;
	if (hit) {
		rc = dpg::split_set_tiles(c, e.cfg);
	} else {
		rc = tune(c, n_rep, &e.cfg, &e.ms);
		if (rc == DPG_OK) {
			std::lock_guard<std::mutex> lk(g_mu);
			g_cache[key] = e;
		}
	}
	dpg::invalidate_step_graph(c);
	if (rc) {
		dpg::split_set_tiles(c, prev);   // a failed search puts back the configuration it started from
		return rc;
	}
	if (best) *best = e.cfg;
	if (best_ms) *best_ms = e.ms;
	return DPG_OK;
}
