// Split-precision contractions (placeholder until the tcgen05 path lands).
#include "dpg_gpu_internal.cuh"

namespace dpg {
int  split_prepare(dpg_gpu_ctx*) { return DPG_ERR_UNSUPPORTED; }
void split_free(dpg_gpu_ctx*) {}
int  split_launch_trace(dpg_gpu_ctx*) { return DPG_ERR_UNSUPPORTED; }
int  split_launch_volume(dpg_gpu_ctx*, int, bool, unsigned long long*) { return DPG_ERR_UNSUPPORTED; }
}
