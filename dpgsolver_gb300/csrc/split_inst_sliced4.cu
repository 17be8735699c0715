// Split-precision kernels instantiated for BF16 slices, S = 4 (one translation unit per mode: compiled in parallel).
#include "split_kernels.cuh"

namespace dpg {
namespace split {

#define DPG_CASE(D_, NV_, KS_, KF_, KC_)                                                                             \
	if (d == D_ && nv == NV_ && ks == KS_ && kf == KF_ && kc == KC_) return table_of<D_, NV_, KS_, KF_, KC_, 1, 4, true>();

KernelTable kernels_sliced4(int d, int nv, int ks, int kf, int kc)
{
	DPG_SPLIT_CASES(DPG_CASE)
	return KernelTable{nullptr, nullptr, nullptr, nullptr};
}

} // namespace split
} // namespace dpg
