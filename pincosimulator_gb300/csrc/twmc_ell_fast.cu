// twmc_ell_fast.cu -- the FP32 fast path of the real-space kernel (Philox
// noise, no F(t), no work / area: the features compiled out), in its own
// translation unit so that it builds in parallel with the general path.
#include "twmc_ell_impl.cuh"

namespace twmc {

bool ell_launch_fast_f32(const StepArgs& a, cudaStream_t s, LaunchInfo* info, std::string* err) {
  using namespace ell_impl;
  return a.hop_kind == 0 ? ell_pick<float, 0, true>(a, s, info, err) : ell_pick<float, 1, true>(a, s, info, err);
}

bool ell_prepare_fast_f32(int variant, StepArgs* a, int* grid, size_t* smem, std::string* err) {
  using namespace ell_impl;
  return a->hop_kind == 0 ? ell_prep_pick<float, 0, true>(variant, a, grid, smem, err)
                          : ell_prep_pick<float, 1, true>(variant, a, grid, smem, err);
}

void ell_launch_dev_fast_f32(int variant, int hop, const StepArgs* dev_args, int grid, size_t smem, cudaStream_t s) {
  using namespace ell_impl;
  if (hop == 0) ell_dev_launch<float, 0, true>(variant, dev_args, grid, smem, s);
  else ell_dev_launch<float, 1, true>(variant, dev_args, grid, smem, s);
}

}  // namespace twmc
