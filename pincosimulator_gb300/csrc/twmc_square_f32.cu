// twmc_square_f32.cu -- FP32 instantiations of the square-lattice FFT step kernel.
#include "twmc_square.cuh"

namespace twmc {
bool square_launch_f32(int bx, int by, const StepArgs& a, int nparams, cudaStream_t s, LaunchInfo* info,
                       std::string* err) {
  return square_dispatch<float>(bx, by, a, nparams, s, info, err);
}
}  // namespace twmc
