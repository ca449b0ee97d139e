// twmc_square_f64.cu -- FP64 instantiations of the square-lattice FFT step kernel
// (parity mode and the FP64 GPU comparator).
#include "twmc_square.cuh"

namespace twmc {
bool square_launch_f64(int bx, int by, const StepArgs& a, int nparams, cudaStream_t s, LaunchInfo* info,
                       std::string* err) {
  return square_dispatch<double>(bx, by, a, nparams, s, info, err);
}
}  // namespace twmc
