// twmc_square.cuh -- launcher of the square-lattice FFT step kernel for the
// compiled shapes (one translation unit per precision).
#pragma once

#include <algorithm>
#include <string>

#include "fft_plans.inc"
#include "twmc_kernels.cuh"
#include "twmc_launch.h"

namespace twmc {

// Threads per CTA: whole trajectories, up to 256 threads, with the two
// exchange buffers and the state slices of all trajectories of the CTA inside
// a ~100 KB shared-memory budget.
template <typename R, class P>
constexpr int cta_for() {
  constexpr int tpt = PlanInfo<P>::TPT;
  constexpr size_t per_traj = (sizeof(R) == 4 ? 3 : 2) * sizeof(c2_t<R>) * size_t(PlanInfo<P>::N) * 17 / 16;
  int tpc = tpt >= 256 ? 1 : 256 / tpt;
  while (tpc > 1 && size_t(tpc) * per_traj > 100 * 1024) tpc /= 2;
  return tpc * tpt;
}

template <typename R, class P, bool FAST, bool SPLIT = false>
bool square_launch_t(const StepArgs& a, int nparams, cudaStream_t s, LaunchInfo* info, std::string* err) {
  constexpr int CTA = cta_for<R, P>();
  using Cfg = SquareCfg<P, CTA, R, true>;  // as square_fft_kernel instantiates it
  (void)nparams;
  StepArgs a2 = a;
  int dev0 = 0, maxsm = 0;
  cudaGetDevice(&dev0);
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev0);
  // the split-step table goes to shared memory where it fits (FP64 4096-site
  // plans read it from global memory)
  a2.kfac_smem = ((SPLIT || !FAST) && a.kfac != nullptr && Cfg::smem_bytes_split() <= size_t(maxsm)) ? 1 : 0;
  const size_t smem = a2.kfac_smem ? Cfg::smem_bytes_split() : Cfg::smem_bytes();
  if (smem > size_t(maxsm)) {
    if (err) *err = "square kernel needs " + std::to_string(smem) + " B of shared memory (device max " +
                    std::to_string(maxsm) + ")";
    return false;
  }
  auto fn = square_fft_kernel<R, P, CTA, FAST, SPLIT>;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e != cudaSuccess) {
    cudaGetLastError();
    if (err) *err = std::string("square kernel smem attribute: ") + cudaGetErrorString(e);
    return false;
  }
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, CTA, smem);
  if (e != cudaSuccess || per_sm <= 0) {
    cudaGetLastError();
    if (err) *err = std::string("square kernel does not fit on an SM (smem ") + std::to_string(smem) + " B)";
    return false;
  }
  const int64_t groups = (a.ntraj + Cfg::TPC - 1) / Cfg::TPC;
  const int grid = int(std::min<int64_t>(groups, int64_t(sms) * per_sm));
  if (info) {
    info->name = FAST ? (SPLIT ? "square_fft_kernel<fast,split>" : "square_fft_kernel<fast>") : "square_fft_kernel";
    info->cta = CTA;
    info->grid = grid;
    info->smem = smem;
    info->blocks_per_sm = per_sm;
  }
  if (grid <= 0) return true;
  fn<<<grid, CTA, smem, s>>>(a2);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    if (err) *err = std::string("square kernel launch: ") + cudaGetErrorString(e);
    return false;
  }
  return true;
}

template <typename R>
bool square_dispatch(int bx, int by, const StepArgs& a, int nparams, cudaStream_t s, LaunchInfo* info,
                     std::string* err) {
  // FP32 runs with Philox noise and scalar U, F take the fast instantiations
  // (Euler, or the split step compiled in); a per-site rsl must have one real
  // part everywhere, except on the plans that keep their twiddles in
  // registers, whose fast kernel reads the whole values
  const bool fast = sizeof(R) == 4 && a.noise_mode == 0 && a.iU == nullptr && a.iF == nullptr;
  const bool split = a.kfac != nullptr;
  const bool rsl_ok = a.rsl == nullptr || a.rsl_re_uniform;
#define TWMC_SHAPE(BX, BY)                                                                                   \
  if (bx == BX && by == BY)                                                                                  \
    return !(fast && (rsl_ok || plan_reg_twiddles<Plan_##BX##_##BY>()))                                     \
               ? square_launch_t<R, Plan_##BX##_##BY, false>(a, nparams, s, info, err)                      \
           : !split ? square_launch_t<R, Plan_##BX##_##BY, sizeof(R) == 4>(a, nparams, s, info, err)        \
                    : square_launch_t<R, Plan_##BX##_##BY, sizeof(R) == 4, sizeof(R) == 4>(a, nparams, s, info, err);
  TWMC_SHAPE(0, 5) TWMC_SHAPE(0, 6) TWMC_SHAPE(0, 7) TWMC_SHAPE(0, 8) TWMC_SHAPE(0, 9) TWMC_SHAPE(0, 10)
  TWMC_SHAPE(0, 11) TWMC_SHAPE(0, 12) TWMC_SHAPE(4, 4) TWMC_SHAPE(5, 5) TWMC_SHAPE(6, 6)
#undef TWMC_SHAPE
  if (err) *err = "square FFT kernel not compiled for this shape";
  return false;
}

}  // namespace twmc
