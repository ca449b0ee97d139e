// twmc_ell.cu -- launcher of the real-space (neighbour list / stencil) step kernel.
#include <algorithm>
#include <string>

#include "twmc_kernels.cuh"
#include "twmc_launch.h"

namespace twmc {

namespace {
template <typename R, int VPT, int CTA, int HOP>
bool ell_launch_t(const StepArgs& a0, cudaStream_t s, LaunchInfo* info, std::string* err) {
  StepArgs a = a0;
  const int64_t half = (a.nsites + 1) / 2;
  const int tpt = int((half + VPT / 2 - 1) / (VPT / 2));
  if (tpt > CTA) { if (err) *err = "ell kernel: lattice too large for this variant"; return false; }
  a.tpt = tpt;
  const int tpc = CTA / tpt;
  using T = c2_t<R>;
  auto fn = ell_kernel<R, VPT, CTA, HOP>;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int maxsm = 0;
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  size_t smem = sizeof(T) * size_t(2) * tpc * size_t(a.nsites);
  a.dbuf = 1;
  if (smem > size_t(maxsm)) { smem /= 2; a.dbuf = 0; }
  if (smem > size_t(maxsm)) { if (err) *err = "ell kernel: trajectory does not fit in shared memory"; return false; }
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e != cudaSuccess) { cudaGetLastError(); if (err) *err = std::string("ell smem: ") + cudaGetErrorString(e); return false; }
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, CTA, smem);
  if (e != cudaSuccess || per_sm <= 0) { cudaGetLastError(); if (err) *err = "ell kernel does not fit on an SM"; return false; }
  const int64_t groups = (a.ntraj + tpc - 1) / tpc;
  const int grid = int(std::min<int64_t>(groups, int64_t(sms) * per_sm));
  if (info) { info->name = "ell_kernel"; info->cta = CTA; info->grid = grid; info->smem = smem; info->blocks_per_sm = per_sm; }
  if (grid <= 0) return true;
  fn<<<grid, CTA, smem, s>>>(a);
  e = cudaGetLastError();
  if (e != cudaSuccess) { if (err) *err = std::string("ell launch: ") + cudaGetErrorString(e); return false; }
  return true;
}

// Variants (sites per thread, threads per CTA); the launcher picks the one
// with the fewest idle site slots (ties: fewer sites per thread).
constexpr int kVariants[][2] = {{2, 256}, {4, 256}, {6, 256}, {8, 256}, {8, 512}, {8, 1024}, {16, 1024}};

template <typename R, int HOP>
bool ell_pick(const StepArgs& a, cudaStream_t s, LaunchInfo* info, std::string* err) {
  const int64_t n = a.nsites, half = (n + 1) / 2;
  int best = -1;
  double best_u = -1.0;
  for (int i = 0; i < int(sizeof(kVariants) / sizeof(kVariants[0])); ++i) {
    const int vpt = kVariants[i][0], cta = kVariants[i][1];
    const int64_t tpt = (half + vpt / 2 - 1) / (vpt / 2);
    if (tpt > cta) continue;
    const int64_t tpc = cta / tpt;
    const double u = double(n * tpc) / double(int64_t(cta) * vpt);
    if (u > best_u + 1e-9) { best_u = u; best = i; }
  }
  switch (best) {
    case 0: return ell_launch_t<R, 2, 256, HOP>(a, s, info, err);
    case 1: return ell_launch_t<R, 4, 256, HOP>(a, s, info, err);
    case 2: return ell_launch_t<R, 6, 256, HOP>(a, s, info, err);
    case 3: return ell_launch_t<R, 8, 256, HOP>(a, s, info, err);
    case 4: return ell_launch_t<R, 8, 512, HOP>(a, s, info, err);
    case 5: return ell_launch_t<R, 8, 1024, HOP>(a, s, info, err);
    case 6: return ell_launch_t<R, 16, 1024, HOP>(a, s, info, err);
    default: break;
  }
  if (err) *err = "ell kernel: more than 16384 sites per trajectory";
  return false;
}
}  // namespace

bool ell_launch(int prec, const StepArgs& a, cudaStream_t s, LaunchInfo* info, std::string* err) {
  if (a.hop_kind == 0) return prec == 0 ? ell_pick<float, 0>(a, s, info, err) : ell_pick<double, 0>(a, s, info, err);
  return prec == 0 ? ell_pick<float, 1>(a, s, info, err) : ell_pick<double, 1>(a, s, info, err);
}

}  // namespace twmc
