// twmc_ell_impl.cuh -- launch configuration of the real-space kernel variants
// (sites per thread x threads per CTA), templated on the fast-path flag; the
// general path and the FP32 fast path are instantiated in separate
// translation units so that the two build in parallel.
#pragma once

#include <algorithm>
#include <string>

#include "twmc_kernels.cuh"
#include "twmc_launch.h"

namespace twmc {
namespace ell_impl {

template <typename R, int VPT, int CTA, int HOP, bool FAST>
bool ell_launch_t(const StepArgs& a0, cudaStream_t s, LaunchInfo* info, std::string* err) {
  StepArgs a = a0;
  const int64_t half = (a.nsites + 1) / 2;
  const int tpt = int((half + VPT / 2 - 1) / (VPT / 2));
  if (tpt > CTA) { if (err) *err = "ell kernel: lattice too large for this variant"; return false; }
  a.tpt = tpt;
  const int tpc = CTA / tpt;
  using T = c2_t<R>;
  auto fn = ell_kernel<R, VPT, CTA, HOP, FAST>;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int maxsm = 0;
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t wbytes = HOP == 0 ? size_t(a.nsites) * 4 * sizeof(R) : 0;  // Lieb weights
  a.dbuf = 1;
  size_t smem = ell_state_bytes(true, tpc, a.nsites, sizeof(T)) + wbytes;
  if (smem > size_t(maxsm)) { a.dbuf = 0; smem = ell_state_bytes(false, tpc, a.nsites, sizeof(T)) + wbytes; }
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

template <typename R, int HOP, bool FAST>
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
    case 0: return ell_launch_t<R, 2, 256, HOP, FAST>(a, s, info, err);
    case 1: return ell_launch_t<R, 4, 256, HOP, FAST>(a, s, info, err);
    case 2: return ell_launch_t<R, 6, 256, HOP, FAST>(a, s, info, err);
    case 3: return ell_launch_t<R, 8, 256, HOP, FAST>(a, s, info, err);
    case 4: return ell_launch_t<R, 8, 512, HOP, FAST>(a, s, info, err);
    case 5: return ell_launch_t<R, 8, 1024, HOP, FAST>(a, s, info, err);
    case 6: return ell_launch_t<R, 16, 1024, HOP, FAST>(a, s, info, err);
    default: break;
  }
  if (err) *err = "ell kernel: more than 16384 sites per trajectory";
  return false;
}
// Configuration of the device-argument variant (ell_kernel_dev): sets a->tpt
// and a->dbuf, returns grid and shared-memory size.
template <typename R, int VPT, int CTA, int HOP, bool FAST>
bool ell_prep_t(StepArgs* a, int* grid, size_t* smem_out, std::string* err) {
  const int64_t half = (a->nsites + 1) / 2;
  const int tpt = int((half + VPT / 2 - 1) / (VPT / 2));
  if (tpt > CTA) { if (err) *err = "ell kernel: lattice too large for this variant"; return false; }
  a->tpt = tpt;
  const int tpc = CTA / tpt;
  using T = c2_t<R>;
  auto fn = ell_kernel_dev<R, VPT, CTA, HOP, FAST>;
  int dev = 0, sms = 0, maxsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const int avail = maxsm - int(sizeof(StepArgs)) - 64;
  const size_t wbytes = HOP == 0 ? size_t(a->nsites) * 4 * sizeof(R) : 0;  // Lieb weights
  a->dbuf = 1;
  size_t smem = ell_state_bytes(true, tpc, a->nsites, sizeof(T)) + wbytes;
  if (smem > size_t(avail)) { a->dbuf = 0; smem = ell_state_bytes(false, tpc, a->nsites, sizeof(T)) + wbytes; }
  if (smem > size_t(avail)) { if (err) *err = "ell kernel: trajectory does not fit in shared memory"; return false; }
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e != cudaSuccess) { cudaGetLastError(); if (err) *err = std::string("ell smem: ") + cudaGetErrorString(e); return false; }
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, CTA, smem);
  if (e != cudaSuccess || per_sm <= 0) { cudaGetLastError(); if (err) *err = "ell kernel does not fit on an SM"; return false; }
  const int64_t groups = (a->ntraj + tpc - 1) / tpc;
  *grid = int(std::min<int64_t>(groups, int64_t(sms) * per_sm));
  *smem_out = smem;
  return true;
}

inline int pick_variant(int64_t n) {
  const int64_t half = (n + 1) / 2;
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
  return best;
}

template <typename R, int HOP, bool FAST>
bool ell_prep_pick(int v, StepArgs* a, int* grid, size_t* smem, std::string* err) {
  switch (v) {
    case 0: return ell_prep_t<R, 2, 256, HOP, FAST>(a, grid, smem, err);
    case 1: return ell_prep_t<R, 4, 256, HOP, FAST>(a, grid, smem, err);
    case 2: return ell_prep_t<R, 6, 256, HOP, FAST>(a, grid, smem, err);
    case 3: return ell_prep_t<R, 8, 256, HOP, FAST>(a, grid, smem, err);
    case 4: return ell_prep_t<R, 8, 512, HOP, FAST>(a, grid, smem, err);
    case 5: return ell_prep_t<R, 8, 1024, HOP, FAST>(a, grid, smem, err);
    case 6: return ell_prep_t<R, 16, 1024, HOP, FAST>(a, grid, smem, err);
    default: if (err) *err = "ell kernel: more than 16384 sites per trajectory"; return false;
  }
}

template <typename R, int HOP, bool FAST>
void ell_dev_launch(int v, const StepArgs* d, int grid, size_t smem, cudaStream_t s) {
  switch (v) {
    case 0: ell_kernel_dev<R, 2, 256, HOP, FAST><<<grid, 256, smem, s>>>(d); break;
    case 1: ell_kernel_dev<R, 4, 256, HOP, FAST><<<grid, 256, smem, s>>>(d); break;
    case 2: ell_kernel_dev<R, 6, 256, HOP, FAST><<<grid, 256, smem, s>>>(d); break;
    case 3: ell_kernel_dev<R, 8, 256, HOP, FAST><<<grid, 256, smem, s>>>(d); break;
    case 4: ell_kernel_dev<R, 8, 512, HOP, FAST><<<grid, 512, smem, s>>>(d); break;
    case 5: ell_kernel_dev<R, 8, 1024, HOP, FAST><<<grid, 1024, smem, s>>>(d); break;
    case 6: ell_kernel_dev<R, 16, 1024, HOP, FAST><<<grid, 1024, smem, s>>>(d); break;
    default: break;
  }
}

}  // namespace ell_impl
}  // namespace twmc
