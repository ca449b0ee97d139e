// twmc_ell.cu -- launcher of the real-space (neighbour list / stencil) step kernel:
// general path (F(t), work / area, noise buffer; FP32 and FP64), the 2-CTA
// cluster kernels (general and power-of-two geometry), and the dispatch to the FP32 fast path (twmc_ell_fast.cu).
#include <algorithm>
#include <string>

#include "twmc_ell_impl.cuh"

namespace twmc {

namespace {
using namespace ell_impl;
// 2-CTA cluster variant (square stencil, FP32, more than 8192 sites, no F(t)
// and no work / area): launch configuration shared by both argument forms.
constexpr int kClusterCta = 1024;
constexpr int kClusterVariant = 7;
constexpr int kClusterPow2Variant = 8;      // power-of-two geometry (general features)
constexpr int kClusterPow2FastVariant = 9;  // power-of-two geometry, Philox noise, scalar U and F
constexpr int kFastOffset = 16;  // variant ids of the FP32 fast path (twmc_ell_fast.cu)
constexpr int kRowRunVariant = 10;  // square stencil with row runs (rowrun_kernel)
constexpr int kRowCta = 512;

// Runs without F(t), work / area or a noise buffer take the fast path (FP32).
bool use_fast(int prec, const StepArgs& a) {
  return prec == 0 && a.ft_vals == nullptr && a.work == nullptr && a.noise_mode == 0;
}

bool use_cluster(int prec, const StepArgs& a) {
  return prec == 0 && a.hop_kind == 1 && a.nsites > 8192 && a.nsites <= 16384 && a.ft_vals == nullptr &&
         a.work == nullptr;
}

// Power-of-two geometry for the cluster kernel: N = 2^k, ny a power of two,
// 2 <= ny <= N / 4 (every row inside one quarter of the lattice).
bool cluster_pow2(const StepArgs& a) {
  const int64_t n = a.nsites, ny = a.ny;
  return (n & (n - 1)) == 0 && a.nx * ny == n && ny >= 2 && (ny & (ny - 1)) == 0 && ny <= n / 4;
}

bool cluster_fast(const StepArgs& a) { return a.noise_mode == 0 && a.iU == nullptr && a.iF == nullptr; }

int cluster_variant(const StepArgs& a) {
  if (!cluster_pow2(a)) return kClusterVariant;
  return cluster_fast(a) ? kClusterPow2FastVariant : kClusterPow2Variant;
}

// Square stencil with runs of four sites per thread (rowrun_kernel): the FP32
// fast run with ny a multiple of 4 on 4096 sites, one trajectory per
// 512-thread CTA -- 6 % faster there than the 8-site x 512-thread variant;
// on 1024 sites and fewer the real-space variants with several trajectories
// per CTA measured 2-11 % faster, so those keep them (the kernel itself
// handles any N with ny and N / 2 multiples of 4 up to 4096).
bool rowrun_ok(int prec, const StepArgs& a) {
  const int64_t n = a.nsites;
  return use_fast(prec, a) && a.hop_kind == 1 && a.ny % 4 == 0 && n == 8 * int64_t(kRowCta);
}

bool rowrun_config(const void* fn, StepArgs* a, size_t static_smem, int* grid, size_t* smem_out, std::string* err) {
  const int tpt = int(a->nsites / 8), tpc = kRowCta / tpt;
  a->tpt = tpt;
  a->dbuf = 1;
  const size_t smem = size_t(2) * tpc * size_t(a->nsites) * sizeof(float2);
  int dev = 0, sms = 0, maxsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (smem + static_smem > size_t(maxsm)) { if (err) *err = "row-run kernel: field does not fit"; return false; }
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e != cudaSuccess) { cudaGetLastError(); if (err) *err = std::string("row-run smem: ") + cudaGetErrorString(e); return false; }
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kRowCta, smem);
  if (e != cudaSuccess || per_sm <= 0) { cudaGetLastError(); if (err) *err = "row-run kernel does not fit on an SM"; return false; }
  const int64_t groups = (a->ntraj + tpc - 1) / tpc;
  *grid = int(std::min<int64_t>(groups, int64_t(sms) * per_sm));
  *smem_out = smem;
  return true;
}

bool rowrun_launch(const StepArgs& a0, cudaStream_t s, LaunchInfo* info, std::string* err) {
  StepArgs a = a0;
  int grid = 0;
  size_t smem = 0;
  if (!rowrun_config(reinterpret_cast<const void*>(rowrun_kernel<kRowCta>), &a, 0, &grid, &smem, err)) return false;
  if (info) { info->name = "rowrun_kernel"; info->cta = kRowCta; info->grid = grid; info->smem = smem; info->blocks_per_sm = 1; }
  if (grid <= 0) return true;
  rowrun_kernel<kRowCta><<<grid, kRowCta, smem, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { if (err) *err = std::string("row-run launch: ") + cudaGetErrorString(e); return false; }
  return true;
}

// Lieb lattice with whole cells per thread (lieb_cell_kernel): Nc even,
// Nc / 2 threads per trajectory within one CTA, no work / area.
constexpr int kLiebCta = 256;
bool lieb_cell_ok(const StepArgs& a) {
  const int64_t n = a.nsites;
  return a.hop_kind == 0 && n % 6 == 0 && n / 6 >= 1 && n / 6 <= kLiebCta && a.work == nullptr;
}

template <typename R>
bool lieb_cell_launch(const StepArgs& a0, cudaStream_t s, LaunchInfo* info, std::string* err) {
  StepArgs a = a0;
  const int tpt = int(a.nsites / 6), tpc = kLiebCta / tpt;
  a.tpt = tpt;
  a.dbuf = 1;
  auto fn = lieb_cell_kernel<R, kLiebCta>;
  const size_t smem = size_t(2) * tpc * size_t(a.nsites) * sizeof(c2_t<R>);
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e != cudaSuccess) { cudaGetLastError(); if (err) *err = std::string("lieb smem: ") + cudaGetErrorString(e); return false; }
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kLiebCta, smem);
  if (e != cudaSuccess || per_sm <= 0) { cudaGetLastError(); if (err) *err = "lieb kernel does not fit on an SM"; return false; }
  const int64_t groups = (a.ntraj + tpc - 1) / tpc;
  const int grid = int(std::min<int64_t>(groups, int64_t(sms) * per_sm));
  if (info) { info->name = "lieb_cell_kernel"; info->cta = kLiebCta; info->grid = grid; info->smem = smem; info->blocks_per_sm = per_sm; }
  if (grid <= 0) return true;
  fn<<<grid, kLiebCta, smem, s>>>(a);
  e = cudaGetLastError();
  if (e != cudaSuccess) { if (err) *err = std::string("lieb launch: ") + cudaGetErrorString(e); return false; }
  return true;
}

bool cluster_config(const void* fn, int64_t ntraj, int64_t nsites, size_t static_smem, int* grid, size_t* smem_out,
                    std::string* err) {
  const int64_t half = (nsites + 1) / 2, q = (half + 1) / 2;
  const size_t smem = sizeof(float2) * 4 * size_t(q);  // two buffers of 2q slots
  int dev = 0, sms = 0, maxsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (smem + static_smem > size_t(maxsm)) { if (err) *err = "ell cluster kernel: field does not fit"; return false; }
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e != cudaSuccess) { cudaGetLastError(); if (err) *err = std::string("ell cluster smem: ") + cudaGetErrorString(e); return false; }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(2, 1, 1);
  cfg.blockDim = dim3(kClusterCta, 1, 1);
  cfg.dynamicSmemBytes = smem;
  int ncl = 0;
  e = cudaOccupancyMaxActiveClusters(&ncl, fn, &cfg);
  if (e != cudaSuccess || ncl <= 0) {
    cudaGetLastError();
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kClusterCta, smem);
    if (e != cudaSuccess || per_sm <= 0) { cudaGetLastError(); if (err) *err = "ell cluster kernel does not fit on an SM"; return false; }
    ncl = sms * per_sm / 2;
  }
  *grid = 2 * int(std::min<int64_t>(ntraj, std::max(ncl, 1)));
  *smem_out = smem;
  return true;
}

bool cluster_launch(const StepArgs& a, cudaStream_t s, LaunchInfo* info, std::string* err) {
  const int v = cluster_variant(a);
  void (*fn)(const StepArgs) = v == kClusterPow2FastVariant ? ell_cluster_pow2_kernel<kClusterCta, true>
                               : v == kClusterPow2Variant   ? ell_cluster_pow2_kernel<kClusterCta, false>
                                                            : ell_cluster_kernel<float, kClusterCta>;
  int grid = 0;
  size_t smem = 0;
  if (!cluster_config(reinterpret_cast<const void*>(fn), a.ntraj, a.nsites, 0, &grid, &smem, err)) return false;
  if (info) {
    info->name = v == kClusterVariant ? "ell_cluster_kernel" : "ell_cluster_pow2_kernel";
    info->cta = kClusterCta; info->grid = grid; info->smem = smem; info->blocks_per_sm = 1;
  }
  if (a.ntraj <= 0) return true;
  fn<<<grid, kClusterCta, smem, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { if (err) *err = std::string("ell cluster launch: ") + cudaGetErrorString(e); return false; }
  return true;
}

}  // namespace

bool ell_prepare(int prec, StepArgs* a, int* variant, int* grid, size_t* smem, std::string* err) {
  if (use_cluster(prec, *a)) {
    *variant = cluster_variant(*a);
    void (*fn)(const StepArgs*) = *variant == kClusterPow2FastVariant ? ell_cluster_pow2_kernel_dev<kClusterCta, true>
                                  : *variant == kClusterPow2Variant   ? ell_cluster_pow2_kernel_dev<kClusterCta, false>
                                                                      : ell_cluster_kernel_dev<float, kClusterCta>;
    return cluster_config(reinterpret_cast<const void*>(fn), a->ntraj, a->nsites, sizeof(StepArgs), grid, smem, err);
  }
  if (rowrun_ok(prec, *a)) {
    *variant = kRowRunVariant;
    return rowrun_config(reinterpret_cast<const void*>(rowrun_kernel_dev<kRowCta>), a, sizeof(StepArgs), grid, smem, err);
  }
  *variant = pick_variant(a->nsites);
  if (use_fast(prec, *a)) {
    const int v = *variant;
    *variant = v + kFastOffset;
    return ell_prepare_fast_f32(v, a, grid, smem, err);
  }
  if (a->hop_kind == 0)
    return prec == 0 ? ell_prep_pick<float, 0, false>(*variant, a, grid, smem, err)
                     : ell_prep_pick<double, 0, false>(*variant, a, grid, smem, err);
  return prec == 0 ? ell_prep_pick<float, 1, false>(*variant, a, grid, smem, err)
                   : ell_prep_pick<double, 1, false>(*variant, a, grid, smem, err);
}

bool ell_launch_dev(int prec, int variant, int hop, const StepArgs* dev_args, int grid, size_t smem, cudaStream_t s,
                    std::string* err) {
  if (grid <= 0) return true;
  if (variant == kClusterVariant) {
    ell_cluster_kernel_dev<float, kClusterCta><<<grid, kClusterCta, smem, s>>>(dev_args);
  } else if (variant == kRowRunVariant) {
    rowrun_kernel_dev<kRowCta><<<grid, kRowCta, smem, s>>>(dev_args);
  } else if (variant == kClusterPow2Variant) {
    ell_cluster_pow2_kernel_dev<kClusterCta, false><<<grid, kClusterCta, smem, s>>>(dev_args);
  } else if (variant == kClusterPow2FastVariant) {
    ell_cluster_pow2_kernel_dev<kClusterCta, true><<<grid, kClusterCta, smem, s>>>(dev_args);
  } else if (variant >= kFastOffset) {
    ell_launch_dev_fast_f32(variant - kFastOffset, hop, dev_args, grid, smem, s);
  } else if (hop == 0) {
    if (prec == 0) ell_dev_launch<float, 0, false>(variant, dev_args, grid, smem, s);
    else ell_dev_launch<double, 0, false>(variant, dev_args, grid, smem, s);
  } else {
    if (prec == 0) ell_dev_launch<float, 1, false>(variant, dev_args, grid, smem, s);
    else ell_dev_launch<double, 1, false>(variant, dev_args, grid, smem, s);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) { if (err) *err = std::string("ell launch: ") + cudaGetErrorString(e); return false; }
  return true;
}

bool ell_launch(int prec, const StepArgs& a, cudaStream_t s, LaunchInfo* info, std::string* err) {
  if (use_cluster(prec, a)) return cluster_launch(a, s, info, err);
  if (lieb_cell_ok(a)) return prec == 0 ? lieb_cell_launch<float>(a, s, info, err) : lieb_cell_launch<double>(a, s, info, err);
  if (rowrun_ok(prec, a)) return rowrun_launch(a, s, info, err);
  if (use_fast(prec, a)) return ell_launch_fast_f32(a, s, info, err);
  if (a.hop_kind == 0)
    return prec == 0 ? ell_pick<float, 0, false>(a, s, info, err) : ell_pick<double, 0, false>(a, s, info, err);
  return prec == 0 ? ell_pick<float, 1, false>(a, s, info, err) : ell_pick<double, 1, false>(a, s, info, err);
}

}  // namespace twmc
