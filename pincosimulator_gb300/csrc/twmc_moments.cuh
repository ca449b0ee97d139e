// twmc_moments.cuh -- FP64 ensemble moment blocks of a batch state (shared by
// the library's reduction launch and the allocation-free entry point).
#pragma once

#include "twmc_common.cuh"
#include "twmc_launch.h"

namespace twmc {

// Neumaier-compensated FP64 accumulator.
struct KSum {
  double s = 0.0, c = 0.0;
  __device__ __forceinline__ void add(double x) {
    const double t = s + x;
    c += (fabs(s) >= fabs(x)) ? ((s - t) + x) : ((x - t) + s);
    s = t;
  }
  __device__ __forceinline__ double value() const { return s + c; }
};

// Ensemble sums over trajectory block b = [b T / B, (b+1) T / B), in
// trajectory order: sum |a|^2, sum |a|^4, sum |a_k|^2. One thread per
// (block, site); deterministic for a given (T, B).
template <typename R>
__device__ __forceinline__ void moments_site(const MomentArgs& a, int64_t p, int b) {
  using T = c2_t<R>;
  const int64_t t0 = (int64_t(b) * a.ntraj) / a.nblocks, t1 = (int64_t(b + 1) * a.ntraj) / a.nblocks;
  // four interleaved partial sums (trajectory tr goes to partial tr % 4),
  // combined in fixed order: deterministic, four loads in flight per thread
  KSum s2[4], s4[4], sk[4];
  const T* st = reinterpret_cast<const T*>(a.state);
  const R* nk = reinterpret_cast<const R*>(a.nk);
  int64_t tr = t0;
  for (; tr + 4 <= t1; tr += 4) {
    T v[4];
    R q[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      v[r] = st[(tr + r) * a.nsites + p];
      q[r] = nk ? nk[(tr + r) * a.nsites + p] : R(0);
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const double ab2 = double(v[r].x) * double(v[r].x) + double(v[r].y) * double(v[r].y);
      s2[r].add(ab2);
      s4[r].add(ab2 * ab2);
      sk[r].add(double(q[r]));
    }
  }
  for (int r = 0; tr < t1; ++tr, ++r) {
    const T v = st[tr * a.nsites + p];
    const double ab2 = double(v.x) * double(v.x) + double(v.y) * double(v.y);
    s2[r].add(ab2);
    s4[r].add(ab2 * ab2);
    sk[r].add(nk ? double(nk[tr * a.nsites + p]) : 0.0);
  }
  KSum f2, f4, fk;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    f2.add(s2[r].s); f2.add(s2[r].c);
    f4.add(s4[r].s); f4.add(s4[r].c);
    fk.add(sk[r].s); fk.add(sk[r].c);
  }
  double* o = a.out + (int64_t(b) * a.nsites + p) * 3;
  o[0] = f2.value();
  o[1] = f4.value();
  o[2] = fk.value();
}

template <typename R>
__global__ void moments_kernel(const MomentArgs a) {
  const int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (p >= a.nsites) return;
  moments_site<R>(a, p, int(blockIdx.y));
}

}  // namespace twmc
