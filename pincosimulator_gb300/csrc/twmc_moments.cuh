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

// Float-float numbers (unevaluated sum h + l, about 48 significant bits) for
// the FP32-state moments: exact products with one FMA (Dekker's product) and
// Knuth's TwoSum run on the FP32 pipe, which GB300 makes 64x wider than its
// FP64 pipe. The _rn intrinsics keep the compiler from contracting them.
struct FF { float h, l; };

__device__ __forceinline__ FF ff_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bp = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp))};
}

__device__ __forceinline__ FF ff_fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ FF ff_abs2(float x, float y) {  // x^2 + y^2
  const float px = __fmul_rn(x, x), ex = __fmaf_rn(x, x, -px);
  const float py = __fmul_rn(y, y), ey = __fmaf_rn(y, y, -py);
  const FF s = ff_two_sum(px, py);
  return ff_fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(ex, ey)));
}

__device__ __forceinline__ FF ff_sqr(FF v) {  // (h + l)^2
  const float p = __fmul_rn(v.h, v.h), e = __fmaf_rn(v.h, v.h, -p);
  return ff_fast_two_sum(p, __fmaf_rn(__fmul_rn(2.0f, v.h), v.l, e));
}

__device__ __forceinline__ void ff_add(FF& acc, FF x) {
  const FF s = ff_two_sum(acc.h, x.h);
  acc = ff_fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(acc.l, x.l)));
}

// FP32 state: the trajectories of a block go in chunks of 32 through
// float-float sums (relative error below 32 x 2^-48 per chunk), each chunk
// then into the FP64 Neumaier sums; values with |a|^2 >= 2^60, whose fourth
// power would overflow FP32, and non-finite ones go to the FP64 sums
// directly. Fixed order: deterministic for a given (T, B).
__device__ __forceinline__ void moments_site_f32(const MomentArgs& a, int64_t p, int b) {
  constexpr int kChunk = 32;
  const int64_t t0 = (int64_t(b) * a.ntraj) / a.nblocks, t1 = (int64_t(b + 1) * a.ntraj) / a.nblocks;
  const float2* st = reinterpret_cast<const float2*>(a.state);
  const float* nk = reinterpret_cast<const float*>(a.nk);
  KSum f2, f4, fk;
  int64_t tr = t0;
  while (tr < t1) {
    const int64_t te = tr + kChunk < t1 ? tr + kChunk : t1;
    FF c2{0.f, 0.f}, c4{0.f, 0.f}, ck{0.f, 0.f};
    auto site = [&](float2 v, float q) {
      const FF a2 = ff_abs2(v.x, v.y);
      if (a2.h < 0x1p60f) {
        ff_add(c2, a2);
        ff_add(c4, ff_sqr(a2));
      } else {
        const double d = double(v.x) * double(v.x) + double(v.y) * double(v.y);
        f2.add(d);
        f4.add(d * d);
      }
      ff_add(ck, FF{q, 0.f});
    };
    for (; tr + 4 <= te; tr += 4) {
      float2 v[4];
      float q[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        v[r] = st[(tr + r) * a.nsites + p];
        q[r] = nk ? nk[(tr + r) * a.nsites + p] : 0.f;
      }
#pragma unroll
      for (int r = 0; r < 4; ++r) site(v[r], q[r]);
    }
    for (; tr < te; ++tr) site(st[tr * a.nsites + p], nk ? nk[tr * a.nsites + p] : 0.f);
    f2.add(double(c2.h)); f2.add(double(c2.l));
    f4.add(double(c4.h)); f4.add(double(c4.l));
    fk.add(double(ck.h)); fk.add(double(ck.l));
  }
  double* o = a.out + (int64_t(b) * a.nsites + p) * 3;
  o[0] = f2.value();
  o[1] = f4.value();
  o[2] = fk.value();
}

// Ensemble sums over trajectory block b = [b T / B, (b+1) T / B), in
// trajectory order: sum |a|^2, sum |a|^4, sum |a_k|^2. One thread per
// (block, site); deterministic for a given (T, B).
template <typename R>
__device__ __forceinline__ void moments_site(const MomentArgs& a, int64_t p, int b) {
  if constexpr (sizeof(R) == 4) {
    moments_site_f32(a, p, b);
    return;
  }
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
