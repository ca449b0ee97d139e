// twmc_common.cuh -- shared device helpers of the TWMC engine: complex
// arithmetic in FP32/FP64, Philox4x32-10 and the Box-Muller normal pairs.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <type_traits>
#include <utility>

namespace twmc {

template <typename R> struct C2;
template <> struct C2<float> { using type = float2; };
template <> struct C2<double> { using type = double2; };
template <typename R> using c2_t = typename C2<R>::type;

template <typename T> __device__ __forceinline__ T cmake(decltype(T::x) x, decltype(T::x) y) { T r; r.x = x; r.y = y; return r; }
template <typename T> __device__ __forceinline__ T cadd(T a, T b) { return cmake<T>(a.x + b.x, a.y + b.y); }
template <typename T> __device__ __forceinline__ T csub(T a, T b) { return cmake<T>(a.x - b.x, a.y - b.y); }
// FP32 complex add/sub as one packed FP32x2 instruction (sm_100+); same
// round-to-nearest results as the two scalar operations.
template <> __device__ __forceinline__ float2 cadd<float2>(float2 a, float2 b) { return __fadd2_rn(a, b); }
template <> __device__ __forceinline__ float2 csub<float2>(float2 a, float2 b) {
  return __fadd2_rn(a, make_float2(-b.x, -b.y));
}
template <typename T> __device__ __forceinline__ T cmul(T a, T b) { return cmake<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
// a * conj(b)
template <typename T> __device__ __forceinline__ T cmulc(T a, T b) { return cmake<T>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y); }
// acc + y * conj(w) as four multiply-adds (one rounding per component step)
template <typename T> __device__ __forceinline__ T cmlac(T acc, T y, T w) {
  return cmake<T>(fma(y.x, w.x, fma(y.y, w.y, acc.x)), fma(y.y, w.x, fma(-y.x, w.y, acc.y)));
}
// 2 a - s: the difference a - u of a butterfly whose sum s = a + u is known
template <typename T> __device__ __forceinline__ T ctwice_minus(T a, T s) {
  using R = decltype(T::x);
  return cmake<T>(fma(R(2), a.x, -s.x), fma(R(2), a.y, -s.y));
}
// -i * a and +i * a
template <typename T> __device__ __forceinline__ T cmul_mi(T a) { return cmake<T>(a.y, -a.x); }
template <typename T> __device__ __forceinline__ T cmul_pi(T a) { return cmake<T>(-a.y, a.x); }

// Shared-memory access through 32-bit shared-window addresses (the
// real-space kernels compute their neighbour indices at run time; keeping the
// address arithmetic in 32 bits avoids 64-bit integer work per access).
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ float2 lds_c(uint32_t a, float2) {
  float2 v;
  asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a) : "memory");
  return v;
}
__device__ __forceinline__ double2 lds_c(uint32_t a, double2) {
  double2 v;
  asm volatile("ld.shared.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "r"(a) : "memory");
  return v;
}
// Four consecutive FP32 complex values (32 bytes, 16-byte aligned) to / from
// shared memory.
__device__ __forceinline__ void lds_run4(uint32_t a, float2* v) {
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v[0].x), "=f"(v[0].y), "=f"(v[1].x), "=f"(v[1].y) : "r"(a) : "memory");
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v[2].x), "=f"(v[2].y), "=f"(v[3].x), "=f"(v[3].y) : "r"(a + 16u) : "memory");
}
__device__ __forceinline__ void sts_run4(uint32_t a, const float2* v) {
  asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(a), "f"(v[0].x), "f"(v[0].y), "f"(v[1].x), "f"(v[1].y)
               : "memory");
  asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(a + 16u), "f"(v[2].x), "f"(v[2].y), "f"(v[3].x),
               "f"(v[3].y) : "memory");
}
// Four consecutive reals from shared memory (16-byte aligned for FP32).
__device__ __forceinline__ void lds_r4(uint32_t a, float* w) {
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(w[0]), "=f"(w[1]), "=f"(w[2]), "=f"(w[3]) : "r"(a) : "memory");
}
__device__ __forceinline__ void lds_r4(uint32_t a, double* w) {
  asm volatile("ld.shared.v2.f64 {%0, %1}, [%2];" : "=d"(w[0]), "=d"(w[1]) : "r"(a) : "memory");
  asm volatile("ld.shared.v2.f64 {%0, %1}, [%2];" : "=d"(w[2]), "=d"(w[3]) : "r"(a + 16u) : "memory");
}
__device__ __forceinline__ void sts_c(uint32_t a, float2 v) {
  asm volatile("st.shared.v2.f32 [%0], {%1, %2};" ::"r"(a), "f"(v.x), "f"(v.y) : "memory");
}
__device__ __forceinline__ void sts_c(uint32_t a, double2 v) {
  asm volatile("st.shared.v2.f64 [%0], {%1, %2};" ::"r"(a), "d"(v.x), "d"(v.y) : "memory");
}
// The same address in the shared memory of cluster CTA `rank`, and a load
// through it (distributed shared memory).
__device__ __forceinline__ uint32_t cluster_addr(uint32_t a, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(rank));
  return r;
}
__device__ __forceinline__ float2 ldc_c(uint32_t a, float2) {
  float2 v;
  asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(a) : "memory");
  return v;
}

// Compile-time loop: f(std::integral_constant<int, I>) for I = 0..N-1.
template <class F, int... Is>
__device__ __forceinline__ void static_for_impl(F&& f, std::integer_sequence<int, Is...>) {
  (f(std::integral_constant<int, Is>{}), ...);
}
template <int N, class F>
__device__ __forceinline__ void static_for(F&& f) {
  static_for_impl(f, std::make_integer_sequence<int, N>{});
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11): 10 rounds of two 32x32->64-bit
// multiplies with Weyl-sequence key bumps. Counter (c0,c1,c2,c3), key (k0,k1).
// ---------------------------------------------------------------------------
struct u32x4 { uint32_t x, y, z, w; };

__host__ __device__ __forceinline__ u32x4 philox4x32_10(u32x4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
    const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
    const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
#else
    const uint64_t p0 = uint64_t(0xD2511F53u) * c.x, p1 = uint64_t(0xCD9E8D57u) * c.z;
    const uint32_t lo0 = uint32_t(p0), hi0 = uint32_t(p0 >> 32);
    const uint32_t lo1 = uint32_t(p1), hi1 = uint32_t(p1 >> 32);
#endif
    c = u32x4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

// Noise streams (counter word 2).
enum : uint32_t { kStreamWiener = 0, kStreamInit = 1, kStreamU = 2, kStreamOmega = 3, kStreamF = 4 };

// Wiener increments use a fixed key, kWienerKey0/1 (hex digits of pi), and
// carry the trajectory in the counter: (site pair, step, id, seed). The key
// schedule is then a compile-time constant that folds into the round's
// XORs instead of two adds per round on per-thread keys. The other streams
// keep the key (seed, id) and the counter (site pair, 0, stream, 0); with
// these constants the two families cannot share an input block.
constexpr uint32_t kWienerKey0 = 0x243F6A88u, kWienerKey1 = 0x85A308D3u;

__host__ __device__ __forceinline__ u32x4 wiener_words(uint32_t pair, uint32_t step, uint32_t seed, uint32_t id) {
  return philox4x32_10(u32x4{pair, step, id, seed}, kWienerKey0, kWienerKey1);
}

// Box-Muller, FP32, scaled by s: s (r cos th, r sin th) with r = sqrt(-2 ln u1),
// u1 = fma(float(a), 2^-32, 2^-33) in (0, 1], th = 2 pi u2 - pi, u2 the same
// map of b. The radius is computed as sqrt(kn log2 u1) with kn = -2 ln(2) s^2
// (hardware log2 and square root), so a scale costs nothing; th is one FMA
// of float(b).
__device__ __forceinline__ float lg2_approx(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float sqrt_approx(float x) {
  float y;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
constexpr float kNegTwoLn2 = -1.38629436111989061883f;  // -2 ln 2: kn of the unscaled normals
__device__ __forceinline__ float2 scaled_normal_pair(uint32_t a, uint32_t b, float kn) {
  const float u1 = __fmaf_rn(__uint2float_rn(a), 0x1p-32f, 0x1p-33f);
  // 2 pi (float(b) 2^-32 + 2^-33) - pi
  const float th = __fmaf_rn(__uint2float_rn(b), 1.46291807926715968e-9f, -3.14159265285833420f);
  const float r = sqrt_approx(fmaxf(kn * lg2_approx(u1), 0.0f));
  float sn, cs;
  __sincosf(th, &sn, &cs);
  return make_float2(r * cs, r * sn);
}
__device__ __forceinline__ float2 normal_pair(uint32_t a, uint32_t b, float) {
  return scaled_normal_pair(a, b, kNegTwoLn2);
}

// Box-Muller, FP64: u = (w + 1/2) 2^-32.
__device__ __forceinline__ double2 normal_pair(uint32_t a, uint32_t b, double) {
  const double u1 = (double(a) + 0.5) * 0x1p-32;
  const double u2 = (double(b) + 0.5) * 0x1p-32;
  const double r = sqrt(-2.0 * log(u1));
  const double th = 6.283185307179586476925 * u2 - 3.141592653589793238463;
  double s, c;
  sincos(th, &s, &c);
  return make_double2(r * c, r * s);
}

// Site pairing on Philox calls: half = ceil(n/2); site p < half uses words
// (0,1) of call p, site p >= half words (2,3) of call p - half.
__host__ __device__ __forceinline__ uint32_t site_ctr(int64_t p, int64_t n, int* hi) {
  const int64_t half = (n + 1) / 2;
  *hi = p >= half;
  return uint32_t(p >= half ? p - half : p);
}

}  // namespace twmc
