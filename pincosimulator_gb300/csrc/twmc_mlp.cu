// twmc_mlp.cu -- the learned warm start: a small MLP with BF16 weights and
// FP32 accumulation on the tensor cores (forward, backward, Adam), mapping a
// parameter point (F, detuning, U, J, gamma) to its steady-state k-mode mean
// field and density, plus the transforms between engine fields and MLP rows.
//
// No counterpart in the reference (it has no learned component). Layout:
//   parameters, one contiguous FP32 master array: for each layer l,
//     W_l [width[l+1]][width[l]] row-major, then b_l [width[l+1]];
//   a BF16 copy of the same array feeds the GEMMs; gradients, Adam moments
//   use the same offsets.
//   Activations are BF16 (the GEMM operands), pre-activations FP32.
// Every GEMM is one templated kernel: a 64 x 64 output tile per 128-thread
// CTA, operands staged through shared memory with arbitrary strides (so the
// transposed products of the backward pass need no transposed copies), and
// mma.sync m16n8k16 BF16 x BF16 -> FP32 per warp on a 32 x 32 sub-tile.
// The epilogue is fused: bias + GELU (hidden forward, keeping the FP32
// pre-activation), bias (output layer), GELU' (backward), or plain store
// (weight gradients).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "twmc.h"

namespace {

using bf16 = __nv_bfloat16;

constexpr int kBM = 64, kBN = 64, kBK = 32, kPadK = kBK + 8;

enum Epi { EPI_BIAS_GELU = 0, EPI_BIAS = 1, EPI_GELU_BWD = 2, EPI_STORE = 3 };

// C[m][n] = sum_k A(m, k) B(n, k), A(m, k) = A[m sam + k sak], B(n, k) = B[n sbn + k sbk].
struct GemmArgs {
  const bf16* A;
  int64_t sam, sak;
  const bf16* B;
  int64_t sbn, sbk;
  int M, N, K;
  const float* bias;  // [N]            (EPI_BIAS_GELU, EPI_BIAS)
  const float* z;     // [M][ldo] FP32  (EPI_GELU_BWD)
  float* outf;        // [M][ldo] FP32  (EPI_BIAS_GELU: z, EPI_BIAS, EPI_STORE)
  bf16* outh;         // [M][ldo] BF16  (EPI_BIAS_GELU: gelu(z), EPI_GELU_BWD)
  int64_t ldo;
};

__device__ __forceinline__ float gelu_f(float z) { return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
  const float cdf = 0.5f * (1.0f + erff(z * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * expf(-0.5f * z * z);
  return cdf + z * pdf;
}

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Stages a rows x kBK tile (row r0.., k k0..) into s[row][k], zero outside.
// Consecutive threads walk the unit-stride dimension of the source.
__device__ __forceinline__ void stage_tile(bf16 (*s)[kPadK], const bf16* src, int64_t sr, int64_t sk, int nrows,
                                           int nk, int r0, int k0) {
  const bf16 zero = __float2bfloat16(0.0f);
  for (int i = threadIdx.x; i < kBM * kBK; i += blockDim.x) {
    int r, c;
    if (sk == 1) { r = i / kBK; c = i % kBK; }
    else { r = i % kBM; c = i / kBM; }
    const int gr = r0 + r, gk = k0 + c;
    s[r][c] = (gr < nrows && gk < nk) ? src[int64_t(gr) * sr + int64_t(gk) * sk] : zero;
  }
}

template <int EPI>
__global__ void __launch_bounds__(128) mlp_gemm_kernel(const GemmArgs g) {
  __shared__ __align__(16) bf16 As[kBM][kPadK];
  __shared__ __align__(16) bf16 Bs[kBN][kPadK];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gq = lane >> 2, tq = lane & 3;
  const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[i][j][c] = 0.0f;
  for (int k0 = 0; k0 < g.K; k0 += kBK) {
    stage_tile(As, g.A, g.sam, g.sak, g.M, g.K, m0, k0);
    stage_tile(Bs, g.B, g.sbn, g.sbk, g.N, g.K, n0, k0);
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kBK; kk += 16) {
      uint32_t af[2][4], bfr[4][2];
#pragma unroll
      for (int mi = 0; mi < 2; ++mi) {
        const int r = wm + mi * 16 + gq;
        af[mi][0] = *reinterpret_cast<const uint32_t*>(&As[r][kk + 2 * tq]);
        af[mi][1] = *reinterpret_cast<const uint32_t*>(&As[r + 8][kk + 2 * tq]);
        af[mi][2] = *reinterpret_cast<const uint32_t*>(&As[r][kk + 2 * tq + 8]);
        af[mi][3] = *reinterpret_cast<const uint32_t*>(&As[r + 8][kk + 2 * tq + 8]);
      }
#pragma unroll
      for (int ni = 0; ni < 4; ++ni) {
        const int c = wn + ni * 8 + gq;
        bfr[ni][0] = *reinterpret_cast<const uint32_t*>(&Bs[c][kk + 2 * tq]);
        bfr[ni][1] = *reinterpret_cast<const uint32_t*>(&Bs[c][kk + 2 * tq + 8]);
      }
#pragma unroll
      for (int mi = 0; mi < 2; ++mi)
#pragma unroll
        for (int ni = 0; ni < 4; ++ni) mma_bf16_16816(acc[mi][ni], af[mi], bfr[ni]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int mi = 0; mi < 2; ++mi)
#pragma unroll
    for (int ni = 0; ni < 4; ++ni)
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const int row = m0 + wm + mi * 16 + gq + 8 * h;
          const int col = n0 + wn + ni * 8 + 2 * tq + c;
          if (row >= g.M || col >= g.N) continue;
          const float v = acc[mi][ni][2 * h + c];
          const int64_t idx = int64_t(row) * g.ldo + col;
          if constexpr (EPI == EPI_BIAS_GELU) {
            const float z = v + g.bias[col];
            g.outf[idx] = z;
            g.outh[idx] = __float2bfloat16(gelu_f(z));
          } else if constexpr (EPI == EPI_BIAS) {
            g.outf[idx] = v + g.bias[col];
          } else if constexpr (EPI == EPI_GELU_BWD) {
            g.outh[idx] = __float2bfloat16(v * gelu_grad(g.z[idx]));
          } else {
            g.outf[idx] = v;
          }
        }
}

__global__ void cast_bf16_kernel(const float* __restrict__ x, int64_t n, bf16* __restrict__ y) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    y[i] = __float2bfloat16(x[i]);
}

// dy = bf16(2 w_o (y - t) / (M O)); *loss += sum w_o (y - t)^2 / (M O).
__global__ void mse_grad_kernel(const float* __restrict__ y, const float* __restrict__ t,
                                const float* __restrict__ w, int64_t M, int O, bf16* __restrict__ dy,
                                float* __restrict__ loss) {
  const int64_t n = M * O;
  const float inv = 1.0f / float(n);
  float part = 0.0f;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const float wo = w ? w[i % O] : 1.0f;
    const float e = y[i] - t[i];
    part += wo * e * e;
    dy[i] = __float2bfloat16(2.0f * wo * e * inv);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  __shared__ float red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x == 0) {
    float s = 0.0f;
    for (int i = 0; i < int(blockDim.x >> 5); ++i) s += red[i];
    atomicAdd(loss, s * inv);
  }
}

// out[n] = sum_m d[m][n] (FP32, sequential in m: deterministic).
__global__ void colsum_kernel(const bf16* __restrict__ d, int64_t M, int N, float* __restrict__ out) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.0f;
  for (int64_t m = 0; m < M; ++m) s += __bfloat162float(d[m * N + n]);
  out[n] = s;
}

// Adam (Kingma & Ba 2015) on the FP32 master copy; refreshes the BF16 copy.
// c1 = 1 / (1 - beta1^t), c2 = 1 / (1 - beta2^t).
__global__ void adam_kernel(float* __restrict__ w, bf16* __restrict__ w16, const float* __restrict__ g,
                            float* __restrict__ m, float* __restrict__ v, int64_t n, float lr, float b1, float b2,
                            float eps, float c1, float c2) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    w[i] = wi;
    w16[i] = __float2bfloat16(wi);
  }
}

// Optional squash v -> asinh(v / s) (s > 0): log-like beyond |v| ~ s, so a
// column spanning decades is fitted to relative accuracy.
__device__ __forceinline__ double squash_f(double v, double s) { return s > 0.0 ? asinh(v / s) : v; }
__device__ __forceinline__ double unsquash_f(double v, double s) { return s > 0.0 ? s * sinh(v) : v; }

__global__ void squash_kernel(float* __restrict__ t, int64_t n, double s) {
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    t[i] = float(squash_f(double(t[i]), s));
}

// Column statistics of t [rows][cols] in FP64: mean and standard deviation.
__global__ void colstats_kernel(const float* __restrict__ t, int64_t rows, int cols, float* __restrict__ mean,
                                float* __restrict__ stdv) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  double s = 0.0, s2 = 0.0;
  for (int64_t r = 0; r < rows; ++r) s += double(t[r * cols + c]);
  const double mu = s / double(rows);
  for (int64_t r = 0; r < rows; ++r) {
    const double e = double(t[r * cols + c]) - mu;
    s2 += e * e;
  }
  mean[c] = float(mu);
  stdv[c] = float(sqrt(s2 / double(rows > 1 ? rows - 1 : 1)));
}

// With m = max_c std_c: w_c = clamp((std_c / m)^2, 1e-4, 1) (optional), then
// std_c = max(std_c, floor_frac m); one CTA.
__global__ void stdfloor_kernel(float* __restrict__ stdv, int cols, float floor_frac, float* __restrict__ w) {
  __shared__ float red[32];
  float mx = 0.0f;
  for (int c = threadIdx.x; c < cols; c += blockDim.x) mx = fmaxf(mx, stdv[c]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x < 32) {
    float v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (threadIdx.x == 0) red[0] = v;
  }
  __syncthreads();
  const float m = fmaxf(red[0], 1e-30f);
  const float fl = fmaxf(floor_frac * m, 1e-30f);
  for (int c = threadIdx.x; c < cols; c += blockDim.x) {
    const float r = stdv[c] / m;
    if (w) w[c] = fminf(fmaxf(r * r, 1e-4f), 1.0f);
    stdv[c] = fmaxf(stdv[c], fl);
  }
}

__global__ void normalize_kernel(float* __restrict__ t, int64_t rows, int cols, const float* __restrict__ mean,
                                 const float* __restrict__ stdv) {
  const int64_t n = rows * cols;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int c = int(i % cols);
    t[i] = (t[i] - mean[c]) / stdv[c];
  }
}

// Separable unitary 2-D DFT of one nx x ny field held in shared memory
// (site p = x ny + y, natural k order k = kx ny + ky):
//   out_k = N^{-1/2} sum_p in_p exp(sign 2 pi i (kx x / nx + ky y / ny)).
// FP64 with exact twiddle phases (the integer product is reduced mod n).
__device__ void dft2_shared(const double2* in, double2* tmp, double2* out, int nx, int ny, double sign) {
  const int n = nx * ny;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {  // along y
    const int x = i / ny, ky = i % ny;
    double sr = 0.0, si = 0.0;
    for (int y = 0; y < ny; ++y) {
      double s, c;
      sincospi(sign * 2.0 * double((int64_t(ky) * y) % ny) / double(ny), &s, &c);
      const double2 v = in[x * ny + y];
      sr += v.x * c - v.y * s;
      si += v.x * s + v.y * c;
    }
    tmp[i] = make_double2(sr, si);
  }
  __syncthreads();
  const double norm = rsqrt(double(n));
  for (int i = threadIdx.x; i < n; i += blockDim.x) {  // along x
    const int kx = i / ny, ky = i % ny;
    double sr = 0.0, si = 0.0;
    for (int x = 0; x < nx; ++x) {
      double s, c;
      sincospi(sign * 2.0 * double((int64_t(kx) * x) % nx) / double(nx), &s, &c);
      const double2 v = tmp[x * ny + ky];
      sr += v.x * c - v.y * s;
      si += v.x * s + v.y * c;
    }
    out[i] = make_double2(sr * norm, si * norm);
  }
  __syncthreads();
}

// One MLP target row per point: (Re a_k, Im a_k) for every k, then the
// density n = mean_p <|a_p|^2> - 1/2, with a_k the unitary DFT of the mean
// field <a_p>. Inputs are sums over `frames` frames (scale = 1 / frames).
__global__ void targets_kernel(const double* __restrict__ mean, const double* __restrict__ abs2, int nx, int ny,
                               double scale, float* __restrict__ rows, int64_t ld) {
  extern __shared__ __align__(16) double2 sm[];
  const int n = nx * ny;
  double2* a = sm;
  double2* tmp = sm + n;
  const int64_t pt = blockIdx.x;
  const double* mp = mean + pt * 2 * n;
  for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = make_double2(mp[2 * i] * scale, mp[2 * i + 1] * scale);
  __syncthreads();
  dft2_shared(a, tmp, a, nx, ny, -1.0);
  float* r = rows + pt * ld;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    r[2 * i] = float(a[i].x);
    r[2 * i + 1] = float(a[i].y);
  }
  __shared__ double red[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += abs2[pt * n + i] * scale;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < int(blockDim.x >> 5); ++i) t += red[i];
    r[2 * n] = float(t / double(n) - 0.5);
  }
}

// Initial fields from one MLP output row per point (de-standardised with
// mean / std when given, then un-squashed): beta_init = inverse unitary DFT
// of the predicted k-mode amplitudes; beta_sigma = sqrt((n_inc + 1/2) / 2)
// per quadrature with n_inc = min(max(n - |beta_init|^2, 0), max_inc), so
// that <|a|^2>_W - 1/2 starts at the predicted density n (vacuum: 1/2) unless
// the incoherent part is capped.
__global__ void fields_kernel(const float* __restrict__ rows, int64_t ld, const float* __restrict__ mu,
                              const float* __restrict__ sd, double squash, double max_inc, int nx, int ny,
                              double* __restrict__ binit, double* __restrict__ bsigma) {
  extern __shared__ __align__(16) double2 sm[];
  const int n = nx * ny;
  double2* a = sm;
  double2* tmp = sm + n;
  const int64_t pt = blockIdx.x;
  const float* r = rows + pt * ld;
  auto val = [&](int c) {
    const double v = mu ? double(r[c]) * double(sd[c]) + double(mu[c]) : double(r[c]);
    return unsquash_f(v, squash);
  };
  for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = make_double2(val(2 * i), val(2 * i + 1));
  __syncthreads();
  dft2_shared(a, tmp, a, nx, ny, 1.0);
  const double dens = val(2 * n);
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double m2 = a[i].x * a[i].x + a[i].y * a[i].y;
    const double sg = sqrt((fmin(fmax(dens - m2, 0.0), max_inc) + 0.5) * 0.5);
    binit[(pt * n + i) * 2] = a[i].x;
    binit[(pt * n + i) * 2 + 1] = a[i].y;
    bsigma[(pt * n + i) * 2] = sg;
    bsigma[(pt * n + i) * 2 + 1] = 0.0;
  }
}

template <typename T>
struct DevArr {
  T* p = nullptr;
  ~DevArr() { if (p) cudaFree(p); }
  bool alloc(size_t n) {
    if (p) cudaFree(p);
    p = nullptr;
    return n == 0 || cudaMalloc(&p, n * sizeof(T)) == cudaSuccess;
  }
};

int grid_for(int64_t n, int cta) { return int(std::max<int64_t>(1, std::min<int64_t>((n + cta - 1) / cta, 4096))); }

}  // namespace

struct twmc_mlp {
  int device = 0;
  int nl = 0;
  std::vector<int> width;
  std::vector<int64_t> w_off, b_off;
  int64_t nparam = 0, max_batch = 0, step = 0;
  int max_width = 0;
  DevArr<float> w, g, m, v;
  DevArr<bf16> w16;
  std::vector<DevArr<bf16>> act;  // act[l]: input of layer l, [max_batch][width[l]]
  std::vector<DevArr<float>> z;   // z[l]: pre-activation output of layer l-1, [max_batch][width[l]] (l = 1..nl-1)
  DevArr<float> y;                // [max_batch][width[nl]]
  DevArr<bf16> d0, d1;            // backward ping-pong, [max_batch][max_width]
  DevArr<float> loss;
  int64_t launches = 0;
  std::string err;
};

namespace {

int mfail(twmc_mlp* m, int code, const std::string& s) {
  if (m) m->err = s;
  return code;
}

template <int EPI>
bool gemm(twmc_mlp* m, const GemmArgs& g, cudaStream_t s) {
  dim3 grid(unsigned((g.N + kBN - 1) / kBN), unsigned((g.M + kBM - 1) / kBM));
  mlp_gemm_kernel<EPI><<<grid, 128, 0, s>>>(g);
  ++m->launches;
  return cudaPeekAtLastError() == cudaSuccess;
}

// Forward pass of `batch` rows of x (device FP32 [batch][width[0]]) into y
// (device FP32 [batch][width[nl]]), keeping activations for the backward.
bool forward_chunk(twmc_mlp* m, const float* x, int64_t batch, float* yout, cudaStream_t s) {
  const int64_t nin = batch * m->width[0];
  cast_bf16_kernel<<<grid_for(nin, 256), 256, 0, s>>>(x, nin, m->act[0].p);
  ++m->launches;
  for (int l = 0; l < m->nl; ++l) {
    const int K = m->width[l], N = m->width[l + 1];
    GemmArgs g{};
    g.A = m->act[l].p; g.sam = K; g.sak = 1;
    g.B = m->w16.p + m->w_off[l]; g.sbn = K; g.sbk = 1;
    g.M = int(batch); g.N = N; g.K = K;
    g.bias = m->w.p + m->b_off[l];
    g.ldo = N;
    bool ok;
    if (l + 1 < m->nl) {
      g.outf = m->z[l + 1].p;
      g.outh = m->act[l + 1].p;
      ok = gemm<EPI_BIAS_GELU>(m, g, s);
    } else {
      g.outf = yout;
      ok = gemm<EPI_BIAS>(m, g, s);
    }
    if (!ok) return false;
  }
  return true;
}

bool fields_smem_ok(int64_t nx, int64_t ny, size_t* smem) {
  const int64_t n = nx * ny;
  if (nx < 1 || ny < 1 || n > 4096) return false;
  *smem = size_t(2 * n) * sizeof(double2);
  return true;
}

}  // namespace

extern "C" {

int twmc_mlp_create(int32_t n_layers, const int32_t* widths, int64_t max_batch, uint64_t seed, twmc_mlp** out) {
  if (!out || !widths || n_layers < 1 || n_layers > 16 || max_batch < 1 || max_batch > (int64_t(1) << 24))
    return TWMC_ERR_INVALID;
  *out = nullptr;
  for (int l = 0; l <= n_layers; ++l)
    if (widths[l] < 1 || widths[l] > 65536) return TWMC_ERR_INVALID;
  auto* m = new twmc_mlp;
  cudaGetDevice(&m->device);
  m->nl = n_layers;
  m->width.assign(widths, widths + n_layers + 1);
  m->max_batch = max_batch;
  int64_t off = 0;
  for (int l = 0; l < n_layers; ++l) {
    m->w_off.push_back(off);
    off += int64_t(widths[l + 1]) * widths[l];
    m->b_off.push_back(off);
    off += widths[l + 1];
  }
  m->nparam = off;
  m->max_width = *std::max_element(m->width.begin(), m->width.end());
  m->act.resize(n_layers);
  m->z.resize(n_layers);
  bool ok = m->w.alloc(off) && m->g.alloc(off) && m->m.alloc(off) && m->v.alloc(off) && m->w16.alloc(off) &&
            m->y.alloc(size_t(max_batch) * widths[n_layers]) && m->d0.alloc(size_t(max_batch) * m->max_width) &&
            m->d1.alloc(size_t(max_batch) * m->max_width) && m->loss.alloc(1);
  for (int l = 0; l < n_layers && ok; ++l) {
    ok = m->act[l].alloc(size_t(max_batch) * widths[l]);
    if (ok && l > 0) ok = m->z[l].alloc(size_t(max_batch) * widths[l]);
  }
  if (!ok) {
    cudaGetLastError();
    delete m;
    return TWMC_ERR_NOMEM;
  }
  // Glorot-uniform weights, zero biases, from a seeded host generator.
  std::vector<float> p(size_t(off), 0.0f);
  std::mt19937_64 gen(seed);
  for (int l = 0; l < n_layers; ++l) {
    const double a = std::sqrt(6.0 / double(widths[l] + widths[l + 1]));
    std::uniform_real_distribution<double> u(-a, a);
    for (int64_t i = 0; i < int64_t(widths[l + 1]) * widths[l]; ++i) p[size_t(m->w_off[l] + i)] = float(u(gen));
  }
  *out = m;
  return twmc_mlp_set_params(m, p.data());
}

int64_t twmc_mlp_param_count(const twmc_mlp* m) { return m ? m->nparam : -1; }

int twmc_mlp_set_params(twmc_mlp* m, const float* host) {
  if (!m || !host) return TWMC_ERR_INVALID;
  cudaSetDevice(m->device);
  const size_t n = size_t(m->nparam);
  if (cudaMemcpy(m->w.p, host, n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(m->m.p, 0, n * sizeof(float)) != cudaSuccess || cudaMemset(m->v.p, 0, n * sizeof(float)) != cudaSuccess ||
      cudaMemset(m->g.p, 0, n * sizeof(float)) != cudaSuccess)
    return mfail(m, TWMC_ERR_CUDA, "parameter upload failed");
  cast_bf16_kernel<<<grid_for(int64_t(n), 256), 256>>>(m->w.p, int64_t(n), m->w16.p);
  ++m->launches;
  m->step = 0;
  const cudaError_t e = cudaDeviceSynchronize();
  return e == cudaSuccess ? TWMC_OK : mfail(m, TWMC_ERR_CUDA, cudaGetErrorString(e));
}

int twmc_mlp_get_params(twmc_mlp* m, float* host) {
  if (!m || !host) return TWMC_ERR_INVALID;
  cudaSetDevice(m->device);
  cudaDeviceSynchronize();
  return cudaMemcpy(host, m->w.p, size_t(m->nparam) * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess
             ? TWMC_OK
             : mfail(m, TWMC_ERR_CUDA, "parameter download failed");
}

int twmc_mlp_get_grads(twmc_mlp* m, float* host) {
  if (!m || !host) return TWMC_ERR_INVALID;
  cudaSetDevice(m->device);
  cudaDeviceSynchronize();
  return cudaMemcpy(host, m->g.p, size_t(m->nparam) * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess
             ? TWMC_OK
             : mfail(m, TWMC_ERR_CUDA, "gradient download failed");
}

int twmc_mlp_forward(twmc_mlp* m, const float* x, int64_t batch, float* y, void* stream) {
  if (!m || !x || !y || batch < 0) return TWMC_ERR_INVALID;
  cudaSetDevice(m->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  for (int64_t r = 0; r < batch; r += m->max_batch) {
    const int64_t b = std::min(m->max_batch, batch - r);
    if (!forward_chunk(m, x + r * m->width[0], b, y + r * m->width[m->nl], s)) {
      cudaGetLastError();
      return mfail(m, TWMC_ERR_CUDA, "forward launch failed");
    }
  }
  return TWMC_OK;
}

int twmc_mlp_backward(twmc_mlp* m, const float* x, const float* target, const float* weights, int64_t batch,
                      float* loss, void* stream) {
  if (!m || !x || !target || batch < 1 || batch > m->max_batch) return TWMC_ERR_INVALID;
  cudaSetDevice(m->device);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nl = m->nl, O = m->width[nl];
  if (!forward_chunk(m, x, batch, m->y.p, s)) { cudaGetLastError(); return mfail(m, TWMC_ERR_CUDA, "forward launch failed"); }
  cudaMemsetAsync(m->loss.p, 0, sizeof(float), s);
  mse_grad_kernel<<<grid_for(batch * O, 256), 256, 0, s>>>(m->y.p, target, weights, batch, O, m->d0.p, m->loss.p);
  ++m->launches;
  bf16* dcur = m->d0.p;
  bf16* dnext = m->d1.p;
  for (int l = nl - 1; l >= 0; --l) {
    const int K = m->width[l], N = m->width[l + 1];
    // dW_l[n][k] = sum_b dZ[b][n] act_l[b][k]
    GemmArgs gw{};
    gw.A = dcur; gw.sam = 1; gw.sak = N;
    gw.B = m->act[l].p; gw.sbn = 1; gw.sbk = K;
    gw.M = N; gw.N = K; gw.K = int(batch);
    gw.outf = m->g.p + m->w_off[l];
    gw.ldo = K;
    if (!gemm<EPI_STORE>(m, gw, s)) { cudaGetLastError(); return mfail(m, TWMC_ERR_CUDA, "backward launch failed"); }
    colsum_kernel<<<(N + 127) / 128, 128, 0, s>>>(dcur, batch, N, m->g.p + m->b_off[l]);
    ++m->launches;
    if (l > 0) {
      // dZ_{l-1}[b][k] = (sum_n dZ[b][n] W_l[n][k]) gelu'(z_l[b][k])
      GemmArgs gd{};
      gd.A = dcur; gd.sam = N; gd.sak = 1;
      gd.B = m->w16.p + m->w_off[l]; gd.sbn = 1; gd.sbk = K;
      gd.M = int(batch); gd.N = K; gd.K = N;
      gd.z = m->z[l].p;
      gd.outh = dnext;
      gd.ldo = K;
      if (!gemm<EPI_GELU_BWD>(m, gd, s)) { cudaGetLastError(); return mfail(m, TWMC_ERR_CUDA, "backward launch failed"); }
      std::swap(dcur, dnext);
    }
  }
  if (loss) {
    if (cudaMemcpyAsync(loss, m->loss.p, sizeof(float), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return mfail(m, TWMC_ERR_CUDA, "loss download failed");
  }
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? TWMC_OK : mfail(m, TWMC_ERR_CUDA, cudaGetErrorString(e));
}

int twmc_mlp_adam(twmc_mlp* m, float lr, float beta1, float beta2, float eps, void* stream) {
  if (!m || !(lr >= 0.0f) || !(beta1 >= 0.0f && beta1 < 1.0f) || !(beta2 >= 0.0f && beta2 < 1.0f) || !(eps > 0.0f))
    return TWMC_ERR_INVALID;
  cudaSetDevice(m->device);
  ++m->step;
  const float c1 = float(1.0 / (1.0 - std::pow(double(beta1), double(m->step))));
  const float c2 = float(1.0 / (1.0 - std::pow(double(beta2), double(m->step))));
  adam_kernel<<<grid_for(m->nparam, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      m->w.p, m->w16.p, m->g.p, m->m.p, m->v.p, m->nparam, lr, beta1, beta2, eps, c1, c2);
  ++m->launches;
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? TWMC_OK : mfail(m, TWMC_ERR_CUDA, cudaGetErrorString(e));
}

int twmc_mlp_last_loss(twmc_mlp* m, float* loss) {
  if (!m || !loss) return TWMC_ERR_INVALID;
  cudaSetDevice(m->device);
  cudaDeviceSynchronize();
  return cudaMemcpy(loss, m->loss.p, sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess
             ? TWMC_OK
             : mfail(m, TWMC_ERR_CUDA, "loss download failed");
}

const char* twmc_mlp_last_error(const twmc_mlp* m) { return m ? m->err.c_str() : "null network"; }
int64_t twmc_mlp_launch_count(const twmc_mlp* m) { return m ? m->launches : -1; }
void twmc_mlp_destroy(twmc_mlp* m) { delete m; }

int twmc_mlp_standardize(float* t, int64_t rows, int32_t cols, double squash, float floor_frac, float* mean,
                         float* stdv, float* weights, void* stream) {
  if (!t || !mean || !stdv || rows < 1 || cols < 1 || !(floor_frac >= 0.0f) || !(squash >= 0.0))
    return TWMC_ERR_INVALID;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (squash > 0.0) squash_kernel<<<grid_for(rows * cols, 256), 256, 0, s>>>(t, rows * cols, squash);
  colstats_kernel<<<(cols + 127) / 128, 128, 0, s>>>(t, rows, cols, mean, stdv);
  stdfloor_kernel<<<1, 1024, 0, s>>>(stdv, cols, floor_frac, weights);
  normalize_kernel<<<grid_for(rows * cols, 256), 256, 0, s>>>(t, rows, cols, mean, stdv);
  return cudaGetLastError() == cudaSuccess ? TWMC_OK : TWMC_ERR_CUDA;
}

int twmc_mlp_targets(const double* mean, const double* abs2, int64_t n_points, int64_t nx, int64_t ny,
                     int32_t frames, float* rows, int64_t ld, void* stream) {
  size_t smem = 0;
  if (!mean || !abs2 || !rows || n_points < 1 || frames < 1 || !fields_smem_ok(nx, ny, &smem) || ld < 2 * nx * ny + 1)
    return TWMC_ERR_INVALID;
  if (cudaFuncSetAttribute(targets_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess) {
    cudaGetLastError();
    return TWMC_ERR_CUDA;
  }
  targets_kernel<<<unsigned(n_points), 256, smem, static_cast<cudaStream_t>(stream)>>>(
      mean, abs2, int(nx), int(ny), 1.0 / double(frames), rows, ld);
  return cudaGetLastError() == cudaSuccess ? TWMC_OK : TWMC_ERR_CUDA;
}

int twmc_mlp_fields(const float* rows, int64_t ld, int64_t n_points, const float* mean, const float* stdv,
                    double squash, double max_incoherent, int64_t nx, int64_t ny, double* beta_init,
                    double* beta_sigma, void* stream) {
  size_t smem = 0;
  if (!rows || !beta_init || !beta_sigma || n_points < 1 || !fields_smem_ok(nx, ny, &smem) ||
      ld < 2 * nx * ny + 1 || (!mean) != (!stdv) || !(squash >= 0.0) || !(max_incoherent >= 0.0))
    return TWMC_ERR_INVALID;
  if (cudaFuncSetAttribute(fields_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess) {
    cudaGetLastError();
    return TWMC_ERR_CUDA;
  }
  fields_kernel<<<unsigned(n_points), 256, smem, static_cast<cudaStream_t>(stream)>>>(
      rows, ld, mean, stdv, squash, max_incoherent, int(nx), int(ny), beta_init, beta_sigma);
  return cudaGetLastError() == cudaSuccess ? TWMC_OK : TWMC_ERR_CUDA;
}

}  // extern "C"
