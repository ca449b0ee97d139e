// twmc_noalloc.cu -- k-space populations and FP64 moment blocks of a
// caller-owned device batch, without any device allocation.
//
// For callers that cannot allocate device memory themselves or through the
// library: a host application that has already handed the whole device to its
// own memory pool, or a latency-critical loop where cudaMalloc's implicit
// synchronisation is not acceptable. The library's own path (twmc_batch_*)
// allocates a k-space scratch buffer per handle; this entry point instead uses
// one file-scope device array of fixed size, shared by every call.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>

#include "twmc.h"
#include "twmc_moments.cuh"
#include "twmc_square.cuh"

namespace twmc {
namespace {

// Scratch for |FFT(state)|^2 / N: at most 4,194,304 floats (16 MiB), i.e.
// n_traj * nx * ny <= 4194304 (1024 trajectories of 64 x 64). Every device
// that loads the library holds it until the process exits.
constexpr size_t kNoAllocScratchFloats = size_t(1) << 22;
static __device__ __align__(256) float g_kspace_scratch[kNoAllocScratchFloats];

// Device address of the scratch array per device (looked up with that device
// current). The cached address serves calls made during stream capture, where
// the lookup must not run; calls outside capture look it up again, so a
// context torn down and recreated (cudaDeviceReset) after an earlier call does
// not leave a stale address behind.
std::mutex g_scratch_mu;
float* g_scratch_ptr[128] = {};
// Bumped when a device's scratch address changes (its context was recreated):
// per-plan launch settings made in the old context are redone.
int g_generation[128] = {};

float* scratch_for_current_device(cudaStream_t s, std::string* err) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 128) {
    *err = "no current CUDA device";
    return nullptr;
  }
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess) {
    cudaGetLastError();
    *err = "cudaStreamIsCapturing failed";
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev] || cap == cudaStreamCaptureStatusNone) {
    if (cap != cudaStreamCaptureStatusNone) {
      *err = "first call on this device made during stream capture";
      return nullptr;
    }
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_kspace_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      *err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return nullptr;
    }
    if (g_scratch_ptr[dev] && g_scratch_ptr[dev] != static_cast<float*>(p)) ++g_generation[dev];
    g_scratch_ptr[dev] = static_cast<float*>(p);
  }
  return g_scratch_ptr[dev];
}

// |FFT(beta)|^2 / N of every trajectory (natural k order) with the register
// FFT plan of the step kernel; twiddles are computed here, not read from a
// library table.
template <class P, int CTA>
__global__ void __launch_bounds__(CTA) kspace_noalloc_kernel(const float2* __restrict__ state, int64_t ntraj,
                                                             float* __restrict__ nk) {
  using T = float2;
  using I = PlanInfo<P>;
  using Cfg = SquareCfg<P, CTA, float>;
  constexpr int E = I::E, N = I::N, TPT = I::TPT, TPC = Cfg::TPC;
  constexpr int NP = P::npass, LAST = NP - 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s_tw = reinterpret_cast<T*>(smem_raw);
  T* s_x = s_tw + (I::TW0 + I::TW1);
  const int tid = threadIdx.x;
  const int slot = TPC == 1 ? 0 : tid / TPT;
  const int t = TPC == 1 ? tid : tid % TPT;
  for (int i = tid; i < I::TW0; i += CTA) {
    double sn, cs;
    sincospi(2.0 * double(i) / double(I::M0), &sn, &cs);
    s_tw[i] = make_float2(float(cs), float(-sn));
  }
  for (int i = tid; i < I::TW1; i += CTA) {
    double sn, cs;
    sincospi(2.0 * double(i) / double(I::M1), &sn, &cs);
    s_tw[I::TW0 + i] = make_float2(float(cs), float(-sn));
  }
  __syncthreads();
  const T* tw0 = s_tw;
  const T* tw1 = s_tw + I::TW0;
  int pos_thr[NP];
  int xbase[NP];
  static_for<NP>([&](auto KK) {
    constexpr int k = decltype(KK)::value;
    int p = 0;
    static_for<P::nthr>([&](auto II) {
      constexpr int i = decltype(II)::value;
      constexpr int b = P::thr[k][i];
      p |= ((t >> i) & 1) << b;
    });
    pos_thr[k] = p;
    xbase[k] = pad16((slot << P::nbits) | p);
  });
  int buf = 0;
  const int64_t ngroups = (ntraj + TPC - 1) / TPC;
  for (int64_t g = blockIdx.x; g < ngroups; g += gridDim.x) {
    const int64_t traj = g * TPC + slot;
    const bool active = traj < ntraj;
    const T* st = state + (active ? traj : 0) * N;
    T x[E];
    static_for<E>([&](auto S) {
      constexpr int s = decltype(S)::value;
      x[s] = st[pos_thr[0] | I::pos_reg(0, s)];
    });
    static_for<NP>([&](auto KK) {
      constexpr int k = decltype(KK)::value;
      if constexpr (k > 0) {
        fft_exchange<P, k - 1, k, Cfg::SYNC_WARP>(x, s_x + buf * Cfg::XSZ, xbase[k - 1], xbase[k]);
        buf ^= 1;
      }
      fft_pass<P, k, false>(x, tw0, tw1, pos_thr[k]);
    });
    if (active) {
      float* out = nk + traj * N;
      static_for<E>([&](auto S) {
        constexpr int s = decltype(S)::value;
        const uint32_t p = uint32_t(pos_thr[LAST] | I::pos_reg(LAST, s));
        const uint32_t pc = p & ((1u << P::by) - 1u), pr = p >> P::by;
        const uint32_t ky = P::by ? (__brev(pc) >> (32 - P::by)) : 0u;
        const uint32_t kx = P::bx ? (__brev(pr) >> (32 - P::bx)) : 0u;
        out[(kx << P::by) | ky] = (x[s].x * x[s].x + x[s].y * x[s].y) / float(N);
      });
    }
  }
}

// Resident CTAs of a plan's kernel on the whole device, per device, found
// once per context (shared-memory attribute, SM count, occupancy) and cached
// under the scratch mutex.
template <class P>
cudaError_t launch_kspace(const float2* state, int64_t ntraj, float* nk, cudaStream_t s) {
  constexpr int CTA = cta_for<float, P>();
  using Cfg = SquareCfg<P, CTA, float>;
  using I = PlanInfo<P>;
  const size_t smem = sizeof(float2) * (size_t(I::TW0 + I::TW1) + 2 * size_t(Cfg::XSZ));
  auto fn = kspace_noalloc_kernel<P, CTA>;
  static int resident[128] = {};
  static int generation[128] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 128) return e != cudaSuccess ? e : cudaErrorInvalidDevice;
  int slots;
  {
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (resident[dev] <= 0 || generation[dev] != g_generation[dev]) {
      generation[dev] = g_generation[dev];
      e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
      if (e != cudaSuccess) return e;
      int sms = 0, per_sm = 0;
      e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) return e;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, CTA, smem);
      if (e != cudaSuccess) return e;
      resident[dev] = sms * std::max(per_sm, 1);
    }
    slots = resident[dev];
  }
  const int64_t groups = (ntraj + Cfg::TPC - 1) / Cfg::TPC;
  const int grid = int(std::min<int64_t>(groups, int64_t(slots)));
  fn<<<grid, CTA, smem, s>>>(state, ntraj, nk);
  e = cudaGetLastError();
  if (e != cudaSuccess) {  // e.g. the attribute was lost with a recreated context: redo the setup next call
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    resident[dev] = 0;
  }
  return e;
}

}  // namespace
}  // namespace twmc

extern "C" int twmc_kspace_moments_noalloc(const void* state, int64_t n_traj, int64_t nx, int64_t ny,
                                            int32_t n_blocks, double* moments, void* stream) {
  using namespace twmc;
  if (!state || !moments || n_traj < 1 || n_blocks < 1 || n_blocks > 65535) return TWMC_ERR_INVALID;
  // the compiled plans have at most 4096 sites: bound both sides before any
  // arithmetic on them
  if (nx < 1 || ny < 1 || nx > 4096 || ny > 4096 || nx * ny > 4096) return TWMC_ERR_INVALID;
  auto lg = [](int64_t v) { int b = 0; while ((int64_t(1) << b) < v) ++b; return (int64_t(1) << b) == v ? b : -1; };
  const int bx = lg(nx), by = lg(ny);
  const int64_t n = nx * ny;
  if (n_traj > int64_t(kNoAllocScratchFloats) / n) return TWMC_ERR_INVALID;  // beyond the scratch array
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  std::string err;
  float* nk = scratch_for_current_device(s, &err);
  if (!nk) return TWMC_ERR_CUDA;
  const float2* st = static_cast<const float2*>(state);
  cudaError_t e = cudaErrorInvalidValue;
  bool shape_ok = true;
#define TWMC_SHAPE(BX, BY) else if (bx == BX && by == BY) e = launch_kspace<Plan_##BX##_##BY>(st, n_traj, nk, s);
  if (bx < 0 || by < 0) shape_ok = false;
  TWMC_SHAPE(0, 5) TWMC_SHAPE(0, 6) TWMC_SHAPE(0, 7) TWMC_SHAPE(0, 8) TWMC_SHAPE(0, 9) TWMC_SHAPE(0, 10)
  TWMC_SHAPE(0, 11) TWMC_SHAPE(0, 12) TWMC_SHAPE(4, 4) TWMC_SHAPE(5, 5) TWMC_SHAPE(6, 6)
  else shape_ok = false;
#undef TWMC_SHAPE
  if (!shape_ok) return TWMC_ERR_INVALID;
  if (e != cudaSuccess) { cudaGetLastError(); return TWMC_ERR_CUDA; }
  MomentArgs m;
  m.ntraj = n_traj;
  m.nsites = n;
  m.prec = 0;
  m.state = state;
  m.nk = nk;
  m.nblocks = n_blocks;
  m.out = moments;
  dim3 grid(unsigned((n + 127) / 128), unsigned(n_blocks));
  moments_kernel<float><<<grid, 128, 0, s>>>(m);
  e = cudaGetLastError();
  return e == cudaSuccess ? TWMC_OK : TWMC_ERR_CUDA;
}
