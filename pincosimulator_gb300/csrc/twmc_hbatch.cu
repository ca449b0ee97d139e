// twmc_hbatch.cu -- heterogeneous batch: parameter points of different
// lattice sizes advanced together, one persistent launch per frame.
//
// Each point is a square lattice (1-D chain or 2-D) with uniform parameters
// and its own trajectories. Points whose shape has a register-FFT plan that
// fits 256 threads per CTA run inside hbatch_kernel: a persistent kernel whose
// CTAs take (point, trajectory group) work items from an atomic counter and
// run the square-lattice step body for that point (tables and arguments are
// reloaded into shared memory when the point changes). Other points (and
// points the autotuner assigns to the real-space kernel) run through
// ell_kernel_dev on a second stream. One frame -- counter reset, the
// persistent launch, the real-space launches, the batched FP64 moments and the
// advance of every point's Philox step counter -- is captured once into a CUDA
// graph and replayed per frame; the per-point arguments live in device memory
// so the replayed graph needs no updates.
//
// Autotuner: for every shape that both paths can run, the first batch that
// needs it times the FFT kernel and the real-space kernel on a trial batch and
// keeps the faster; choices are cached per device and shape in a JSON file
// ($TWMC_TUNE_CACHE, default ~/.cache/twmc_tune.json).
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include <sys/stat.h>

#include "twmc.h"
#include "twmc_moments.cuh"
#include "twmc_square.cuh"

namespace twmc {

bool ell_prepare(int prec, StepArgs* a, int* variant, int* grid, size_t* smem, std::string* err);
bool ell_launch_dev(int prec, int variant, int hop, const StepArgs* dev_args, int grid, size_t smem, cudaStream_t s,
                    std::string* err);

namespace {

constexpr int HB_CTA = 256;

// shapes of the persistent kernel (256 threads hold 4096 sites)
#define TWMC_HB_SHAPES(X) X(0, 5) X(0, 6) X(0, 7) X(0, 8) X(0, 9) X(0, 10) X(4, 4) X(5, 5) X(6, 6)

template <class P>
constexpr size_t hb_smem() {
  using C = SquareCfg<P, HB_CTA, float>;
  using I = PlanInfo<P>;
  return sizeof(float2) * (size_t(I::TW0 + I::TW1) + 2 * size_t(C::XSZ) + size_t(C::TPC) * I::N) +
         sizeof(float) * size_t(I::M0 + I::M1);
}
constexpr size_t cmax(size_t a, size_t b) { return a > b ? a : b; }
constexpr size_t kHbSmem =
    cmax(cmax(cmax(hb_smem<Plan_0_5>(), hb_smem<Plan_0_6>()), cmax(hb_smem<Plan_0_7>(), hb_smem<Plan_0_8>())),
         cmax(cmax(hb_smem<Plan_0_9>(), hb_smem<Plan_0_10>()),
              cmax(hb_smem<Plan_4_4>(), cmax(hb_smem<Plan_5_5>(), hb_smem<Plan_6_6>()))));

enum HbShape : int {
#define TWMC_HB_ENUM(BX, BY) kShape_##BX##_##BY,
  TWMC_HB_SHAPES(TWMC_HB_ENUM)
#undef TWMC_HB_ENUM
  kShapeCount
};

int hb_shape_id(int bx, int by) {
#define TWMC_HB_ID(BX, BY) if (bx == BX && by == BY) return kShape_##BX##_##BY;
  TWMC_HB_SHAPES(TWMC_HB_ID)
#undef TWMC_HB_ID
  return -1;
}

int hb_tpc(int shape) {
  switch (shape) {
#define TWMC_HB_TPC(BX, BY) case kShape_##BX##_##BY: return SquareCfg<Plan_##BX##_##BY, HB_CTA, float>::TPC;
    TWMC_HB_SHAPES(TWMC_HB_TPC)
#undef TWMC_HB_TPC
    default: return 1;
  }
}

template <class P>
__device__ __forceinline__ void hb_run(unsigned char* smem, const StepArgs& a, bool reload, int64_t group, int& buf) {
  SquareGroup<float, P, HB_CTA, true> g(smem);  // batch points: Philox noise, scalar U, F
  if (reload) {
    g.load_tables(a);
    __syncthreads();
  }
  g.run(a, group, buf);
}

__global__ void __launch_bounds__(HB_CTA, 2)
hbatch_kernel(const StepArgs* __restrict__ pts, const int* __restrict__ pshape, const int2* __restrict__ items,
              int nitems, int* __restrict__ counter) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(16) StepArgs s_a;
  __shared__ int s_item;
  int cur = -1;
  int buf = 0;
  for (;;) {
    __syncthreads();  // the previous item is done with the tables and arguments
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= nitems) break;
    const int2 w = items[it];
    const bool reload = w.x != cur;
    if (reload) {
      for (int i = threadIdx.x; i < int(sizeof(StepArgs) / 4); i += HB_CTA)
        reinterpret_cast<uint32_t*>(&s_a)[i] = reinterpret_cast<const uint32_t*>(pts + w.x)[i];
      __syncthreads();
      cur = w.x;
    }
    switch (pshape[w.x]) {
#define TWMC_HB_CASE(BX, BY) \
  case kShape_##BX##_##BY: hb_run<Plan_##BX##_##BY>(smem_raw, s_a, reload, w.y, buf); break;
      TWMC_HB_SHAPES(TWMC_HB_CASE)
#undef TWMC_HB_CASE
      default: break;
    }
  }
}

// FP64 moment blocks of every point: grid (site chunk, block, point).
__global__ void hbatch_moments_kernel(const MomentArgs* __restrict__ ma) {
  const MomentArgs& a = ma[blockIdx.z];
  const int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (p >= a.nsites || int(blockIdx.y) >= a.nblocks) return;
  moments_site<float>(a, p, int(blockIdx.y));
}

// Trajectory means of a and |a|^2 per site of every point, FP64 compensated,
// in trajectory order: grid (site chunk, point). Point i's sites start at
// site_off[i] in mean (complex) and abs2.
__global__ void hbatch_field_kernel(const MomentArgs* __restrict__ ma, const int64_t* __restrict__ site_off,
                                    double* __restrict__ mean, double* __restrict__ abs2, int accumulate) {
  const MomentArgs& a = ma[blockIdx.y];
  const int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (p >= a.nsites) return;
  const float2* st = reinterpret_cast<const float2*>(a.state);
  KSum sr, si, s2;
  for (int64_t tr = 0; tr < a.ntraj; ++tr) {
    const float2 v = st[tr * a.nsites + p];
    sr.add(double(v.x));
    si.add(double(v.y));
    s2.add(double(v.x) * double(v.x) + double(v.y) * double(v.y));
  }
  const double inv = 1.0 / double(a.ntraj);
  const int64_t o = site_off[blockIdx.y] + p;
  const double mr = sr.value() * inv, mi = si.value() * inv, m2 = s2.value() * inv;
  mean[2 * o] = accumulate ? mean[2 * o] + mr : mr;
  mean[2 * o + 1] = accumulate ? mean[2 * o + 1] + mi : mi;
  abs2[o] = accumulate ? abs2[o] + m2 : m2;
}

// Site averages of every moment block: out[(blk_off[i] + b) * 3 + c] =
// mean over sites of moments[i][b][site][c]; grid (block, point), FP64.
__global__ void hbatch_block_means_kernel(const MomentArgs* __restrict__ ma, const int64_t* __restrict__ blk_off,
                                          double* __restrict__ out) {
  const MomentArgs& a = ma[blockIdx.y];
  const int b = blockIdx.x;
  if (b >= a.nblocks) return;
  double s[3] = {0.0, 0.0, 0.0};
  for (int64_t p = threadIdx.x; p < a.nsites; p += blockDim.x)
#pragma unroll
    for (int c = 0; c < 3; ++c) s[c] += a.out[(int64_t(b) * a.nsites + p) * 3 + c];
  __shared__ double red[3][32];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    double v = s[c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[c][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double v = 0.0;
    for (int w = 0; w < int(blockDim.x >> 5); ++w) v += red[threadIdx.x][w];
    out[(blk_off[blockIdx.y] + b) * 3 + threadIdx.x] = v / double(a.nsites);
  }
}

__global__ void hbatch_bump_kernel(StepArgs* pts, int n, uint32_t steps) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) pts[i].step0 += steps;
}

template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  ~DBuf() { if (p) cudaFree(p); }
  bool alloc(size_t count) {
    if (p) cudaFree(p);
    p = nullptr;
    n = count;
    if (!count) return true;
    return cudaMalloc(&p, count * sizeof(T)) == cudaSuccess;
  }
};

std::string tune_cache_path() {
  if (const char* e = std::getenv("TWMC_TUNE_CACHE")) return e;
  const char* home = std::getenv("HOME");
  return std::string(home ? home : ".") + "/.cache/twmc_tune.json";
}

// cache: one line per entry: "<device>|<bx>x<by>": "fft"|"ell"
std::map<std::string, std::string> read_cache(const std::string& path) {
  std::map<std::string, std::string> m;
  std::ifstream f(path);
  std::string line;
  while (std::getline(f, line)) {
    const size_t a = line.find('"'), b = line.find('"', a + 1), c = line.find('"', b + 1), d = line.find('"', c + 1);
    if (a == std::string::npos || d == std::string::npos) continue;
    m[line.substr(a + 1, b - a - 1)] = line.substr(c + 1, d - c - 1);
  }
  return m;
}

void write_cache(const std::string& path, const std::map<std::string, std::string>& m) {
  const size_t slash = path.rfind('/');
  if (slash != std::string::npos) {
    const std::string dir = path.substr(0, slash);
    for (size_t i = 1; i <= dir.size(); ++i)
      if (i == dir.size() || dir[i] == '/') mkdir(dir.substr(0, i).c_str(), 0755);
  }
  std::ofstream f(path);
  f << "{\n";
  size_t k = 0;
  for (auto& e : m) f << "  \"" << e.first << "\": \"" << e.second << "\"" << (++k < m.size() ? "," : "") << "\n";
  f << "}\n";
}

std::mutex g_tune_mu;

}  // namespace
}  // namespace twmc

using namespace twmc;
using cd = std::complex<double>;

constexpr int kEllStreams = 8;

struct twmc_hbatch {
  int device = 0;
  cudaStream_t s0 = nullptr, s1 = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr, e0 = nullptr, e1 = nullptr;
  // real-space points run on kEllStreams captured streams (parallel graph
  // branches), so that small points do not serialise behind each other
  std::vector<cudaStream_t> ell_streams;
  std::vector<cudaEvent_t> ell_joins;
  std::string err;
  int64_t frame_steps = 1;
  size_t npts = 0;
  std::vector<twmc_point_desc> desc;
  std::vector<int> shape;          // persistent-kernel shape id, or -1 (real-space kernel)
  std::vector<std::string> plan;
  std::vector<int64_t> nsites, ntraj, off_state, nblocks;
  std::vector<int> ell_variant, ell_grid;
  std::vector<size_t> ell_smem;
  DBuf<float2> state;
  DBuf<float> nk;
  DBuf<uint32_t> seeds, ids;
  DBuf<int> status;
  DBuf<float2> tw;
  DBuf<float> kt;
  DBuf<StepArgs> args;
  DBuf<int> pshape;
  DBuf<int2> items;
  DBuf<int> counter;
  DBuf<MomentArgs> margs;
  DBuf<double> moments;
  std::vector<int64_t> mom_off;
  std::vector<int64_t> traj_off;   // first trajectory of each point in seeds / ids / status
  DBuf<int64_t> site_off;          // first site of each point in the per-site outputs
  int64_t total_sites = 0;
  DBuf<int64_t> blk_off;           // first moment block of each point in the block-mean output
  DBuf<double> blk_means;
  int64_t total_blocks = 0;
  int nitems = 0, grid = 0;
  int64_t max_sites = 0;
  int max_blocks = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t frames_run = 0;
  int64_t launches = 0;
};

namespace {

int hfail(twmc_hbatch* b, int code, const std::string& m) {
  b->err = m;
  return code;
}

// Draws the initial fields of point i (ReadFromSettings): beta_init +
// beta_init_sigma * xi per site, from the per-site device arrays binit /
// bsigma ([sites] complex128) where given, else the point's uniform values.
bool init_point(twmc_hbatch* b, size_t i, const double* binit, const double* bsigma, std::string* e) {
  const twmc_point_desc& p = b->desc[i];
  InitArgs ia;
  std::memset(&ia, 0, sizeof(ia));
  ia.ntraj = b->ntraj[i];
  ia.nsites = b->nsites[i];
  ia.prec = 0;
  ia.state = b->state.p + b->off_state[i];
  ia.seeds = b->seeds.p + b->traj_off[i];
  ia.ids = b->ids.p + b->traj_off[i];
  ia.ic_kind = TWMC_IC_SETTINGS;
  ia.binit = binit;
  ia.bsigma = bsigma;
  ia.binit_s[0] = p.beta_init[0];
  ia.binit_s[1] = p.beta_init[1];
  ia.bsigma_s[0] = p.beta_init_sigma[0];
  ia.bsigma_s[1] = p.beta_init_sigma[1];
  ia.lattice = 0;
  ia.gamma = p.gamma;
  if (!init_launch(ia, b->s0, e)) return false;
  ++b->launches;
  return true;
}

int lg2(int64_t v) {
  if (v <= 0 || (v & (v - 1))) return -1;
  int k = 0;
  while ((int64_t(1) << k) < v) ++k;
  return k;
}

// Fill the step arguments of point i (device pointers filled by the caller).
void fill_args(const twmc_hbatch* b, size_t i, StepArgs* a) {
  const twmc_point_desc& d = b->desc[i];
  std::memset(a, 0, sizeof(*a));
  a->ntraj = d.n_traj;
  a->nsteps = b->frame_steps;
  a->step0 = 0;
  const cd om(d.omega[0], d.omega[1]), U(d.U[0], d.U[1]), F(d.F[0], d.F[1]);
  const cd rsl(om.imag() - d.gamma / 2.0, -om.real());
  const cd iU(-U.imag(), U.real()), iF(-F.imag(), F.real());
  a->rsl_s[0] = rsl.real(); a->rsl_s[1] = rsl.imag();
  a->iU_s[0] = iU.real(); a->iU_s[1] = iU.imag();
  a->iF_s[0] = iF.real(); a->iF_s[1] = iF.imag();
  a->dt = d.dt;
  a->dt4 = std::sqrt(d.gamma * d.dt / 4.0);
  const double sc[6] = {rsl.real(), rsl.imag(), iU.real(), iU.imag(), iF.real(), iF.imag()};
  for (int k = 0; k < 6; ++k) a->f_par[k] = float(sc[k]);
  a->f_dt = float(a->dt);
  a->f_dt4 = float(a->dt4);
  a->f_kn = float(-2.0 * M_LN2 * d.gamma * d.dt / 4.0);
  a->noise_mode = TWMC_NOISE_PHILOX;
  a->nsites = d.nx * d.ny;
  a->nx = d.nx;
  a->ny = d.ny;
  a->hop_kind = 1;
  a->J = d.J;
  a->f_J = float(d.J);
}

}  // namespace

extern "C" {

int twmc_hbatch_create(const twmc_point_desc* points, size_t n, int64_t frame_steps, int32_t tune, twmc_hbatch** out) {
  if (!out) return TWMC_ERR_INVALID;
  *out = nullptr;
  twmc_hbatch* b = new (std::nothrow) twmc_hbatch();
  if (!b) return TWMC_ERR_NOMEM;
  *out = b;
  if (!points || n == 0) return hfail(b, TWMC_ERR_INVALID, "no points");
  if (frame_steps < 1) return hfail(b, TWMC_ERR_INVALID, "frame_steps must be >= 1");
  cudaGetDevice(&b->device);
  b->frame_steps = frame_steps;
  b->npts = n;
  b->desc.assign(points, points + n);
  for (size_t i = 0; i < n; ++i) {
    const twmc_point_desc& d = points[i];
    if (d.nx < 1 || d.ny < 1 || d.n_traj < 1 || !(d.dt > 0) || d.gamma < 0 || d.n_moment_blocks < 0)
      return hfail(b, TWMC_ERR_INVALID, "point " + std::to_string(i) + ": invalid parameters");
    if (d.nx * d.ny > 16384) return hfail(b, TWMC_ERR_INVALID, "point " + std::to_string(i) + ": more than 16384 sites");
  }
  cudaStreamCreateWithFlags(&b->s0, cudaStreamNonBlocking);
  cudaStreamCreateWithFlags(&b->s1, cudaStreamNonBlocking);
  cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming);
  b->ell_streams.assign(kEllStreams, nullptr);
  b->ell_joins.assign(kEllStreams, nullptr);
  b->ell_streams[0] = b->s1;
  b->ell_joins[0] = b->join;
  for (int k = 1; k < kEllStreams; ++k) {
    cudaStreamCreateWithFlags(&b->ell_streams[k], cudaStreamNonBlocking);
    cudaEventCreateWithFlags(&b->ell_joins[k], cudaEventDisableTiming);
  }
  cudaEventCreate(&b->e0);
  cudaEventCreate(&b->e1);
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, b->device);
  const std::string devname = prop.name;

  // kernel per point: persistent FFT kernel where a plan exists (subject to the
  // autotuner), real-space kernel otherwise
  b->shape.assign(n, -1);
  b->plan.assign(n, "ell_kernel<stencil>");
  std::map<std::string, std::string> cache;
  const std::string cpath = tune_cache_path();
  if (tune) cache = read_cache(cpath);
  bool cache_dirty = false;
  for (size_t i = 0; i < n; ++i) {
    const int bx = lg2(points[i].nx), by = lg2(points[i].ny);
    const int sid = (bx >= 0 && by >= 0) ? hb_shape_id(bx, by) : -1;
    if (sid < 0) continue;
    std::string choice = "fft";
    if (tune) {
      const std::string key = devname + "|" + std::to_string(points[i].nx) + "x" + std::to_string(points[i].ny);
      std::lock_guard<std::mutex> lock(g_tune_mu);
      auto it = cache.find(key);
      if (it != cache.end()) {
        choice = it->second;
      } else {
        // trial: both kernels on up to 1024 trajectories, 50 steps
        twmc_system_desc sd;
        std::memset(&sd, 0, sizeof(sd));
        sd.lattice = TWMC_LATTICE_SQUARE;
        sd.nx = points[i].nx;
        sd.ny = points[i].ny;
        sd.J = points[i].J;
        sd.gamma = points[i].gamma;
        sd.dt = points[i].dt;
        sd.frame_steps = 50;
        double rate[2] = {0, 0};
        for (int hop = 0; hop < 2; ++hop) {
          sd.hop_mode = hop;
          twmc_handle* h = nullptr;
          if (twmc_create(&sd, &h) != TWMC_OK) { twmc_destroy(h); continue; }
          const int64_t nt = std::min<int64_t>(1024, std::max<int64_t>(points[i].n_traj, 64));
          std::vector<twmc_task_desc> td(static_cast<size_t>(nt));
          for (int64_t k = 0; k < nt; ++k) {
            std::memset(&td[size_t(k)], 0, sizeof(twmc_task_desc));
            td[size_t(k)].id = uint64_t(k + 1);
            td[size_t(k)].seed = uint32_t(k + 7);
            td[size_t(k)].ic_kind = TWMC_IC_FIXED;
          }
          double ms = 0;
          if (twmc_batch_init(h, td.data(), td.size()) == TWMC_OK && twmc_batch_advance(h, 10) == TWMC_OK &&
              twmc_sync(h, &ms) == TWMC_OK && twmc_batch_advance(h, 50) == TWMC_OK && twmc_sync(h, &ms) == TWMC_OK &&
              ms > 0)
            rate[hop] = double(nt) * 50.0 * double(sd.nx * sd.ny) / (ms * 1e-3);
          twmc_destroy(h);
        }
        choice = rate[1] > rate[0] ? "ell" : "fft";
        cache[key] = choice;
        cache_dirty = true;
      }
    }
    if (choice == "fft") {
      b->shape[i] = sid;
      b->plan[i] = "hbatch_kernel<" + std::to_string(points[i].nx) + "x" + std::to_string(points[i].ny) + ">";
    }
  }
  if (cache_dirty) write_cache(cpath, cache);
  cudaSetDevice(b->device);

  // layout and buffers
  int64_t total = 0, max_sites = 0;
  int max_blocks = 1;
  b->nsites.resize(n);
  b->ntraj.resize(n);
  b->off_state.resize(n);
  b->nblocks.resize(n);
  b->mom_off.resize(n);
  int64_t mtotal = 0;
  for (size_t i = 0; i < n; ++i) {
    b->nsites[i] = points[i].nx * points[i].ny;
    b->ntraj[i] = points[i].n_traj;
    b->off_state[i] = total;
    total += b->nsites[i] * b->ntraj[i];
    max_sites = std::max(max_sites, b->nsites[i]);
    const int nb = int(std::min<int64_t>(points[i].n_moment_blocks > 0 ? points[i].n_moment_blocks : 32, points[i].n_traj));
    b->nblocks[i] = nb;
    max_blocks = std::max(max_blocks, nb);
    b->mom_off[i] = mtotal;
    mtotal += int64_t(nb) * b->nsites[i] * 3;
  }
  b->max_sites = max_sites;
  b->max_blocks = max_blocks;
  std::vector<int64_t> soff(n);
  b->total_sites = 0;
  for (size_t i = 0; i < n; ++i) { soff[i] = b->total_sites; b->total_sites += b->nsites[i]; }
  std::vector<int64_t> boff(n);
  b->total_blocks = 0;
  for (size_t i = 0; i < n; ++i) { boff[i] = b->total_blocks; b->total_blocks += b->nblocks[i]; }
  if (!b->site_off.alloc(n) || !b->blk_off.alloc(n) || !b->blk_means.alloc(size_t(b->total_blocks) * 3))
    return hfail(b, TWMC_ERR_NOMEM, "device allocation failed");
  cudaMemcpy(b->site_off.p, soff.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice);
  cudaMemcpy(b->blk_off.p, boff.data(), n * sizeof(int64_t), cudaMemcpyHostToDevice);
  int64_t trajs = 0;
  for (size_t i = 0; i < n; ++i) trajs += b->ntraj[i];
  if (!b->state.alloc(size_t(total)) || !b->nk.alloc(size_t(total)) || !b->seeds.alloc(size_t(trajs)) ||
      !b->ids.alloc(size_t(trajs)) || !b->status.alloc(size_t(trajs)) || !b->moments.alloc(size_t(mtotal)))
    return hfail(b, TWMC_ERR_NOMEM, "device allocation failed");
  cudaMemset(b->status.p, 0, size_t(trajs) * sizeof(int));
  // tables per point: twiddles [M0 + M1], separable k table [M0 + M1] (dt folded in)
  std::vector<float2> tw;
  std::vector<float> kt;
  std::vector<int64_t> tw_off(n);
  std::vector<int64_t>& traj_off = b->traj_off;
  traj_off.assign(n, 0);
  std::vector<uint32_t> hseeds(static_cast<size_t>(trajs)), hids(static_cast<size_t>(trajs));
  int64_t to = 0;
  for (size_t i = 0; i < n; ++i) {
    const twmc_point_desc& d = points[i];
    tw_off[i] = int64_t(tw.size());
    const double fx = d.nx == 1 ? 0.0 : 1.0, fy = d.ny == 1 ? 0.0 : 1.0;
    const double scale = 2.0 * d.J / double(b->nsites[i]) * d.dt;
    for (int64_t j = 0; j < d.ny; ++j) {
      const cd w = std::polar(1.0, -2.0 * M_PI * double(j) / double(d.ny));
      tw.push_back(make_float2(float(w.real()), float(w.imag())));
      kt.push_back(float(scale * fy * std::cos(2.0 * M_PI / double(d.ny) * double(j))));
    }
    for (int64_t j = 0; j < d.nx; ++j) {
      const cd w = std::polar(1.0, -2.0 * M_PI * double(j) / double(d.nx));
      tw.push_back(make_float2(float(w.real()), float(w.imag())));
      kt.push_back(float(scale * fx * std::cos(2.0 * M_PI / double(d.nx) * double(j))));
    }
    traj_off[i] = to;
    for (int64_t k = 0; k < d.n_traj; ++k) {
      hseeds[size_t(to + k)] = d.seed0 + uint32_t(k);
      hids[size_t(to + k)] = uint32_t(d.id0 + uint64_t(k));
    }
    to += d.n_traj;
  }
  if (!b->tw.alloc(tw.size()) || !b->kt.alloc(kt.size()) || !b->args.alloc(n) || !b->pshape.alloc(n) ||
      !b->counter.alloc(1) || !b->margs.alloc(n))
    return hfail(b, TWMC_ERR_NOMEM, "device allocation failed");
  cudaMemcpy(b->tw.p, tw.data(), tw.size() * sizeof(float2), cudaMemcpyHostToDevice);
  cudaMemcpy(b->kt.p, kt.data(), kt.size() * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemcpy(b->seeds.p, hseeds.data(), hseeds.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(b->ids.p, hids.data(), hids.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(b->pshape.p, b->shape.data(), n * sizeof(int), cudaMemcpyHostToDevice);
  // arguments, real-space launch configurations, work items, moment args
  std::vector<StepArgs> hargs(n);
  std::vector<MomentArgs> hm(n);
  std::vector<int2> hitems;
  b->ell_variant.assign(n, -1);
  b->ell_grid.assign(n, 0);
  b->ell_smem.assign(n, 0);
  for (size_t i = 0; i < n; ++i) {
    StepArgs& a = hargs[i];
    fill_args(b, i, &a);
    a.state = b->state.p + b->off_state[i];
    a.seeds = b->seeds.p + traj_off[i];
    a.ids = b->ids.p + traj_off[i];
    a.status = b->status.p + traj_off[i];
    a.nk = b->nk.p + b->off_state[i];
    a.tw = b->tw.p + tw_off[i];
    a.ktab = b->kt.p + tw_off[i];
    if (b->shape[i] >= 0) {
      const int tpc = hb_tpc(b->shape[i]);
      for (int64_t g = 0; g < (b->ntraj[i] + tpc - 1) / tpc; ++g) hitems.push_back(make_int2(int(i), int(g)));
    } else {
      a.nk = nullptr;  // the real-space kernel has no k-space output
      std::string e;
      if (!ell_prepare(0, &a, &b->ell_variant[i], &b->ell_grid[i], &b->ell_smem[i], &e))
        return hfail(b, TWMC_ERR_INVALID, "point " + std::to_string(i) + ": " + e);
    }
    MomentArgs& m = hm[i];
    m.ntraj = b->ntraj[i];
    m.nsites = b->nsites[i];
    m.prec = 0;
    m.state = a.state;
    m.nk = b->shape[i] >= 0 ? a.nk : nullptr;
    m.nblocks = int(b->nblocks[i]);
    m.out = b->moments.p + b->mom_off[i];
  }
  b->nitems = int(hitems.size());
  if (!b->items.alloc(std::max<size_t>(hitems.size(), 1))) return hfail(b, TWMC_ERR_NOMEM, "device allocation failed");
  if (!hitems.empty()) cudaMemcpy(b->items.p, hitems.data(), hitems.size() * sizeof(int2), cudaMemcpyHostToDevice);
  cudaMemcpy(b->args.p, hargs.data(), n * sizeof(StepArgs), cudaMemcpyHostToDevice);
  cudaMemcpy(b->margs.p, hm.data(), n * sizeof(MomentArgs), cudaMemcpyHostToDevice);

  // initial fields (ReadFromSettings with uniform beta_init / sigma)
  for (size_t i = 0; i < n; ++i) {
    std::string e;
    if (!init_point(b, i, nullptr, nullptr, &e)) return hfail(b, TWMC_ERR_CUDA, e);
  }

  // persistent kernel configuration
  if (b->nitems > 0) {
    cudaError_t e = cudaFuncSetAttribute(hbatch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kHbSmem));
    if (e != cudaSuccess) { cudaGetLastError(); return hfail(b, TWMC_ERR_CUDA, std::string("hbatch smem: ") + cudaGetErrorString(e)); }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, hbatch_kernel, HB_CTA, kHbSmem);
    b->grid = std::max(1, std::min(b->nitems, prop.multiProcessorCount * std::max(per_sm, 1)));
  }

  // capture one frame
  cudaStream_t s0 = b->s0;
  cudaStreamSynchronize(s0);
  if (cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return hfail(b, TWMC_ERR_CUDA, "stream capture failed to start");
  cudaEventRecord(b->fork, s0);
  for (cudaStream_t es : b->ell_streams) cudaStreamWaitEvent(es, b->fork, 0);
  std::string cerr;
  bool ok = true;
  {
    // longest-processing-time-first assignment of the real-space points to
    // the least loaded stream (load = trajectories x sites)
    std::vector<size_t> order;
    for (size_t i = 0; i < n; ++i) if (b->shape[i] < 0) order.push_back(i);
    std::sort(order.begin(), order.end(), [&](size_t x, size_t y) {
      return b->ntraj[x] * b->nsites[x] > b->ntraj[y] * b->nsites[y];
    });
    std::vector<double> load(b->ell_streams.size(), 0.0);
    for (size_t i : order) {
      if (!ok) break;
      const size_t k = size_t(std::min_element(load.begin(), load.end()) - load.begin());
      load[k] += double(b->ntraj[i]) * double(b->nsites[i]);
      ok = ell_launch_dev(0, b->ell_variant[i], 1, b->args.p + i, b->ell_grid[i], b->ell_smem[i],
                          b->ell_streams[k], &cerr);
    }
  }
  for (size_t k = 0; k < b->ell_streams.size(); ++k) cudaEventRecord(b->ell_joins[k], b->ell_streams[k]);
  if (b->nitems > 0) {
    cudaMemsetAsync(b->counter.p, 0, sizeof(int), s0);
    hbatch_kernel<<<b->grid, HB_CTA, kHbSmem, s0>>>(b->args.p, b->pshape.p, b->items.p, b->nitems, b->counter.p);
  }
  for (cudaEvent_t ej : b->ell_joins) cudaStreamWaitEvent(s0, ej, 0);
  dim3 mg(unsigned((b->max_sites + 127) / 128), unsigned(b->max_blocks), unsigned(n));
  hbatch_moments_kernel<<<mg, 128, 0, s0>>>(b->margs.p);
  hbatch_bump_kernel<<<unsigned((n + 127) / 128), 128, 0, s0>>>(b->args.p, int(n), uint32_t(frame_steps));
  cudaError_t ce = cudaStreamEndCapture(s0, &b->graph);
  if (!ok || ce != cudaSuccess) {
    cudaGetLastError();
    return hfail(b, TWMC_ERR_CUDA, "graph capture failed: " + (ok ? std::string(cudaGetErrorString(ce)) : cerr));
  }
  ce = cudaGraphInstantiate(&b->exec, b->graph, 0);
  if (ce != cudaSuccess) { cudaGetLastError(); return hfail(b, TWMC_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce)); }
  return TWMC_OK;
}

int twmc_hbatch_run(twmc_hbatch* b, int64_t n_frames) {
  if (!b || !b->exec || n_frames < 0) return TWMC_ERR_INVALID;
  cudaSetDevice(b->device);
  cudaEventRecord(b->e0, b->s0);
  for (int64_t f = 0; f < n_frames; ++f) {
    cudaError_t e = cudaGraphLaunch(b->exec, b->s0);
    if (e != cudaSuccess) return hfail(b, TWMC_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(e));
    ++b->launches;
  }
  cudaEventRecord(b->e1, b->s0);
  b->frames_run += n_frames;
  return TWMC_OK;
}

int twmc_hbatch_sync(twmc_hbatch* b, double* ms) {
  if (!b) return TWMC_ERR_INVALID;
  cudaSetDevice(b->device);
  cudaError_t e = cudaStreamSynchronize(b->s0);
  if (e != cudaSuccess) return hfail(b, TWMC_ERR_CUDA, std::string("sync: ") + cudaGetErrorString(e));
  if (ms) {
    float x = 0;
    *ms = cudaEventElapsedTime(&x, b->e0, b->e1) == cudaSuccess ? double(x) : 0.0;
  }
  return TWMC_OK;
}

int twmc_hbatch_moments(twmc_hbatch* b, size_t point, double* out) {
  if (!b || !out || point >= b->npts) return TWMC_ERR_INVALID;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->s0);
  const size_t cnt = size_t(b->nblocks[point] * b->nsites[point] * 3);
  cudaError_t e = cudaMemcpy(out, b->moments.p + b->mom_off[point], cnt * sizeof(double), cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? TWMC_OK : hfail(b, TWMC_ERR_CUDA, cudaGetErrorString(e));
}

int twmc_hbatch_state(twmc_hbatch* b, size_t point, double* out) {
  if (!b || !out || point >= b->npts) return TWMC_ERR_INVALID;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->s0);
  const size_t cnt = size_t(b->ntraj[point] * b->nsites[point]);
  std::vector<float2> tmp(cnt);
  cudaError_t e = cudaMemcpy(tmp.data(), b->state.p + b->off_state[point], cnt * sizeof(float2), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return hfail(b, TWMC_ERR_CUDA, cudaGetErrorString(e));
  for (size_t k = 0; k < cnt; ++k) { out[2 * k] = tmp[k].x; out[2 * k + 1] = tmp[k].y; }
  return TWMC_OK;
}

int twmc_hbatch_set_init(twmc_hbatch* b, size_t point, const double* beta_init, const double* beta_sigma) {
  if (!b || point >= b->npts) return TWMC_ERR_INVALID;
  if (b->frames_run > 0) return hfail(b, TWMC_ERR_INVALID, "initial fields can only be set before the first run");
  cudaSetDevice(b->device);
  std::string e;
  if (!init_point(b, point, beta_init, beta_sigma, &e)) return hfail(b, TWMC_ERR_CUDA, e);
  return TWMC_OK;
}

int twmc_hbatch_field_moments(twmc_hbatch* b, double* mean, double* abs2, int32_t accumulate) {
  if (!b || !mean || !abs2) return TWMC_ERR_INVALID;
  cudaSetDevice(b->device);
  dim3 g(unsigned((b->max_sites + 127) / 128), unsigned(b->npts));
  hbatch_field_kernel<<<g, 128, 0, b->s0>>>(b->margs.p, b->site_off.p, mean, abs2, accumulate ? 1 : 0);
  ++b->launches;
  cudaError_t ce = cudaGetLastError();
  return ce == cudaSuccess ? TWMC_OK : hfail(b, TWMC_ERR_CUDA, cudaGetErrorString(ce));
}

int64_t twmc_hbatch_total_sites(const twmc_hbatch* b) { return b ? b->total_sites : -1; }

int twmc_hbatch_block_means(twmc_hbatch* b, double* out) {
  if (!b || !out) return TWMC_ERR_INVALID;
  cudaSetDevice(b->device);
  dim3 g(unsigned(b->max_blocks), unsigned(b->npts));
  hbatch_block_means_kernel<<<g, 128, 0, b->s0>>>(b->margs.p, b->blk_off.p, b->blk_means.p);
  ++b->launches;
  cudaError_t e = cudaMemcpyAsync(out, b->blk_means.p, size_t(b->total_blocks) * 3 * sizeof(double),
                                  cudaMemcpyDeviceToHost, b->s0);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->s0);
  return e == cudaSuccess ? TWMC_OK : hfail(b, TWMC_ERR_CUDA, cudaGetErrorString(e));
}

void* twmc_hbatch_stream(const twmc_hbatch* b) { return b ? static_cast<void*>(b->s0) : nullptr; }

const char* twmc_hbatch_plan(const twmc_hbatch* b, size_t point) {
  if (!b || point >= b->npts) return "";
  return b->plan[point].c_str();
}

const char* twmc_hbatch_last_error(const twmc_hbatch* b) { return b ? b->err.c_str() : "null batch"; }

int64_t twmc_hbatch_launch_count(const twmc_hbatch* b) { return b ? b->launches : -1; }

void twmc_hbatch_destroy(twmc_hbatch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->s0) cudaStreamSynchronize(b->s0);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (cudaEvent_t e : {b->fork, b->join, b->e0, b->e1}) if (e) cudaEventDestroy(e);
  for (size_t k = 1; k < b->ell_streams.size(); ++k) {
    if (b->ell_joins[k]) cudaEventDestroy(b->ell_joins[k]);
    if (b->ell_streams[k]) cudaStreamDestroy(b->ell_streams[k]);
  }
  if (b->s0) cudaStreamDestroy(b->s0);
  if (b->s1) cudaStreamDestroy(b->s1);
  delete b;
}

}  // extern "C"
