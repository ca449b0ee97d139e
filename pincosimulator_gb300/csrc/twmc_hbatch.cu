// twmc_hbatch.cu -- heterogeneous batch: parameter points of different
// lattice sizes advanced together, one CUDA graph per frame.
//
// Each point is a square lattice (1-D chain or 2-D) with uniform parameters
// and its own trajectories, and takes one step variant: the register FFT
// (plans of 32..1024-site chains and 16x16, 32x32, 64x64), the real-space
// stencil with 2, 4 or 8 sites per thread, row runs of four sites, or the
// 2-CTA cluster stencil above 4096 sites. Every (point, trajectory group) is
// a work item of a persistent work-queue kernel -- one per CTA geometry:
// hbatch_kernel (256 threads), hbatch_kernel_512 and hbatch_cluster_kernel
// (2-CTA clusters of 1024 threads) -- whose CTAs take items from an atomic
// counter, longest item first, and run the variant's step body for that
// point (arguments and tables reloaded into shared memory when the point
// changes). One frame -- counter reset, the three queues on parallel graph
// branches, the batched FP64 moments and the advance of every point's
// Philox step counter -- is captured once into a CUDA graph and replayed per
// frame; the per-point arguments live in device memory so the replayed graph
// needs no updates.
//
// Autotuner: for every shape, the first batch that needs it times each
// variant the shape admits (FFT plan, real-space stencil with 2 / 4 / 8
// sites per thread -- i.e. trajectories per CTA --, row runs, cluster forms)
// on a trial batch of that point alone and keeps the fastest; choices are
// cached per device and shape in a JSON file ($TWMC_TUNE_CACHE, default
// ~/.cache/twmc_tune.json).
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

// Step variants of a batch point. Each runs in one of three persistent
// work-queue kernels, by CTA geometry: 256 threads (register-FFT plans and
// real-space stencils with 2, 4 or 8 sites per thread), 512 threads (row
// runs, 8 sites per thread) and 2-CTA clusters of 1024 threads (lattices
// above 4096 sites).
enum HbVariant : int {
  kVarFft = 0, kVarEll2, kVarEll4, kVarEll8, kVarRowrun, kVarEll8w, kVarClusterPow2, kVarCluster, kVarCount
};
constexpr const char* kVarName[kVarCount] = {"fft", "ell2", "ell4", "ell8", "rowrun", "ell8w", "cluster_pow2",
                                             "cluster"};
enum HbQueue : int { kQ256 = 0, kQ512, kQCluster, kQueues };
constexpr int kVarQueue[kVarCount] = {kQ256, kQ256, kQ256, kQ256, kQ512, kQ512, kQCluster, kQCluster};
constexpr int kQueueCta[kQueues] = {256, 512, 1024};
constexpr int64_t kOneGroup = int64_t(1) << 62;  // group stride past any batch: a body runs exactly one group

// Fetches the next work item (point, trajectory group) of a queue into
// s_item; returns false when the queue is empty. Copies the point's step
// arguments into shared memory when the point changes.
__device__ __forceinline__ bool hb_next(const StepArgs* __restrict__ pts, const int2* __restrict__ items, int nitems,
                                        int* __restrict__ counter, StepArgs& s_a, int& s_item, int& cur, int2& w,
                                        bool& reload) {
  __syncthreads();  // the previous item is done with the shared arguments and buffers
  if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
  __syncthreads();
  const int it = s_item;
  if (it >= nitems) return false;
  w = items[it];
  reload = w.x != cur;
  if (reload) {
    for (int i = threadIdx.x; i < int(sizeof(StepArgs) / 4); i += blockDim.x)
      reinterpret_cast<uint32_t*>(&s_a)[i] = reinterpret_cast<const uint32_t*>(pts + w.x)[i];
    __syncthreads();
    cur = w.x;
  }
  return true;
}

// 256-thread queue: register-FFT plans and real-space stencils.
__global__ void __launch_bounds__(HB_CTA, 2)
hbatch_kernel(const StepArgs* __restrict__ pts, const int* __restrict__ pvar, const int* __restrict__ pshape,
              const int2* __restrict__ items, int nitems, int* __restrict__ counter) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(16) StepArgs s_a;
  __shared__ int s_item;
  int cur = -1, buf = 0;
  int2 w;
  bool reload;
  while (hb_next(pts, items, nitems, counter, s_a, s_item, cur, w, reload)) {
    switch (pvar[w.x]) {
      case kVarFft:
        switch (pshape[w.x]) {
#define TWMC_HB_CASE(BX, BY) \
  case kShape_##BX##_##BY: hb_run<Plan_##BX##_##BY>(smem_raw, s_a, reload, w.y, buf); break;
          TWMC_HB_SHAPES(TWMC_HB_CASE)
#undef TWMC_HB_CASE
          default: break;
        }
        break;
      case kVarEll2: ell_body<float, 2, HB_CTA, 1, true>(s_a, smem_raw, w.y, kOneGroup); break;
      case kVarEll4: ell_body<float, 4, HB_CTA, 1, true>(s_a, smem_raw, w.y, kOneGroup); break;
      case kVarEll8: ell_body<float, 8, HB_CTA, 1, true>(s_a, smem_raw, w.y, kOneGroup); break;
      default: break;
    }
  }
}

// 512-thread queue: row runs of four sites and the 8-site real-space stencil.
__global__ void __launch_bounds__(512, 1)
hbatch_kernel_512(const StepArgs* __restrict__ pts, const int* __restrict__ pvar, const int2* __restrict__ items,
                  int nitems, int* __restrict__ counter) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(16) StepArgs s_a;
  __shared__ int s_item;
  int cur = -1;
  int2 w;
  bool reload;
  while (hb_next(pts, items, nitems, counter, s_a, s_item, cur, w, reload)) {
    if (pvar[w.x] == kVarRowrun) rowrun_body<512>(s_a, smem_raw, w.y, kOneGroup);
    else ell_body<float, 8, 512, 1, true>(s_a, smem_raw, w.y, kOneGroup);
  }
}

// Cluster queue: one item is one trajectory, run by both CTAs of a 2-CTA
// cluster; rank 0 takes the item and rank 1 reads it through distributed
// shared memory, so both ranks leave the loop together.
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(1024, 1)
hbatch_cluster_kernel(const StepArgs* __restrict__ pts, const int* __restrict__ pvar,
                      const int2* __restrict__ items, int nitems, int* __restrict__ counter) {
  namespace cg = cooperative_groups;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(16) StepArgs s_a;
  __shared__ int s_item;
  cg::cluster_group cl = cg::this_cluster();
  const unsigned rank = cl.block_rank();
  int cur = -1;
  for (;;) {
    cl.sync();  // both ranks are done with the previous item (buffers, peer reads, s_item)
    if (rank == 0 && threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    cl.sync();
    const int it = rank == 0 ? s_item : *cl.map_shared_rank(&s_item, 0);
    if (it >= nitems) break;
    const int2 w = items[it];
    if (w.x != cur) {
      __syncthreads();
      for (int i = threadIdx.x; i < int(sizeof(StepArgs) / 4); i += 1024)
        reinterpret_cast<uint32_t*>(&s_a)[i] = reinterpret_cast<const uint32_t*>(pts + w.x)[i];
      __syncthreads();
      cur = w.x;
    }
    if (pvar[w.x] == kVarClusterPow2) ell_cluster_pow2_body<1024, true>(s_a, smem_raw, w.y, kOneGroup);
    else ell_cluster_body<float, 1024>(s_a, smem_raw, w.y, kOneGroup);
  }
  cl.sync();  // rank 0's shared memory stays until rank 1 has read the last item index
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

// cache: one line per entry: "<device>|<nx>x<ny>": "<variant name>"
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

struct twmc_hbatch {
  int device = 0;
  cudaStream_t s0 = nullptr;
  // the 512-thread and cluster queues run on their own captured streams,
  // parallel graph branches beside the 256-thread queue on s0
  cudaStream_t sq[kQueues] = {nullptr, nullptr, nullptr};
  cudaEvent_t fork = nullptr, e0 = nullptr, e1 = nullptr;
  cudaEvent_t qjoin[kQueues] = {nullptr, nullptr, nullptr};
  std::string err;
  int64_t frame_steps = 1;
  size_t npts = 0;
  std::vector<twmc_point_desc> desc;
  std::vector<int> var;            // step variant (HbVariant) per point
  std::vector<int> shape;          // register-FFT plan id per point (kVarFft), else -1
  std::vector<std::string> plan;
  std::vector<int64_t> nsites, ntraj, off_state, nblocks;
  DBuf<float2> state;
  DBuf<float> nk;
  DBuf<uint32_t> seeds, ids;
  DBuf<int> status;
  DBuf<float2> tw;
  DBuf<float> kt;
  DBuf<StepArgs> args;
  DBuf<int> pvar, pshape;
  DBuf<int2> qitems[kQueues];
  int qn[kQueues] = {0, 0, 0}, qgrid[kQueues] = {0, 0, 0};
  size_t qsmem[kQueues] = {0, 0, 0};
  DBuf<int> counter;               // one work counter per queue
  DBuf<MomentArgs> margs;
  DBuf<double> moments;
  std::vector<int64_t> mom_off;
  std::vector<int64_t> traj_off;   // first trajectory of each point in seeds / ids / status
  DBuf<int64_t> site_off;          // first site of each point in the per-site outputs
  int64_t total_sites = 0;
  DBuf<int64_t> blk_off;           // first moment block of each point in the block-mean output
  DBuf<double> blk_means;
  int64_t total_blocks = 0;
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


// Whether variant v can run point d (N = nx ny sites, all FP32 fast runs:
// Philox noise, uniform parameters).
bool var_ok(int v, const twmc_point_desc& d) {
  const int64_t n = d.nx * d.ny, half = (n + 1) / 2;
  const int bx = lg2(d.nx), by = lg2(d.ny);
  switch (v) {
    case kVarFft: return bx >= 0 && by >= 0 && hb_shape_id(bx, by) >= 0;
    case kVarEll2: return (half + 0) / 1 <= HB_CTA;
    case kVarEll4: return (half + 1) / 2 <= HB_CTA;
    case kVarEll8: return (half + 3) / 4 <= HB_CTA;
    case kVarRowrun: return n <= 4096 && n % 8 == 0 && d.ny % 4 == 0;
    case kVarEll8w: return (half + 3) / 4 <= 512;
    case kVarClusterPow2:
      return n > 4096 && n <= 16384 && (n & (n - 1)) == 0 && d.ny >= 2 && (d.ny & (d.ny - 1)) == 0 && d.ny <= n / 4;
    case kVarCluster: return n > 4096 && n <= 16384;
    default: return false;
  }
}

// Threads per trajectory of the real-space variants, and trajectories per
// work item of every variant.
int var_tpt(int v, int64_t n) {
  const int64_t half = (n + 1) / 2;
  switch (v) {
    case kVarEll2: return int(half);
    case kVarEll4: return int((half + 1) / 2);
    case kVarEll8: case kVarEll8w: return int((half + 3) / 4);
    case kVarRowrun: return int(n / 8);
    default: return 0;
  }
}
int var_tpc(int v, const twmc_point_desc& d, int shape) {
  if (v == kVarFft) return hb_tpc(shape);
  if (v == kVarClusterPow2 || v == kVarCluster) return 1;
  return kQueueCta[kVarQueue[v]] / var_tpt(v, d.nx * d.ny);
}
// Dynamic shared memory of one item of variant v.
size_t var_smem(int v, const twmc_point_desc& d, int shape) {
  const int64_t n = d.nx * d.ny;
  if (v == kVarFft) return kHbSmem;
  if (v == kVarClusterPow2 || v == kVarCluster) {
    const int64_t half = (n + 1) / 2, q = (half + 1) / 2;
    return sizeof(float2) * 4 * size_t(q);
  }
  return ell_state_bytes(true, var_tpc(v, d, shape), n, sizeof(float2));
}

// The variant a point takes without tuning: the register FFT where a plan
// exists; else, up to 4096 sites, row runs on 4096-site lattices and
// otherwise the real-space stencil with the fewest idle site slots; above
// 4096 sites the cluster stencil (power-of-two geometry where it applies).
int default_var(const twmc_point_desc& d) {
  if (var_ok(kVarFft, d)) return kVarFft;
  const int64_t n = d.nx * d.ny;
  if (n > 4096) return var_ok(kVarClusterPow2, d) ? kVarClusterPow2 : kVarCluster;
  if (n == 4096 && var_ok(kVarRowrun, d)) return kVarRowrun;
  int best = kVarEll8w;
  double best_u = -1.0;
  for (int v : {kVarEll2, kVarEll4, kVarEll8, kVarEll8w}) {
    if (!var_ok(v, d)) continue;
    const int vpt = v == kVarEll2 ? 2 : v == kVarEll4 ? 4 : 8;
    const int cta = kQueueCta[kVarQueue[v]];
    const int64_t tpc = cta / var_tpt(v, n);
    const double u = double(n * tpc) / double(int64_t(cta) * vpt);
    if (u > best_u + 1e-9) { best_u = u; best = v; }
  }
  return best;
}

int hb_build(twmc_hbatch* b, const twmc_point_desc* points, size_t n, int64_t frame_steps, const int* forced,
             int32_t tune);

// Site-updates per second of variant v on point d alone: a trial batch of
// the point (at most 2048 trajectories), one untimed 50-step frame, then two
// timed frames.
double trial_rate(const twmc_point_desc& d, int v) {
  twmc_point_desc t = d;
  t.n_traj = std::min<int64_t>(std::max<int64_t>(d.n_traj, 256), 2048);
  t.n_moment_blocks = 1;
  twmc_hbatch* tb = new (std::nothrow) twmc_hbatch();
  if (!tb) return 0.0;
  double rate = 0.0;
  double ms = 0.0;
  if (hb_build(tb, &t, 1, 50, &v, 0) == TWMC_OK && twmc_hbatch_run(tb, 1) == TWMC_OK &&
      twmc_hbatch_sync(tb, nullptr) == TWMC_OK && twmc_hbatch_run(tb, 2) == TWMC_OK &&
      twmc_hbatch_sync(tb, &ms) == TWMC_OK && ms > 0)
    rate = double(t.n_traj) * 100.0 * double(t.nx * t.ny) / (ms * 1e-3);
  twmc_hbatch_destroy(tb);
  return rate;
}

int hb_build(twmc_hbatch* b, const twmc_point_desc* points, size_t n, int64_t frame_steps, const int* forced,
             int32_t tune) {
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
    if (d.n_traj > (int64_t(1) << 30)) return hfail(b, TWMC_ERR_INVALID, "point " + std::to_string(i) + ": too many trajectories");
  }
  cudaStreamCreateWithFlags(&b->s0, cudaStreamNonBlocking);
  cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  for (int q = 0; q < kQueues; ++q) {
    cudaStreamCreateWithFlags(&b->sq[q], cudaStreamNonBlocking);
    cudaEventCreateWithFlags(&b->qjoin[q], cudaEventDisableTiming);
  }
  cudaEventCreate(&b->e0);
  cudaEventCreate(&b->e1);
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, b->device);
  const std::string devname = prop.name;

  // step variant per point: forced, tuned (per shape, cached) or the default
  b->var.assign(n, -1);
  b->shape.assign(n, -1);
  b->plan.assign(n, "");
  std::map<std::string, std::string> cache;
  const std::string cpath = tune_cache_path();
  if (tune) cache = read_cache(cpath);
  bool cache_dirty = false;
  for (size_t i = 0; i < n; ++i) {
    const twmc_point_desc& d = points[i];
    int v = forced ? forced[i] : default_var(d);
    if (!forced && tune) {
      const std::string key = devname + "|" + std::to_string(d.nx) + "x" + std::to_string(d.ny);
      std::lock_guard<std::mutex> lock(g_tune_mu);
      auto it = cache.find(key);
      int cached = -1;
      if (it != cache.end())
        for (int k = 0; k < kVarCount; ++k) if (it->second == kVarName[k] && var_ok(k, d)) cached = k;
      if (cached >= 0) {
        v = cached;
      } else {
        double best = -1.0;
        for (int k = 0; k < kVarCount; ++k) {
          if (!var_ok(k, d)) continue;
          const double r = trial_rate(d, k);
          if (r > best) { best = r; v = k; }
        }
        cache[key] = kVarName[v];
        cache_dirty = true;
      }
    }
    if (v < 0 || v >= kVarCount || !var_ok(v, d))
      return hfail(b, TWMC_ERR_INVALID, "point " + std::to_string(i) + ": no step variant for this lattice");
    b->var[i] = v;
    if (v == kVarFft) b->shape[i] = hb_shape_id(lg2(d.nx), lg2(d.ny));
    static const char* qname[kQueues] = {"hbatch_kernel", "hbatch_kernel_512", "hbatch_cluster_kernel"};
    b->plan[i] = std::string(qname[kVarQueue[v]]) + "<" + kVarName[v] + " " + std::to_string(d.nx) + "x" +
                 std::to_string(d.ny) + ">";
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
  if (!b->tw.alloc(tw.size()) || !b->kt.alloc(kt.size()) || !b->args.alloc(n) || !b->pvar.alloc(n) ||
      !b->pshape.alloc(n) || !b->counter.alloc(kQueues) || !b->margs.alloc(n))
    return hfail(b, TWMC_ERR_NOMEM, "device allocation failed");
  cudaMemcpy(b->tw.p, tw.data(), tw.size() * sizeof(float2), cudaMemcpyHostToDevice);
  cudaMemcpy(b->kt.p, kt.data(), kt.size() * sizeof(float), cudaMemcpyHostToDevice);
  cudaMemcpy(b->seeds.p, hseeds.data(), hseeds.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(b->ids.p, hids.data(), hids.size() * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(b->pvar.p, b->var.data(), n * sizeof(int), cudaMemcpyHostToDevice);
  cudaMemcpy(b->pshape.p, b->shape.data(), n * sizeof(int), cudaMemcpyHostToDevice);
  // arguments, work items (longest item first in every queue), moment args
  std::vector<StepArgs> hargs(n);
  std::vector<MomentArgs> hm(n);
  std::vector<std::pair<double, size_t>> order[kQueues];
  for (size_t i = 0; i < n; ++i) {
    StepArgs& a = hargs[i];
    fill_args(b, i, &a);
    const int v = b->var[i];
    a.state = b->state.p + b->off_state[i];
    a.seeds = b->seeds.p + traj_off[i];
    a.ids = b->ids.p + traj_off[i];
    a.status = b->status.p + traj_off[i];
    a.nk = v == kVarFft ? b->nk.p + b->off_state[i] : nullptr;  // k-space populations from the FFT only
    a.tw = b->tw.p + tw_off[i];
    a.ktab = b->kt.p + tw_off[i];
    a.tpt = var_tpt(v, b->nsites[i]);
    a.dbuf = 1;
    const int q = kVarQueue[v];
    const int tpc = var_tpc(v, points[i], b->shape[i]);
    order[q].push_back({double(b->nsites[i]) * double(tpc), i});
    b->qsmem[q] = std::max(b->qsmem[q], var_smem(v, points[i], b->shape[i]));
    MomentArgs& m = hm[i];
    m.ntraj = b->ntraj[i];
    m.nsites = b->nsites[i];
    m.prec = 0;
    m.state = a.state;
    m.nk = a.nk;
    m.nblocks = int(b->nblocks[i]);
    m.out = b->moments.p + b->mom_off[i];
  }
  for (int q = 0; q < kQueues; ++q) {
    std::stable_sort(order[q].begin(), order[q].end(),
                     [](const std::pair<double, size_t>& x, const std::pair<double, size_t>& y) { return x.first > y.first; });
    std::vector<int2> items;
    for (const auto& o : order[q]) {
      const size_t i = o.second;
      const int tpc = var_tpc(b->var[i], points[i], b->shape[i]);
      for (int64_t g = 0; g < (b->ntraj[i] + tpc - 1) / tpc; ++g) items.push_back(make_int2(int(i), int(g)));
    }
    b->qn[q] = int(items.size());
    if (!b->qitems[q].alloc(std::max<size_t>(items.size(), 1))) return hfail(b, TWMC_ERR_NOMEM, "device allocation failed");
    if (!items.empty()) cudaMemcpy(b->qitems[q].p, items.data(), items.size() * sizeof(int2), cudaMemcpyHostToDevice);
  }
  cudaMemcpy(b->args.p, hargs.data(), n * sizeof(StepArgs), cudaMemcpyHostToDevice);
  cudaMemcpy(b->margs.p, hm.data(), n * sizeof(MomentArgs), cudaMemcpyHostToDevice);

  // initial fields (ReadFromSettings with uniform beta_init / sigma)
  for (size_t i = 0; i < n; ++i) {
    std::string e;
    if (!init_point(b, i, nullptr, nullptr, &e)) return hfail(b, TWMC_ERR_CUDA, e);
  }

  // persistent grids: every resident CTA (cluster) of the device, at most one per item
  int maxsm = 0;
  cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, b->device);
  const void* qfn[kQueues] = {reinterpret_cast<const void*>(hbatch_kernel),
                              reinterpret_cast<const void*>(hbatch_kernel_512),
                              reinterpret_cast<const void*>(hbatch_cluster_kernel)};
  for (int q = 0; q < kQueues; ++q) {
    if (b->qn[q] == 0) continue;
    const size_t smem = b->qsmem[q];
    if (smem + sizeof(StepArgs) + 64 > size_t(maxsm)) return hfail(b, TWMC_ERR_INVALID, "batch queue: field does not fit");
    cudaError_t e = cudaFuncSetAttribute(qfn[q], cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) { cudaGetLastError(); return hfail(b, TWMC_ERR_CUDA, std::string("batch queue smem: ") + cudaGetErrorString(e)); }
    int slots = 0;
    if (q == kQCluster) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(2, 1, 1);
      cfg.blockDim = dim3(1024, 1, 1);
      cfg.dynamicSmemBytes = smem;
      int ncl = 0;
      e = cudaOccupancyMaxActiveClusters(&ncl, qfn[q], &cfg);
      if (e != cudaSuccess || ncl <= 0) { cudaGetLastError(); return hfail(b, TWMC_ERR_CUDA, "batch cluster queue does not fit"); }
      b->qgrid[q] = 2 * std::min(b->qn[q], ncl);
    } else {
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&slots, qfn[q], kQueueCta[q], smem);
      if (e != cudaSuccess || slots <= 0) { cudaGetLastError(); return hfail(b, TWMC_ERR_CUDA, "batch queue does not fit on an SM"); }
      b->qgrid[q] = std::max(1, std::min(b->qn[q], prop.multiProcessorCount * slots));
    }
  }

  // capture one frame: counters reset, the three queues on parallel
  // branches, then the batched moments and the step-counter bump
  cudaStream_t s0 = b->s0;
  cudaStreamSynchronize(s0);
  if (cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return hfail(b, TWMC_ERR_CUDA, "stream capture failed to start");
  cudaMemsetAsync(b->counter.p, 0, kQueues * sizeof(int), s0);
  cudaEventRecord(b->fork, s0);
  for (int q = 0; q < kQueues; ++q) cudaStreamWaitEvent(b->sq[q], b->fork, 0);
  if (b->qn[kQ256] > 0)
    hbatch_kernel<<<b->qgrid[kQ256], HB_CTA, b->qsmem[kQ256], b->sq[kQ256]>>>(
        b->args.p, b->pvar.p, b->pshape.p, b->qitems[kQ256].p, b->qn[kQ256], b->counter.p + kQ256);
  if (b->qn[kQ512] > 0)
    hbatch_kernel_512<<<b->qgrid[kQ512], 512, b->qsmem[kQ512], b->sq[kQ512]>>>(
        b->args.p, b->pvar.p, b->qitems[kQ512].p, b->qn[kQ512], b->counter.p + kQ512);
  if (b->qn[kQCluster] > 0)
    hbatch_cluster_kernel<<<b->qgrid[kQCluster], 1024, b->qsmem[kQCluster], b->sq[kQCluster]>>>(
        b->args.p, b->pvar.p, b->qitems[kQCluster].p, b->qn[kQCluster], b->counter.p + kQCluster);
  cudaError_t le = cudaGetLastError();
  for (int q = 0; q < kQueues; ++q) {
    cudaEventRecord(b->qjoin[q], b->sq[q]);
    cudaStreamWaitEvent(s0, b->qjoin[q], 0);
  }
  dim3 mg(unsigned((b->max_sites + 127) / 128), unsigned(b->max_blocks), unsigned(n));
  hbatch_moments_kernel<<<mg, 128, 0, s0>>>(b->margs.p);
  hbatch_bump_kernel<<<unsigned((n + 127) / 128), 128, 0, s0>>>(b->args.p, int(n), uint32_t(frame_steps));
  cudaError_t ce = cudaStreamEndCapture(s0, &b->graph);
  if (le != cudaSuccess || ce != cudaSuccess) {
    cudaGetLastError();
    return hfail(b, TWMC_ERR_CUDA, "graph capture failed: " + std::string(cudaGetErrorString(le != cudaSuccess ? le : ce)));
  }
  ce = cudaGraphInstantiate(&b->exec, b->graph, 0);
  if (ce != cudaSuccess) { cudaGetLastError(); return hfail(b, TWMC_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce)); }
  return TWMC_OK;
}

}  // namespace

extern "C" {

int twmc_hbatch_create(const twmc_point_desc* points, size_t n, int64_t frame_steps, int32_t tune, twmc_hbatch** out) {
  if (!out) return TWMC_ERR_INVALID;
  *out = nullptr;
  twmc_hbatch* b = new (std::nothrow) twmc_hbatch();
  if (!b) return TWMC_ERR_NOMEM;
  *out = b;
  return hb_build(b, points, n, frame_steps, nullptr, tune);
}

int twmc_hbatch_create_variants(const twmc_point_desc* points, size_t n, int64_t frame_steps,
                                const char* const* variants, twmc_hbatch** out) {
  if (!out) return TWMC_ERR_INVALID;
  *out = nullptr;
  twmc_hbatch* b = new (std::nothrow) twmc_hbatch();
  if (!b) return TWMC_ERR_NOMEM;
  *out = b;
  if (!points || !variants || n == 0) return hfail(b, TWMC_ERR_INVALID, "no points");
  std::vector<int> forced(n, -1);
  for (size_t i = 0; i < n; ++i) {
    for (int k = 0; k < kVarCount; ++k)
      if (variants[i] && std::strcmp(variants[i], kVarName[k]) == 0) forced[i] = k;
    if (forced[i] < 0) return hfail(b, TWMC_ERR_INVALID, "point " + std::to_string(i) + ": unknown step variant");
  }
  return hb_build(b, points, n, frame_steps, forced.data(), 0);
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
  for (cudaEvent_t e : {b->fork, b->e0, b->e1}) if (e) cudaEventDestroy(e);
  for (int q = 0; q < kQueues; ++q) {
    if (b->qjoin[q]) cudaEventDestroy(b->qjoin[q]);
    if (b->sq[q]) cudaStreamDestroy(b->sq[q]);
  }
  if (b->s0) cudaStreamDestroy(b->s0);
  delete b;
}

}  // extern "C"
