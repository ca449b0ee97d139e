// twmc_api.cu -- host side of libtwmc_cuda.so: the C ABI declared in
// include/twmc.h. Builds the solver tables (TWMCBaseSolver::Setup /
// TWMCLiebSolver::Setup of the reference), replays the reference's step and
// frame loop on the host to fix the step count and save points
// (TWMCBaseSolver.cpp:215-274), and drives the step kernels on one stream.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <limits>
#include <map>
#include <new>
#include <string>
#include <tuple>
#include <vector>

#include "twmc.h"
#include "fft_plans.inc"
#include "twmc_kernels.cuh"
#include "twmc_launch.h"

using cd = std::complex<double>;

namespace twmc {

template <class P>
static void fill_view(PlanView* v) {
  v->nbits = P::nbits; v->bx = P::bx; v->by = P::by; v->e = P::e; v->npass = P::npass; v->nthr = P::nthr;
  for (int j = 0; j < P::e; ++j) v->reg_last[j] = P::reg[P::npass - 1][j];
  for (int i = 0; i < P::nthr; ++i) v->thr_last[i] = P::thr[P::npass - 1][i];
}

bool square_plan(int bx, int by, PlanView* out) {
#define TWMC_SHAPE(BX, BY) if (bx == BX && by == BY) { fill_view<Plan_##BX##_##BY>(out); return true; }
  TWMC_SHAPE(0, 5) TWMC_SHAPE(0, 6) TWMC_SHAPE(0, 7) TWMC_SHAPE(0, 8) TWMC_SHAPE(0, 9) TWMC_SHAPE(0, 10)
  TWMC_SHAPE(0, 11) TWMC_SHAPE(0, 12) TWMC_SHAPE(4, 4) TWMC_SHAPE(5, 5) TWMC_SHAPE(6, 6)
#undef TWMC_SHAPE
  return false;
}

}  // namespace twmc

using namespace twmc;

namespace {

struct Matrix {
  std::vector<cd> base;   // n_sites
  std::vector<cd> amp;    // n_sites (noise amplitudes)
  int kind = TWMC_DISORDER_NONE;
  bool uniform() const {
    if (kind != TWMC_DISORDER_NONE) return false;
    for (const cd& v : base) if (v != base[0]) return false;
    return true;
  }
};

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  ~DevBuf() { if (p) cudaFree(p); }
  bool ensure(size_t n) {
    if (n <= bytes && p) return true;
    if (p) cudaFree(p);
    p = nullptr; bytes = 0;
    if (n == 0) return true;
    if (cudaMalloc(&p, n) != cudaSuccess) { cudaGetLastError(); return false; }
    bytes = n;
    return true;
  }
  template <typename T> T* as() const { return reinterpret_cast<T*>(p); }
};

int ilog2_exact(int64_t v) {
  if (v <= 0 || (v & (v - 1))) return -1;
  int b = 0;
  while ((int64_t(1) << b) < v) ++b;
  return b;
}

}  // namespace

struct twmc_handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  // system
  int lattice = 0, prec = 0, noise_mode = 0, hop_mode = 0, pbc = 0;
  int64_t nx = 0, ny = 0, nsites = 0, frame_steps = 1;
  double J = 0, J_AB = 0, J_BC = 0, gamma = 0, detuning = 0, dt = 0;
  int nblocks = 32;
  Matrix m_omega, m_U, m_F, m_binit, m_bsigma;
  // F(t)
  bool timedep = false;
  bool thermo = false;     // work / area accumulators (TWMCThermoSolver)
  int integrator = TWMC_INTEGRATOR_EULER;
  // every trajectory's per-site rsl has the real part par_scalar[0][0]
  // (square lattice: Im omega uniform over the base, the disorder and any
  // given realisations); set by the batch initialisation
  bool rsl_re_uniform = false;
  DevBuf d_work, d_area;
  DevBuf d_wide;           // FP32 -> FP64 download staging (bounded chunk)
  // final-field pipeline of twmc_run: the last steps run in kFinalChunks
  // trajectory ranges; each range is widened into d_snap and copied to the
  // host on dl_stream while the next range computes
  cudaStream_t dl_stream = nullptr;
  std::vector<cudaEvent_t> dl_ev;
  cudaEvent_t snap_ready = nullptr, snap_free = nullptr;  // d_snap written (stream) / read (dl_stream)
  DevBuf d_snap;
  // page-locked host staging for fields copied row by row to the caller
  double* h_stage = nullptr;
  size_t h_stage_bytes = 0;
  std::vector<double> ft_times;   // with sentinel
  std::vector<cd> ft_vals, ft_slopes;
  // kernel selection
  bool use_fft = false;
  int bx = 0, by = 0;
  std::string kname;
  // device tables
  DevBuf d_tw, d_ktab, d_kfac, d_nbr_idx, d_nbr_w, d_ft_vals, d_ft_slopes, d_ft_id, d_ft_dt, d_ft_dt_f;
  DevBuf d_shared_par[3];  // shared per-site rsl / iU / iF when not per-trajectory
  // batch
  int64_t ntraj = 0;
  DevBuf d_state, d_par[3], d_seeds, d_ids, d_nk, d_moments, d_status, d_noise;
  DevBuf d_given, d_given_real[3], d_binit, d_bsigma, d_base[3], d_amp[3], d_real_out[3];
  bool par_per_traj[3] = {false, false, false};
  bool par_shared[3] = {false, false, false};
  double par_scalar[3][2] = {{0, 0}, {0, 0}, {0, 0}};
  uint32_t step_pos = 0;          // global step index of the batch
  int64_t noise_steps = 0;
  std::vector<double> noise_host;  // deterministic noise buffer (complex, interleaved)
  bool noise_set = false;
  // timing / counters
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pending;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_free;
  int64_t launches = 0;
  double carry_ms = 0.0;  // step-kernel device time of the last twmc_run, not yet reported
  double progress = 0.0;
  LaunchInfo last_info;
};

namespace {

int fail(twmc_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

int cuda_fail(twmc_handle* h, cudaError_t e, const char* what) {
  return fail(h, TWMC_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define TWMC_CUDA(h, call)                                   \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return cuda_fail(h, e_, #call);   \
  } while (0)

void read_matrix(const twmc_matrix& src, int64_t n, Matrix* m) {
  m->base.assign(size_t(n), cd(0, 0));
  m->amp.assign(size_t(n), cd(0, 0));
  if (src.base) for (int64_t i = 0; i < n; ++i) m->base[size_t(i)] = cd(src.base[2 * i], src.base[2 * i + 1]);
  m->kind = src.noise_kind;
  if (m->kind != TWMC_DISORDER_NONE && src.noise_amp)
    for (int64_t i = 0; i < n; ++i) m->amp[size_t(i)] = cd(src.noise_amp[2 * i], src.noise_amp[2 * i + 1]);
}

size_t rsize(int prec) { return prec ? sizeof(double) : sizeof(float); }

// Upload complex values in the state precision.
bool upload_c(DevBuf* b, const std::vector<cd>& v, int prec) {
  const size_t n = v.size();
  if (!b->ensure(n * 2 * rsize(prec))) return false;
  if (prec) {
    return cudaMemcpy(b->p, v.data(), n * sizeof(cd), cudaMemcpyHostToDevice) == cudaSuccess;
  }
  std::vector<float> f(2 * n);
  for (size_t i = 0; i < n; ++i) { f[2 * i] = float(v[i].real()); f[2 * i + 1] = float(v[i].imag()); }
  return cudaMemcpy(b->p, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess;
}

bool upload_r(DevBuf* b, const std::vector<double>& v, int prec) {
  if (!b->ensure(v.size() * rsize(prec))) return false;
  if (prec) return cudaMemcpy(b->p, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess;
  std::vector<float> f(v.begin(), v.end());
  return cudaMemcpy(b->p, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess;
}

template <typename T>
bool upload_raw(DevBuf* b, const T* data, size_t n) {
  if (!b->ensure(n * sizeof(T))) return false;
  return cudaMemcpy(b->p, data, n * sizeof(T), cudaMemcpyHostToDevice) == cudaSuccess;
}

// NoisyMatrix::SetTemporalValue (NoisyMatrix.cpp:164-250).
void build_time_table(twmc_handle* h, const double* times, const double* vals, int64_t nrec) {
  const int64_t n = h->nsites;
  std::vector<cd> m(size_t(nrec * n));
  for (int64_t i = 0; i < nrec * n; ++i) m[size_t(i)] = cd(vals[2 * i], vals[2 * i + 1]);
  std::vector<double> tt(times, times + nrec);
  for (int64_t s = 0; s < n; ++s) {
    for (int64_t pt = 0; pt < nrec; ++pt) {
      const cd v = m[size_t(pt * n + s)];
      if (!(std::isnan(v.real()) || std::isnan(v.imag()))) continue;
      cd prev(NAN, NAN), next(NAN, NAN);
      int64_t tp = pt - 1;
      for (; tp >= 0 && std::isnan(prev.real()); --tp) prev = m[size_t(tp * n + s)];
      ++tp;
      int64_t tn = pt + 1;
      for (; tn < nrec && std::isnan(next.real()); ++tn) next = m[size_t(tn * n + s)];
      --tn;
      if (std::isnan(prev.real()) && std::isnan(next.real())) break;
      if (std::isnan(next.real())) m[size_t(pt * n + s)] = prev;
      else if (std::isnan(prev.real())) m[size_t(pt * n + s)] = next;
      else m[size_t(pt * n + s)] = prev + (next - prev) / (tt[size_t(tn)] - tt[size_t(tp)]) * (tt[size_t(pt)] - tt[size_t(tp)]);
    }
  }
  h->ft_vals.assign(size_t((nrec + 1) * n), cd(0, 0));
  h->ft_slopes.assign(size_t((nrec + 1) * n), cd(0, 0));
  for (int64_t i = 0; i < nrec * n; ++i) h->ft_vals[size_t(i)] = m[size_t(i)];
  for (int64_t s = 0; s < n; ++s) h->ft_vals[size_t(nrec * n + s)] = m[size_t((nrec - 1) * n + s)];
  for (int64_t i = 1; i < nrec; ++i)
    for (int64_t s = 0; s < n; ++s)
      h->ft_slopes[size_t((i - 1) * n + s)] =
          (m[size_t(i * n + s)] - m[size_t((i - 1) * n + s)]) / (tt[size_t(i)] - tt[size_t(i - 1)]);
  tt.push_back(std::numeric_limits<double>::max());
  h->ft_times = tt;
}

// GetAtTimeWithSuggestion's segment choice (NoisyMatrix.cpp:252-265).
// Returns id and the offset t - t_id (0 when t <= t_0, where F = F_0).
std::pair<int, double> time_segment(const std::vector<double>& times, double t, int64_t hint) {
  if (t <= times[0]) return {0, 0.0};
  int64_t id;
  if (hint >= 0 && hint + 1 < int64_t(times.size()) && times[size_t(hint + 1)] > t) id = hint;
  else id = int64_t(std::lower_bound(times.begin(), times.end(), t) - times.begin()) - 1;
  return {int(id), t - times[size_t(id)]};
}

struct Schedule {
  int64_t n_frames = 0;            // frames the task asks for (incl. initial)
  int64_t steps = 0;               // loop iterations executed
  double t_final = 0;
  int64_t frames_written = 0;
  std::vector<int64_t> save_steps; // step counts after which a frame is saved (excl. initial)
  std::vector<double> step_t;      // pre-step t of every step (for F(t))
};

// The reference's time loop (TWMCBaseSolver.cpp:215-274 with
// TWMCSystemData::ComputeNFrames, TWMCSystemData.cpp:117-134).
Schedule make_schedule(double t_start, double t_end, double dt, int64_t frame_steps, bool store_initial,
                       bool keep_t) {
  Schedule s;
  const double dt_obs = dt * double(frame_steps);
  s.n_frames = int64_t(std::nearbyint((t_end - t_start) / dt_obs)) + (store_initial ? 1 : 0);
  int64_t i_frame = 0;
  if (store_initial && s.n_frames > 0) i_frame = 1;
  double t = t_start;
  int64_t i_step = 0;
  while (t <= t_end) {
    if (keep_t) s.step_t.push_back(t);
    t += dt;
    ++i_step;
    if ((i_step % frame_steps == 0) && i_frame < s.n_frames) {
      s.save_steps.push_back(i_step);
      ++i_frame;
      if (i_frame == s.n_frames) break;
    }
  }
  s.steps = i_step;
  s.t_final = t;
  s.frames_written = i_frame;
  return s;
}

void setup_params(twmc_handle* h) {
  // which of (rsl <- omega/E, iU <- U, iF <- F) vary per trajectory / per site
  const Matrix* ms[3] = {&h->m_omega, &h->m_U, &h->m_F};
  for (int k = 0; k < 3; ++k) {
    h->par_per_traj[k] = ms[k]->kind != TWMC_DISORDER_NONE;
    h->par_shared[k] = !h->par_per_traj[k] && !ms[k]->uniform();
  }
  if (h->timedep) { h->par_per_traj[2] = false; h->par_shared[2] = false; }
  // scalar values
  const cd om = h->m_omega.base.empty() ? cd(0, 0) : h->m_omega.base[0];
  cd rsl;
  if (h->lattice == TWMC_LATTICE_SQUARE) rsl = cd(om.imag() - h->gamma / 2.0, -om.real());
  else { const cd d(h->detuning - om.real(), -om.imag()); rsl = cd(d.imag() - h->gamma / 2.0, -d.real()); }
  const cd u = h->m_U.base.empty() ? cd(0, 0) : h->m_U.base[0];
  const cd f = h->m_F.base.empty() ? cd(0, 0) : h->m_F.base[0];
  h->par_scalar[0][0] = rsl.real(); h->par_scalar[0][1] = rsl.imag();
  h->par_scalar[1][0] = -u.imag(); h->par_scalar[1][1] = u.real();
  h->par_scalar[2][0] = -f.imag(); h->par_scalar[2][1] = f.real();
}

int build_tables(twmc_handle* h) {
  const int prec = h->prec;
  if (h->use_fft) {
    const int64_t M0 = int64_t(1) << h->by, M1 = int64_t(1) << h->bx;
    std::vector<cd> tw;
    for (int64_t j = 0; j < M0; ++j) tw.push_back(std::polar(1.0, -2.0 * M_PI * double(j) / double(M0)));
    for (int64_t j = 0; j < M1; ++j) tw.push_back(std::polar(1.0, -2.0 * M_PI * double(j) / double(M1)));
    if (!upload_c(&h->d_tw, tw, prec)) return fail(h, TWMC_ERR_NOMEM, "twiddle table upload");
    // separable k-space table: [2J fy cos(2 pi ky / ny) / N for ky < M0 |
    // 2J fx cos(2 pi kx / nx) / N for kx < M1]; the kernel adds the two.
    // the FP32 kernel folds dt into the hopping term (local_update_fused)
    const double fx = (h->nx == 1) ? 0.0 : 1.0, fy = (h->ny == 1) ? 0.0 : 1.0;
    const double scale = 2.0 * h->J / double(h->nsites) * (prec == TWMC_PREC_F32 ? h->dt : 1.0);
    std::vector<double> kt;
    for (int64_t k = 0; k < M0; ++k) kt.push_back(scale * fy * std::cos(2.0 * M_PI / double(h->ny) * double(k)));
    for (int64_t k = 0; k < M1; ++k) kt.push_back(scale * fx * std::cos(2.0 * M_PI / double(h->nx) * double(k)));
    if (!upload_r(&h->d_ktab, kt, prec)) return fail(h, TWMC_ERR_NOMEM, "k table upload");
    if (h->integrator == TWMC_INTEGRATOR_SPLIT) {
      // (exp(-i theta) - 1) / N, theta = 2J (fx cos(2 pi kx / nx) + fy cos(2 pi ky / ny)) dt, at every
      // position p of the forward plan's output (frequencies bit-reversed per dimension);
      // cos(theta) - 1 as -2 sin^2(theta / 2), free of cancellation
      auto bitrev = [](int64_t v, int nb) {
        int64_t r = 0;
        for (int i = 0; i < nb; ++i) r |= ((v >> i) & 1) << (nb - 1 - i);
        return r;
      };
      std::vector<cd> kf(size_t(h->nsites));
      for (int64_t p = 0; p < h->nsites; ++p) {
        const int64_t ky = bitrev(p & (M0 - 1), h->by), kx = h->bx ? bitrev(p >> h->by, h->bx) : 0;
        const double th = 2.0 * h->J * h->dt *
                          (fx * std::cos(2.0 * M_PI / double(h->nx) * double(kx)) +
                           fy * std::cos(2.0 * M_PI / double(h->ny) * double(ky)));
        const double sh = std::sin(0.5 * th);
        kf[size_t(p)] = cd(-2.0 * sh * sh, -std::sin(th)) / double(h->nsites);
      }
      if (!upload_c(&h->d_kfac, kf, prec)) return fail(h, TWMC_ERR_NOMEM, "split-step table upload");
    }
  } else if (h->lattice == TWMC_LATTICE_LIEB) {
    // Coupling triplets of TWMCLiebSolver::Setup (TWMCLiebSolver.cpp:54-85).
    const int64_t nc = h->nsites / 3;
    std::vector<std::tuple<int64_t, int64_t, double>> trips;
    for (int64_t i = 0; i != nc; ++i) {
      trips.emplace_back(3 * i, 3 * i + 1, h->J_AB);
      trips.emplace_back(3 * i + 1, 3 * i, h->J_AB);
      trips.emplace_back(3 * i + 1, 3 * i + 2, h->J_BC);
      trips.emplace_back(3 * i + 2, 3 * i + 1, h->J_BC);
      if (i == nc - 1) {
        if (h->pbc) {
          trips.emplace_back(3 * i + 2, 1, h->J_BC);
          trips.emplace_back(1, 3 * i + 2, h->J_BC);
        }
        break;
      }
      trips.emplace_back(3 * i + 2, 3 * (i + 1) + 1, h->J_BC);
      trips.emplace_back(3 * (i + 1) + 1, 3 * i + 2, h->J_BC);
    }
    // h_c = -i sum_r beta_r C_rc: column c collects (r, -i C_rc), duplicates summed.
    std::vector<std::vector<std::pair<int64_t, double>>> col(size_t(h->nsites));
    for (const auto& tr : trips) {
      auto& lst = col[size_t(std::get<1>(tr))];
      bool merged = false;
      for (auto& e : lst) if (e.first == std::get<0>(tr)) { e.second += std::get<2>(tr); merged = true; }
      if (!merged) lst.emplace_back(std::get<0>(tr), std::get<2>(tr));
    }
    std::vector<int> idx(size_t(h->nsites * 4));
    std::vector<cd> w(size_t(h->nsites * 4), cd(0, 0));
    for (int64_t c = 0; c < h->nsites; ++c) {
      auto& lst = col[size_t(c)];
      if (lst.size() > 4) return fail(h, TWMC_ERR_INVALID, "Lieb coupling with more than 4 neighbours");
      std::sort(lst.begin(), lst.end());
      for (int j = 0; j < 4; ++j) {
        if (j < int(lst.size())) { idx[size_t(c * 4 + j)] = int(lst[size_t(j)].first); w[size_t(c * 4 + j)] = cd(0, -lst[size_t(j)].second); }
        else { idx[size_t(c * 4 + j)] = int(c); w[size_t(c * 4 + j)] = cd(0, 0); }
      }
    }
    if (!upload_raw(&h->d_nbr_idx, idx.data(), idx.size())) return fail(h, TWMC_ERR_NOMEM, "neighbour upload");
    if (!upload_c(&h->d_nbr_w, w, prec)) return fail(h, TWMC_ERR_NOMEM, "neighbour upload");
  }
  if (h->timedep) {
    std::vector<cd> iv(h->ft_vals.size()), is(h->ft_slopes.size());
    for (size_t i = 0; i < iv.size(); ++i) iv[i] = cd(0, 1) * h->ft_vals[i];
    for (size_t i = 0; i < is.size(); ++i) is[i] = cd(0, 1) * h->ft_slopes[i];
    if (!upload_c(&h->d_ft_vals, iv, prec) || !upload_c(&h->d_ft_slopes, is, prec))
      return fail(h, TWMC_ERR_NOMEM, "F(t) table upload");
  }
  // shared (non-noisy, non-uniform) per-site parameters
  for (int k = 0; k < 3; ++k) {
    if (!h->par_shared[k]) continue;
    std::vector<cd> v(size_t(h->nsites));
    for (int64_t p = 0; p < h->nsites; ++p) {
      if (k == 0) {
        const cd om = h->m_omega.base[size_t(p)];
        if (h->lattice == TWMC_LATTICE_SQUARE) v[size_t(p)] = cd(om.imag() - h->gamma / 2.0, -om.real());
        else { const cd d(h->detuning - om.real(), -om.imag()); v[size_t(p)] = cd(d.imag() - h->gamma / 2.0, -d.real()); }
      } else {
        const cd x = (k == 1 ? h->m_U : h->m_F).base[size_t(p)];
        v[size_t(p)] = cd(-x.imag(), x.real());
      }
    }
    if (!upload_c(&h->d_shared_par[k], v, prec)) return fail(h, TWMC_ERR_NOMEM, "parameter upload");
  }
  return TWMC_OK;
}

std::pair<cudaEvent_t, cudaEvent_t> get_events(twmc_handle* h) {
  if (!h->ev_free.empty()) { auto e = h->ev_free.back(); h->ev_free.pop_back(); return e; }
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  return {a, b};
}

// Advances the batch by n steps (n may be 0 to refresh the k-space buffer).
// n steps of trajectories [t0, t1) of the batch (all when t1 < 0); the
// step counter advances only when `bump` (a caller stepping the batch in
// several ranges bumps it once).
int advance(twmc_handle* h, int64_t n, bool want_nk, int64_t t0 = 0, int64_t t1 = -1, bool bump = true) {
  if (t1 < 0) t1 = h->ntraj;
  if (t1 <= t0) return TWMC_OK;
  const size_t c2 = 2 * rsize(h->prec), r1 = rsize(h->prec);
  const size_t row_c = size_t(h->nsites) * c2, row_r = size_t(h->nsites) * r1;  // bytes per trajectory
  auto at = [&](const void* base, size_t row) -> void* {
    return base ? static_cast<void*>(static_cast<char*>(const_cast<void*>(base)) + size_t(t0) * row) : nullptr;
  };
  StepArgs a;
  std::memset(&a, 0, sizeof(a));
  a.state = at(h->d_state.p, row_c);
  a.ntraj = t1 - t0;
  a.nsteps = n;
  a.step0 = h->step_pos;
  a.seeds = h->d_seeds.as<uint32_t>() + t0;
  a.ids = h->d_ids.as<uint32_t>() + t0;
  const void** par[3] = {&a.rsl, &a.iU, &a.iF};
  double* sc[3] = {a.rsl_s, a.iU_s, a.iF_s};
  bool any_traj = false;
  for (int k = 0; k < 3; ++k) {
    sc[k][0] = h->par_scalar[k][0];
    sc[k][1] = h->par_scalar[k][1];
    if (h->par_per_traj[k]) { *par[k] = h->d_par[k].p; any_traj = true; }
    else if (h->par_shared[k]) *par[k] = h->d_shared_par[k].p;
    else *par[k] = nullptr;
  }
  // per-trajectory arrays have stride N; shared arrays stride 0 (mixing: both
  // kinds are stored per trajectory in d_par when any is per trajectory)
  a.par_stride = any_traj ? h->nsites : 0;
  if (any_traj) for (int k = 0; k < 3; ++k) if (h->par_shared[k]) *par[k] = h->d_par[k].p;
  if (any_traj) for (int k = 0; k < 3; ++k) *par[k] = at(*par[k], row_c);
  a.dt = h->dt;
  a.dt4 = std::sqrt(h->gamma * h->dt / 4.0);
  for (int k = 0; k < 3; ++k) { a.f_par[2 * k] = float(sc[k][0]); a.f_par[2 * k + 1] = float(sc[k][1]); }
  a.f_dt = float(a.dt);
  a.f_dt4 = float(a.dt4);
  a.f_kn = float(-2.0 * M_LN2 * h->gamma * h->dt / 4.0);
  a.noise_mode = h->noise_mode;
  a.noise_traj_stride = h->noise_steps * h->nsites;
  a.noise = at(h->d_noise.p, size_t(a.noise_traj_stride) * c2);
  a.nk = (want_nk && h->use_fft) ? at(h->d_nk.p, row_r) : nullptr;
  a.status = h->d_status.as<int>() + t0;
  a.tw = h->d_tw.p;
  a.ktab = h->d_ktab.p;
  a.kfac = h->integrator == TWMC_INTEGRATOR_SPLIT ? h->d_kfac.p : nullptr;
  a.rsl_re_uniform = h->rsl_re_uniform ? 1 : 0;
  a.nsites = h->nsites;
  a.nx = h->lattice == TWMC_LATTICE_SQUARE ? h->nx : 1;
  a.ny = h->lattice == TWMC_LATTICE_SQUARE ? h->ny : h->nsites;
  a.hop_kind = h->lattice == TWMC_LATTICE_SQUARE ? 1 : 0;
  a.nbr_idx = h->d_nbr_idx.as<int>();
  a.nbr_w = h->d_nbr_w.p;
  a.J = h->J;
  a.f_J = float(h->J);
  a.lieb_pbc = h->pbc;
  a.lieb_jab = h->J_AB;
  a.lieb_jbc = h->J_BC;
  a.f_lieb_jab = float(h->J_AB);
  a.f_lieb_jbc = float(h->J_BC);
  if (h->timedep) {
    a.ft_vals = h->d_ft_vals.p;
    a.ft_slopes = h->d_ft_slopes.p;
    a.ft_id = h->d_ft_id.as<int>();
    a.ft_dt = h->d_ft_dt.as<double>();
    a.ft_dt_f = h->d_ft_dt_f.as<float>();
  }
  if (h->thermo) {
    a.work = at(h->d_work.p, row_r);
    a.area = at(h->d_area.p, row_r);
  }
  if (h->noise_mode == TWMC_NOISE_BUFFER && n > 0 && int64_t(h->step_pos) + n > h->noise_steps)
    return fail(h, TWMC_ERR_INVALID, "noise buffer shorter than the run");
  int nparams = 0;
  for (int k = 0; k < 3; ++k) nparams += (*par[k] != nullptr);
  auto ev = get_events(h);
  cudaEventRecord(ev.first, h->stream);
  std::string err;
  bool ok;
  if (h->use_fft) {
    ok = h->prec == 0 ? square_launch_f32(h->bx, h->by, a, nparams, h->stream, &h->last_info, &err)
                      : square_launch_f64(h->bx, h->by, a, nparams, h->stream, &h->last_info, &err);
    if (ok) h->kname = h->last_info.name;  // "square_fft_kernel<fast>" for the compiled-in common run
  } else {
    ok = ell_launch(h->prec, a, h->stream, &h->last_info, &err);
    if (ok && (std::strncmp(h->last_info.name, "ell_cluster", 11) == 0 || std::strcmp(h->last_info.name, "lieb_cell_kernel") == 0 ||
               std::strcmp(h->last_info.name, "rowrun_kernel") == 0))
      h->kname = h->last_info.name;
  }
  cudaEventRecord(ev.second, h->stream);
  h->ev_pending.push_back(ev);
  if (!ok) return fail(h, TWMC_ERR_CUDA, err);
  ++h->launches;
  if (bump) h->step_pos += uint32_t(n);
  return TWMC_OK;
}

int reduce(twmc_handle* h) {
  MomentArgs m;
  m.ntraj = h->ntraj;
  m.nsites = h->nsites;
  m.prec = h->prec;
  m.state = h->d_state.p;
  m.nk = h->use_fft ? h->d_nk.p : nullptr;
  m.nblocks = int(std::min<int64_t>(h->nblocks, std::max<int64_t>(h->ntraj, 1)));
  m.out = h->d_moments.as<double>();
  std::string err;
  if (!moments_launch(m, h->stream, &err)) return fail(h, TWMC_ERR_CUDA, err);
  ++h->launches;
  return TWMC_OK;
}

// Allocates the batch and draws initial fields / disorder on the GPU.
int batch_init(twmc_handle* h, const twmc_task_desc* tasks, size_t n) {
  const int64_t N = h->nsites;
  const int prec = h->prec;
  h->ntraj = int64_t(n);
  h->step_pos = 0;
  const size_t c2 = 2 * rsize(prec);
  if (!h->d_state.ensure(n * N * c2)) return fail(h, TWMC_ERR_NOMEM, "state allocation");
  if (h->use_fft && !h->d_nk.ensure(n * N * rsize(prec))) return fail(h, TWMC_ERR_NOMEM, "nk allocation");
  if (!h->d_moments.ensure(size_t(h->nblocks) * N * 3 * sizeof(double))) return fail(h, TWMC_ERR_NOMEM, "moments allocation");
  if (!h->d_status.ensure(n * sizeof(int))) return fail(h, TWMC_ERR_NOMEM, "status allocation");
  TWMC_CUDA(h, cudaMemsetAsync(h->d_status.p, 0, n * sizeof(int), h->stream));
  if (h->thermo) {
    if (!h->d_work.ensure(n * N * rsize(prec)) || !h->d_area.ensure(n * N * rsize(prec)))
      return fail(h, TWMC_ERR_NOMEM, "work / area allocation");
    TWMC_CUDA(h, cudaMemsetAsync(h->d_work.p, 0, n * N * rsize(prec), h->stream));
    TWMC_CUDA(h, cudaMemsetAsync(h->d_area.p, 0, n * N * rsize(prec), h->stream));
  }
  std::vector<uint32_t> seeds(n), ids(n);
  int ic = tasks[0].ic_kind;
  for (size_t i = 0; i < n; ++i) {
    seeds[i] = tasks[i].seed;
    ids[i] = uint32_t(tasks[i].id);
    if (tasks[i].ic_kind != ic) return fail(h, TWMC_ERR_INVALID, "tasks of one batch must share ic_kind");
  }
  if (!upload_raw(&h->d_seeds, seeds.data(), n) || !upload_raw(&h->d_ids, ids.data(), n))
    return fail(h, TWMC_ERR_NOMEM, "seed upload");
  InitArgs ia;
  std::memset(&ia, 0, sizeof(ia));
  ia.ntraj = int64_t(n);
  ia.nsites = N;
  ia.prec = prec;
  ia.state = h->d_state.p;
  ia.seeds = h->d_seeds.as<uint32_t>();
  ia.ids = h->d_ids.as<uint32_t>();
  ia.ic_kind = ic;
  ia.lattice = h->lattice;
  ia.gamma = h->gamma;
  ia.detuning = h->detuning;
  auto up_cd = [&](DevBuf* b, const std::vector<cd>& v) -> const double* {
    if (!upload_raw(b, reinterpret_cast<const double*>(v.data()), 2 * v.size())) return nullptr;
    return b->as<double>();
  };
  ia.binit = up_cd(&h->d_binit, h->m_binit.base);
  ia.bsigma = up_cd(&h->d_bsigma, h->m_bsigma.base);
  if (ic == TWMC_IC_GIVEN) {
    std::vector<double> g(size_t(2 * N) * n);
    for (size_t i = 0; i < n; ++i) {
      if (!tasks[i].init_field) return fail(h, TWMC_ERR_INVALID, "TWMC_IC_GIVEN task without init_field");
      std::memcpy(&g[size_t(2 * N) * i], tasks[i].init_field, sizeof(double) * size_t(2 * N));
    }
    if (!upload_raw(&h->d_given, g.data(), g.size())) return fail(h, TWMC_ERR_NOMEM, "initial field upload");
    ia.given = h->d_given.as<double>();
  }
  // Real part of rsl = Im(omega) - gamma/2 the same at every site of every
  // trajectory: Im of the base uniform, no imaginary disorder amplitude, and
  // given realisations with that imaginary part (square lattice).
  {
    bool uni = h->lattice == TWMC_LATTICE_SQUARE;
    const Matrix& mo = h->m_omega;
    const double im0 = mo.base.empty() ? 0.0 : mo.base[0].imag();
    for (const cd& v : mo.base) uni = uni && v.imag() == im0;
    if (mo.kind != TWMC_DISORDER_NONE)
      for (const cd& v : mo.amp) uni = uni && v.imag() == 0.0;
    if (tasks[0].omega_realization)
      for (size_t i = 0; i < n && uni; ++i) {
        const double* w = tasks[i].omega_realization;
        if (!w) { uni = false; break; }  // rejected below: all tasks or none
        for (int64_t j = 0; j < N && uni; ++j) uni = w[2 * j + 1] == im0;
      }
    h->rsl_re_uniform = uni;
  }
  // matrices: 0 = U, 1 = omega/E, 2 = F ; per-site parameter buffers: rsl <- omega, iU <- U, iF <- F
  const Matrix* mats[3] = {&h->m_U, &h->m_omega, &h->m_F};
  const uint32_t streams[3] = {kStreamU, kStreamOmega, kStreamF};
  for (int m = 0; m < 3; ++m) {
    ia.base[m] = up_cd(&h->d_base[m], mats[m]->base);
    ia.amp[m] = up_cd(&h->d_amp[m], mats[m]->amp);
    ia.kind[m] = mats[m]->kind;
    ia.stream[m] = streams[m];
    const double* given_ptr[3] = {tasks[0].U_realization, tasks[0].omega_realization, tasks[0].F_realization};
    if (given_ptr[m]) {
      std::vector<double> g(size_t(2 * N) * n);
      for (size_t i = 0; i < n; ++i) {
        const double* src = m == 0 ? tasks[i].U_realization : m == 1 ? tasks[i].omega_realization : tasks[i].F_realization;
        if (!src) return fail(h, TWMC_ERR_INVALID, "disorder realisations must be given for all tasks of a batch or none");
        std::memcpy(&g[size_t(2 * N) * i], src, sizeof(double) * size_t(2 * N));
      }
      if (!upload_raw(&h->d_given_real[m], g.data(), g.size())) return fail(h, TWMC_ERR_NOMEM, "realisation upload");
      ia.given_real[m] = h->d_given_real[m].as<double>();
    }
  }
  // Per-trajectory parameter arrays: needed when any matrix is noisy; then
  // every non-uniform matrix is stored per trajectory.
  bool any_traj = false;
  for (int k = 0; k < 3; ++k) any_traj |= h->par_per_traj[k];
  void** dst[3] = {&ia.rsl, &ia.iU, &ia.iF};
  for (int k = 0; k < 3; ++k) {
    const bool need = any_traj && (h->par_per_traj[k] || h->par_shared[k]);
    if (need) {
      if (!h->d_par[k].ensure(n * N * c2)) return fail(h, TWMC_ERR_NOMEM, "parameter allocation");
      *dst[k] = h->d_par[k].p;
    }
  }
  for (int m = 0; m < 3; ++m) {
    if (h->d_real_out[m].ensure(n * N * 2 * sizeof(double))) ia.real_out[m] = h->d_real_out[m].as<double>();
    else return fail(h, TWMC_ERR_NOMEM, "realisation allocation");
  }
  std::string err;
  if (!init_launch(ia, h->stream, &err)) return fail(h, TWMC_ERR_CUDA, err);
  ++h->launches;
  return TWMC_OK;
}

// Copies n real values (state precision) of a device buffer to host doubles.
int download_real(twmc_handle* h, const DevBuf& b, double* out, size_t n) {
  TWMC_CUDA(h, cudaStreamSynchronize(h->stream));
  if (h->prec == 0) {
    std::vector<float> tmp(n);
    TWMC_CUDA(h, cudaMemcpy(tmp.data(), b.p, n * sizeof(float), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; ++i) out[i] = double(tmp[i]);
  } else {
    TWMC_CUDA(h, cudaMemcpy(out, b.p, n * sizeof(double), cudaMemcpyDeviceToHost));
  }
  return TWMC_OK;
}

// The batch's field as complex128 into host memory, trajectory r at
// out + r * row_stride doubles (row_stride >= 2 N), enqueued on the handle's
// stream without a final synchronisation: with a pinned destination the copy
// overlaps whatever the caller enqueues next. FP32 state is widened on the
// GPU in chunks of whole trajectories of at most kWideChunk doubles (a
// bounded per-handle buffer), each chunk copied straight to its rows by one
// strided copy.
constexpr size_t kWideChunk = size_t(1) << 25;  // 256 MB of doubles
constexpr int kFinalChunks = 4;                  // trajectory ranges of the final-field pipeline
constexpr size_t kSnapMax = size_t(8) << 30;     // largest final field (bytes) the pipeline stages

// m device rows of `row` doubles (consecutive) to host rows `row_stride`
// doubles apart: one flat copy, one strided copy, or one copy per row when
// the pitch exceeds the device's limit.
cudaError_t copy_rows_d2h(int device, double* dst, size_t row_stride, const void* src_rows, size_t row, size_t m,
                          cudaStream_t s) {
  if (row_stride == row) return cudaMemcpyAsync(dst, src_rows, m * row * sizeof(double), cudaMemcpyDeviceToHost, s);
  int maxpitch = 0;
  cudaDeviceGetAttribute(&maxpitch, cudaDevAttrMaxPitch, device);
  if (row_stride * sizeof(double) <= size_t(maxpitch))
    return cudaMemcpy2DAsync(dst, row_stride * sizeof(double), src_rows, row * sizeof(double), row * sizeof(double), m,
                             cudaMemcpyDeviceToHost, s);
  for (size_t r = 0; r < m; ++r) {
    const cudaError_t e = cudaMemcpyAsync(dst + r * row_stride, static_cast<const double*>(src_rows) + r * row,
                                          row * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

int download_rows(twmc_handle* h, double* out, size_t row_stride) {
  const size_t rows = size_t(h->ntraj), row = size_t(2 * h->nsites);  // doubles per trajectory
  if (rows == 0) return TWMC_OK;
  auto copy_rows = [&](double* dst, const void* src_rows, size_t m) -> cudaError_t {
    return copy_rows_d2h(h->device, dst, row_stride, src_rows, row, m, h->stream);
  };
  if (h->prec) {
    TWMC_CUDA(h, copy_rows(out, h->d_state.p, rows));
    return TWMC_OK;
  }
  const size_t per = std::max<size_t>(1, std::min(rows, kWideChunk / row));  // trajectories per chunk
  if (!h->d_wide.ensure(per * row * sizeof(double))) return fail(h, TWMC_ERR_NOMEM, "download buffer allocation");
  const float* src = static_cast<const float*>(h->d_state.p);
  for (size_t r0 = 0; r0 < rows; r0 += per) {
    const size_t m = std::min(per, rows - r0);
    std::string err;
    if (!widen_launch(src + r0 * row, h->d_wide.as<double>(), int64_t(m * row), h->stream, &err))
      return fail(h, TWMC_ERR_CUDA, err);
    TWMC_CUDA(h, copy_rows(out + r0 * row_stride, h->d_wide.p, m));
  }
  return TWMC_OK;
}

// The batch's field, trajectory r to dst(r) (complex128 rows of N), through
// the handle's page-locked staging buffer: one flat copy from the GPU, then
// one host memcpy per trajectory. Frames of small runs and of any layout
// take this route: a strided copy of short rows straight into pageable
// memory cost about 1 ms per frame of 1000 x 64 sites.
template <typename Dst>
int download_scatter(twmc_handle* h, Dst dst) {
  const size_t rows = size_t(h->ntraj), row = size_t(2 * h->nsites);
  const size_t bytes = rows * row * sizeof(double);
  if (bytes > h->h_stage_bytes) {
    if (h->h_stage) cudaFreeHost(h->h_stage);
    h->h_stage = nullptr;
    h->h_stage_bytes = 0;
    TWMC_CUDA(h, cudaHostAlloc(reinterpret_cast<void**>(&h->h_stage), bytes, cudaHostAllocDefault));
    h->h_stage_bytes = bytes;
  }
  int rc = download_rows(h, h->h_stage, row);
  if (rc) return rc;
  TWMC_CUDA(h, cudaStreamSynchronize(h->stream));
  for (size_t r = 0; r < rows; ++r) std::memcpy(dst(r), h->h_stage + r * row, row * sizeof(double));
  return TWMC_OK;
}

// The batch's field as contiguous complex128 rows; returns after the copy.
int download_field(twmc_handle* h, double* out) {
  int rc = download_rows(h, out, size_t(2 * h->nsites));
  if (rc) return rc;
  TWMC_CUDA(h, cudaStreamSynchronize(h->stream));
  return TWMC_OK;
}

int validate_desc(const twmc_system_desc* d, std::string* why) {
  if (!d) { *why = "null descriptor"; return TWMC_ERR_INVALID; }
  if (d->lattice != TWMC_LATTICE_SQUARE && d->lattice != TWMC_LATTICE_LIEB) { *why = "unknown lattice"; return TWMC_ERR_INVALID; }
  if (d->nx < 1 || d->ny < 1) { *why = "nx and ny must be >= 1"; return TWMC_ERR_INVALID; }
  if (d->lattice == TWMC_LATTICE_LIEB && d->nx > 1 && d->ny > 1) { *why = "2D not supported for the Lieb lattice"; return TWMC_ERR_INVALID; }
  const int64_t n = (d->lattice == TWMC_LATTICE_LIEB ? 3 : 1) * d->nx * d->ny;
  if (n > 16384) { *why = "more than 16384 sites per trajectory"; return TWMC_ERR_INVALID; }
  if (!(d->dt > 0)) { *why = "dt must be > 0"; return TWMC_ERR_INVALID; }
  if (d->frame_steps < 1) { *why = "frame_steps must be >= 1"; return TWMC_ERR_INVALID; }
  if (d->precision != TWMC_PREC_F32 && d->precision != TWMC_PREC_F64) { *why = "unknown precision"; return TWMC_ERR_INVALID; }
  if (d->noise_mode != TWMC_NOISE_PHILOX && d->noise_mode != TWMC_NOISE_BUFFER) { *why = "unknown noise mode"; return TWMC_ERR_INVALID; }
  if (d->hop_mode != TWMC_HOP_FFT && d->hop_mode != TWMC_HOP_STENCIL) { *why = "unknown hop mode"; return TWMC_ERR_INVALID; }
  if (d->gamma < 0) { *why = "gamma must be >= 0"; return TWMC_ERR_INVALID; }
  const twmc_matrix* ms[5] = {&d->omega, &d->U, &d->F, &d->beta_init, &d->beta_init_sigma};
  for (const twmc_matrix* m : ms) {
    if (m->noise_kind < 0 || m->noise_kind > 2) { *why = "unknown noise kind"; return TWMC_ERR_INVALID; }
    if (m->noise_kind != 0 && !m->noise_amp) { *why = "noisy matrix without amplitudes"; return TWMC_ERR_INVALID; }
  }
  if (d->beta_init.noise_kind != 0 || d->beta_init_sigma.noise_kind != 0) {
    *why = "noise on beta_init / beta_init_sigma is not supported";
    return TWMC_ERR_INVALID;
  }
  if (d->integrator != TWMC_INTEGRATOR_EULER && d->integrator != TWMC_INTEGRATOR_SPLIT) {
    *why = "unknown integrator";
    return TWMC_ERR_INVALID;
  }
  if (d->thermo != 0 && d->lattice != TWMC_LATTICE_SQUARE) {
    *why = "work / area accumulation is defined for the square lattice only";
    return TWMC_ERR_INVALID;
  }
  if (d->ft_nrec > 0) {
    if (!d->ft_times || !d->ft_values) { *why = "F(t) table without data"; return TWMC_ERR_INVALID; }
    for (int64_t i = 1; i < d->ft_nrec; ++i)
      if (!(d->ft_times[i] > d->ft_times[i - 1])) { *why = "F(t) times must increase"; return TWMC_ERR_INVALID; }
  }
  return TWMC_OK;
}

}  // namespace

extern "C" {

int twmc_version(void) { return TWMC_ABI_VERSION; }

int twmc_create(const twmc_system_desc* d, twmc_handle** out) {
  if (!out) return TWMC_ERR_INVALID;
  *out = nullptr;
  std::string why;
  int rc = validate_desc(d, &why);
  twmc_handle* h = new (std::nothrow) twmc_handle();
  if (!h) return TWMC_ERR_NOMEM;
  if (rc != TWMC_OK) { h->err = why; *out = h; return rc; }
  try {
    cudaError_t e = cudaGetDevice(&h->device);
    if (e != cudaSuccess) { *out = h; return cuda_fail(h, e, "cudaGetDevice"); }
    e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { *out = h; return cuda_fail(h, e, "cudaStreamCreate"); }
    h->lattice = d->lattice;
    h->prec = d->precision;
    h->noise_mode = d->noise_mode;
    h->hop_mode = d->hop_mode;
    h->pbc = d->pbc;
    h->nx = d->nx; h->ny = d->ny;
    h->nsites = (d->lattice == TWMC_LATTICE_LIEB ? 3 : 1) * d->nx * d->ny;
    h->frame_steps = d->frame_steps;
    h->J = d->J; h->J_AB = d->J_AB; h->J_BC = d->J_BC;
    h->gamma = d->gamma; h->detuning = d->detuning; h->dt = d->dt;
    h->nblocks = d->n_moment_blocks > 0 ? d->n_moment_blocks : 32;
    read_matrix(d->omega, h->nsites, &h->m_omega);
    read_matrix(d->U, h->nsites, &h->m_U);
    read_matrix(d->F, h->nsites, &h->m_F);
    read_matrix(d->beta_init, h->nsites, &h->m_binit);
    read_matrix(d->beta_init_sigma, h->nsites, &h->m_bsigma);
    if (d->ft_nrec > 0) {
      h->timedep = true;
      build_time_table(h, d->ft_times, d->ft_values, d->ft_nrec);
    }
    h->thermo = d->thermo != 0;
    h->integrator = d->integrator;
    setup_params(h);
    if (h->lattice == TWMC_LATTICE_SQUARE && h->hop_mode == TWMC_HOP_FFT && !h->timedep && !h->thermo) {
      const int bx = ilog2_exact(h->nx), by = ilog2_exact(h->ny);
      PlanView pv;
      if (bx >= 0 && by >= 0 && square_plan(bx, by, &pv)) { h->use_fft = true; h->bx = bx; h->by = by; }
    }
    if (h->integrator == TWMC_INTEGRATOR_SPLIT && !h->use_fft) {
      h->err = "the split-step integrator needs the FFT path (square lattice, hop_mode FFT, power-of-two sides "
               "of a compiled plan, no F(t), no work / area)";
      *out = h;
      return TWMC_ERR_INVALID;
    }
    h->kname = h->use_fft ? "square_fft_kernel" : (h->lattice == TWMC_LATTICE_LIEB ? "ell_kernel<table>" : "ell_kernel<stencil>");
    if (!h->use_fft && h->lattice == TWMC_LATTICE_SQUARE && h->prec == TWMC_PREC_F32 && h->nsites > 8192 &&
        !h->timedep && !h->thermo)
      h->kname = "ell_cluster_kernel";  // 2-CTA cluster per trajectory (see twmc_ell.cu use_cluster)
    rc = build_tables(h);
    *out = h;
    return rc;
  } catch (const std::exception& ex) {
    h->err = ex.what();
    *out = h;
    return TWMC_ERR_INVALID;
  }
}

int twmc_set_noise_buffer(twmc_handle* h, const double* xi, size_t count) {
  if (!h) return TWMC_ERR_INVALID;
  if (!xi && count) return fail(h, TWMC_ERR_INVALID, "null noise buffer");
  h->noise_host.assign(xi, xi + 2 * count);
  h->noise_set = true;
  return TWMC_OK;
}

int twmc_progress(const twmc_handle* h, double* fraction) {
  if (!h || !fraction) return TWMC_ERR_INVALID;
  *fraction = h->progress;
  return TWMC_OK;
}

const char* twmc_last_error(const twmc_handle* h) { return h ? h->err.c_str() : "null handle"; }

void twmc_destroy(twmc_handle* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->dl_stream) cudaStreamSynchronize(h->dl_stream);
  for (cudaEvent_t e : h->dl_ev) cudaEventDestroy(e);
  if (h->h_stage) cudaFreeHost(h->h_stage);
  if (h->snap_ready) cudaEventDestroy(h->snap_ready);
  if (h->snap_free) cudaEventDestroy(h->snap_free);
  if (h->dl_stream) cudaStreamDestroy(h->dl_stream);
  for (auto& e : h->ev_pending) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
  for (auto& e : h->ev_free) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

int twmc_batch_init(twmc_handle* h, const twmc_task_desc* tasks, size_t n) {
  if (!h || (!tasks && n)) return TWMC_ERR_INVALID;
  if (n == 0) return fail(h, TWMC_ERR_INVALID, "empty batch");
  try {
    cudaSetDevice(h->device);
    h->err.clear();
    h->noise_steps = 0;
    return batch_init(h, tasks, n);
  } catch (const std::bad_alloc&) {
    return fail(h, TWMC_ERR_NOMEM, "host allocation failed");
  }
}

int twmc_batch_advance(twmc_handle* h, int64_t n_steps) {
  if (!h || n_steps < 0) return TWMC_ERR_INVALID;
  if (h->noise_mode == TWMC_NOISE_BUFFER) return fail(h, TWMC_ERR_INVALID, "batch API runs Philox noise only");
  if (h->timedep) return fail(h, TWMC_ERR_INVALID, "batch API does not take an F(t) table");
  cudaSetDevice(h->device);
  return advance(h, n_steps, true);
}

int twmc_batch_reduce(twmc_handle* h) {
  if (!h) return TWMC_ERR_INVALID;
  cudaSetDevice(h->device);
  return reduce(h);
}

int twmc_sync(twmc_handle* h, double* kernel_ms) {
  if (!h) return TWMC_ERR_INVALID;
  cudaSetDevice(h->device);
  cudaError_t e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamSynchronize");
  double ms = h->carry_ms;  // step launches of twmc_run calls since the last twmc_sync
  h->carry_ms = 0.0;
  for (auto& ev : h->ev_pending) {
    float x = 0;
    if (cudaEventElapsedTime(&x, ev.first, ev.second) == cudaSuccess) ms += x;
    h->ev_free.push_back(ev);
  }
  h->ev_pending.clear();
  if (kernel_ms) *kernel_ms = ms;
  return TWMC_OK;
}

int twmc_batch_download(twmc_handle* h, double* field, double* moments) {
  if (!h) return TWMC_ERR_INVALID;
  cudaSetDevice(h->device);
  if (field) { int rc = download_field(h, field); if (rc) return rc; }
  if (moments) {
    const int nb = int(std::min<int64_t>(h->nblocks, std::max<int64_t>(h->ntraj, 1)));
    std::vector<double> tmp(size_t(h->nblocks) * h->nsites * 3, 0.0);
    TWMC_CUDA(h, cudaMemcpyAsync(tmp.data(), h->d_moments.p, size_t(nb) * h->nsites * 3 * sizeof(double),
                                 cudaMemcpyDeviceToHost, h->stream));
    TWMC_CUDA(h, cudaStreamSynchronize(h->stream));
    std::memcpy(moments, tmp.data(), tmp.size() * sizeof(double));
  }
  return TWMC_OK;
}

int64_t twmc_launch_count(const twmc_handle* h) { return h ? h->launches : -1; }

const char* twmc_kernel_name(const twmc_handle* h) { return h ? h->kname.c_str() : ""; }

void* twmc_stream(const twmc_handle* h) { return h ? reinterpret_cast<void*>(h->stream) : nullptr; }

int twmc_measure_fp32_peak(double* tflops) {
  if (!tflops) return TWMC_ERR_INVALID;
  std::string err;
  return fp32_peak(tflops, &err) ? TWMC_OK : TWMC_ERR_CUDA;
}

int twmc_run(twmc_handle* h, const twmc_task_desc* tasks, size_t n, twmc_outputs* out) {
  if (!h) return TWMC_ERR_INVALID;
  if (!tasks && n) return fail(h, TWMC_ERR_INVALID, "null tasks");
  if (n == 0) return TWMC_OK;
  try {
    cudaSetDevice(h->device);
    h->err.clear();
    h->progress = 0.0;
    double run_ms = h->carry_ms;  // step time not yet reported to the caller
    h->carry_ms = 0.0;
    const int64_t N = h->nsites;
    // group tasks by (t_start, t_end, store_initial, ic_kind)
    std::map<std::tuple<double, double, int, int>, std::vector<size_t>> groups;
    for (size_t i = 0; i < n; ++i)
      groups[{tasks[i].t_start, tasks[i].t_end, tasks[i].store_initial ? 1 : 0, tasks[i].ic_kind}].push_back(i);
    // frame stride of the output buffer: the largest n_frames of any group
    int64_t max_frames = 0;
    std::vector<Schedule> scheds;
    int64_t total_steps = 0;
    for (auto& g : groups) {
      Schedule s = make_schedule(std::get<0>(g.first), std::get<1>(g.first), h->dt, h->frame_steps,
                                 std::get<2>(g.first) != 0, h->timedep);
      max_frames = std::max(max_frames, s.n_frames);
      total_steps += s.steps * int64_t(g.second.size());
      scheds.push_back(std::move(s));
    }
    int64_t done_steps = 0;
    size_t gi = 0;
    const int nb = h->nblocks;
    for (auto& g : groups) {
      const Schedule& s = scheds[gi++];
      const std::vector<size_t>& idx = g.second;
      const size_t bn = idx.size();
      std::vector<twmc_task_desc> bt(bn);
      for (size_t i = 0; i < bn; ++i) bt[i] = tasks[idx[i]];
      int rc = batch_init(h, bt.data(), bn);
      if (rc) return rc;
      // deterministic noise for this group: [task][step][site]
      h->noise_steps = 0;
      if (h->noise_mode == TWMC_NOISE_BUFFER) {
        if (!h->noise_set) return fail(h, TWMC_ERR_INVALID, "noise buffer mode without twmc_set_noise_buffer");
        const size_t need = n * size_t(s.steps) * size_t(N);
        if (h->noise_host.size() / 2 != need || groups.size() != 1)
          return fail(h, TWMC_ERR_INVALID, "noise buffer must hold n_tasks x steps x n_sites values (one task group)");
        std::vector<cd> nz(need);
        for (size_t i = 0; i < need; ++i) nz[i] = cd(h->noise_host[2 * i], h->noise_host[2 * i + 1]);
        if (!upload_c(&h->d_noise, nz, h->prec)) return fail(h, TWMC_ERR_NOMEM, "noise upload");
        h->noise_steps = s.steps;
      }
      if (h->timedep) {
        std::vector<int> ids(size_t(s.steps));
        std::vector<double> offs(size_t(s.steps));
        int64_t hint = 0;
        for (int64_t k = 0; k < s.steps; ++k) {
          auto seg = time_segment(h->ft_times, s.step_t[size_t(k)], hint);
          ids[size_t(k)] = seg.first;
          offs[size_t(k)] = seg.second;
          hint = seg.first;
        }
        std::vector<float> offs_f(offs.begin(), offs.end());
        if (!upload_raw(&h->d_ft_id, ids.data(), ids.size()) || !upload_raw(&h->d_ft_dt, offs.data(), offs.size()) ||
            !upload_raw(&h->d_ft_dt_f, offs_f.data(), offs_f.size()))
          return fail(h, TWMC_ERR_NOMEM, "F(t) schedule upload");
      }
      // realisations of noisy matrices
      TWMC_CUDA(h, cudaStreamSynchronize(h->stream));
      double* real_dst[3] = {out ? out->U_realization : nullptr, out ? out->omega_realization : nullptr,
                             out ? out->F_realization : nullptr};
      for (int m = 0; m < 3; ++m) {
        if (!real_dst[m]) continue;
        std::vector<double> tmp(size_t(bn * N * 2));
        TWMC_CUDA(h, cudaMemcpy(tmp.data(), h->d_real_out[m].p, tmp.size() * sizeof(double), cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < bn; ++i)
          std::memcpy(real_dst[m] + idx[i] * N * 2, &tmp[i * N * 2], sizeof(double) * size_t(N * 2));
      }
      // tasks of this group in consecutive output rows: frames and the final
      // field are copied to their places by strided asynchronous copies
      bool contiguous = true;
      for (size_t i = 1; i < bn && contiguous; ++i) contiguous = idx[i] == idx[0] + i;
      // Staging for host copies on the handle's second stream (dl_stream): the
      // batch widened into d_snap (FP32 runs, consecutive output rows, at
      // most kSnapMax bytes) is copied to the caller while the next steps
      // compute. snap_free (recorded on dl_stream after each copy from
      // d_snap) orders the next write of d_snap after it.
      const bool stage = contiguous && h->prec == 0 && size_t(bn) * size_t(N) * 16 <= kSnapMax &&
                         int64_t(bn) * N >= (int64_t(1) << 20);
      bool dl_used = false;
      // copies into the caller's arrays may still be in flight when a group
      // ends early with an error: drain both streams on every exit
      struct Drain {
        twmc_handle* h;
        ~Drain() {
          if (h->stream) cudaStreamSynchronize(h->stream);
          if (h->dl_stream) cudaStreamSynchronize(h->dl_stream);
        }
      } drain{h};
      const size_t row = size_t(2 * N);  // doubles per trajectory
      auto stage_setup = [&]() -> int {
        if (!h->dl_stream) TWMC_CUDA(h, cudaStreamCreateWithFlags(&h->dl_stream, cudaStreamNonBlocking));
        while (h->dl_ev.size() < size_t(kFinalChunks)) {
          cudaEvent_t e;
          TWMC_CUDA(h, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
          h->dl_ev.push_back(e);
        }
        if (!h->snap_ready) TWMC_CUDA(h, cudaEventCreateWithFlags(&h->snap_ready, cudaEventDisableTiming));
        if (!h->snap_free) TWMC_CUDA(h, cudaEventCreateWithFlags(&h->snap_free, cudaEventDisableTiming));
        if (!h->d_snap.ensure(size_t(bn) * row * sizeof(double))) return fail(h, TWMC_ERR_NOMEM, "staging buffer");
        dl_used = true;
        return TWMC_OK;
      };
      // final-field pipeline: the steps that end the run go in kFinalChunks
      // trajectory ranges, each range widened into d_snap and copied to the
      // caller's rows on dl_stream while the next range computes (also Philox
      // noise and no work / area)
      const bool pipe = stage && out && out->final_field && !h->thermo && h->noise_mode == TWMC_NOISE_PHILOX &&
                        int64_t(bn) >= kFinalChunks;
      bool final_sent = false, frame_sent = false;
      // fdst: the last saved frame's rows when this step ends on it (sent
      // range by range as well)
      auto step = [&](int64_t nsteps, bool nk, bool last, double* fdst) -> int {
        if (!(pipe && last && nsteps > 0)) return advance(h, nsteps, nk);
        int r2 = stage_setup();
        if (r2) return r2;
        double* snap = h->d_snap.as<double>();
        const float* st = static_cast<const float*>(h->d_state.p);
        for (int c = 0; c < kFinalChunks; ++c) {
          const int64_t t0 = int64_t(bn) * c / kFinalChunks, t1 = int64_t(bn) * (c + 1) / kFinalChunks;
          r2 = advance(h, nsteps, nk, t0, t1, false);
          if (r2) return r2;
          if (c == 0) TWMC_CUDA(h, cudaStreamWaitEvent(h->stream, h->snap_free, 0));
          std::string err;
          if (!widen_launch(st + size_t(t0) * row, snap + size_t(t0) * row, int64_t(size_t(t1 - t0) * row), h->stream, &err))
            return fail(h, TWMC_ERR_CUDA, err);
          TWMC_CUDA(h, cudaEventRecord(h->dl_ev[size_t(c)], h->stream));
          TWMC_CUDA(h, cudaStreamWaitEvent(h->dl_stream, h->dl_ev[size_t(c)], 0));
          TWMC_CUDA(h, cudaMemcpyAsync(out->final_field + (idx[0] + size_t(t0)) * row, snap + size_t(t0) * row,
                                       size_t(t1 - t0) * row * sizeof(double), cudaMemcpyDeviceToHost, h->dl_stream));
          if (fdst)
            TWMC_CUDA(h, copy_rows_d2h(h->device, fdst + size_t(t0) * size_t(max_frames) * row, size_t(max_frames) * row,
                                       snap + size_t(t0) * row, row, size_t(t1 - t0), h->dl_stream));
        }
        frame_sent = fdst != nullptr;
        TWMC_CUDA(h, cudaEventRecord(h->snap_free, h->dl_stream));
        h->step_pos += uint32_t(nsteps);
        final_sent = true;
        return TWMC_OK;
      };
      // a saved frame through d_snap (the last frame of a pipelined run is
      // already staged there)
      auto stage_frame = [&](double* dst) -> int {
        int r2 = stage_setup();
        if (r2) return r2;
        if (!final_sent) {
          TWMC_CUDA(h, cudaStreamWaitEvent(h->stream, h->snap_free, 0));
          std::string err;
          if (!widen_launch(h->d_state.p, h->d_snap.as<double>(), int64_t(size_t(bn) * row), h->stream, &err))
            return fail(h, TWMC_ERR_CUDA, err);
          TWMC_CUDA(h, cudaEventRecord(h->snap_ready, h->stream));
          TWMC_CUDA(h, cudaStreamWaitEvent(h->dl_stream, h->snap_ready, 0));
        }
        TWMC_CUDA(h, copy_rows_d2h(h->device, dst, size_t(max_frames) * row, h->d_snap.p, row, size_t(bn), h->dl_stream));
        TWMC_CUDA(h, cudaEventRecord(h->snap_free, h->dl_stream));
        return TWMC_OK;
      };
      auto save_frame = [&](int64_t f) -> int {
        if (out && out->moments) {
          int r2 = reduce(h);
          if (r2) return r2;
          double* dst = out->moments + size_t(f) * nb * N * 3;
          if (int64_t(bn) >= nb) {  // every block holds trajectories: one copy, no wait
            TWMC_CUDA(h, cudaMemcpyAsync(dst, h->d_moments.p, size_t(nb) * N * 3 * sizeof(double),
                                         cudaMemcpyDeviceToHost, h->stream));
          } else {
            r2 = twmc_batch_download(h, nullptr, dst);
            if (r2) return r2;
          }
        }
        if (out && out->frames) {
          if (stage) {
            if (!frame_sent) {
              int r2 = stage_frame(out->frames + (idx[0] * max_frames + f) * N * 2);
              if (r2) return r2;
            }
            frame_sent = false;
          } else {
            int r2 = download_scatter(h, [&](size_t i) { return out->frames + (idx[i] * max_frames + f) * N * 2; });
            if (r2) return r2;
          }
        }
        if (h->thermo) {  // work / area since the previous save, then reset
          double* dst[2] = {out ? out->work : nullptr, out ? out->area : nullptr};
          DevBuf* src[2] = {&h->d_work, &h->d_area};
          for (int k = 0; k < 2; ++k) {
            if (dst[k]) {
              std::vector<double> v(size_t(bn * N));
              int r2 = download_real(h, *src[k], v.data(), size_t(bn * N));
              if (r2) return r2;
              for (size_t i = 0; i < bn; ++i)
                std::memcpy(dst[k] + (idx[i] * max_frames + f) * N, &v[i * N], sizeof(double) * size_t(N));
            }
            TWMC_CUDA(h, cudaMemsetAsync(src[k]->p, 0, size_t(bn * N) * rsize(h->prec), h->stream));
          }
        }
        return TWMC_OK;
      };
      int64_t f = 0, cur = 0;
      const bool want_nk = out && out->moments;
      if (std::get<2>(g.first) && s.n_frames > 0) {
        if (want_nk && h->use_fft) { rc = advance(h, 0, true); if (rc) return rc; }
        rc = save_frame(f++);
        if (rc) return rc;
      }
      for (int64_t ss : s.save_steps) {
        const bool last = ss == s.steps;
        double* fdst = last && stage && out && out->frames ? out->frames + (idx[0] * max_frames + f) * N * 2 : nullptr;
        rc = step(ss - cur, want_nk, last, fdst);
        if (rc) return rc;
        done_steps += (ss - cur) * int64_t(bn);
        cur = ss;
        rc = save_frame(f++);
        if (rc) return rc;
        h->progress = total_steps ? double(done_steps) / double(total_steps) : 1.0;
      }
      if (s.steps > cur) {
        rc = step(s.steps - cur, false, true, nullptr);
        if (rc) return rc;
        done_steps += (s.steps - cur) * int64_t(bn);
      }
      if (out && out->final_field && !final_sent) {  // (a pipelined run has sent it already)
        if (contiguous) {
          rc = download_rows(h, out->final_field + idx[0] * N * 2, size_t(N * 2));
          if (rc) return rc;
        } else {
          rc = download_scatter(h, [&](size_t i) { return out->final_field + idx[i] * N * 2; });
          if (rc) return rc;
        }
      }
      std::vector<int> st(bn);
      TWMC_CUDA(h, cudaMemcpyAsync(st.data(), h->d_status.p, bn * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
      TWMC_CUDA(h, cudaStreamSynchronize(h->stream));
      if (dl_used) TWMC_CUDA(h, cudaStreamSynchronize(h->dl_stream));
      for (size_t i = 0; i < bn; ++i) {
        if (out && out->status) out->status[idx[i]] = st[i];
        if (out && out->t_final) out->t_final[idx[i]] = s.t_final;
        if (out && out->frames_written) out->frames_written[idx[i]] = s.frames_written;
      }
      double ms = 0.0;
      rc = twmc_sync(h, &ms);
      if (rc) return rc;
      run_ms += ms;
    }
    h->progress = 1.0;
    h->noise_set = false;
    h->carry_ms = run_ms;  // reported by the caller's next twmc_sync
    return TWMC_OK;
  } catch (const std::bad_alloc&) {
    return fail(h, TWMC_ERR_NOMEM, "host allocation failed");
  } catch (const std::exception& ex) {
    return fail(h, TWMC_ERR_INVALID, ex.what());
  }
}

int twmc_debug_philox(const uint32_t* ctr, size_t n, const uint32_t* key, uint32_t* out) {
  if ((!ctr || !out) && n) return TWMC_ERR_INVALID;
  if (!key) return TWMC_ERR_INVALID;
  DevBuf dc, dout;
  if (!dc.ensure(n * 16) || !dout.ensure(n * 16)) return TWMC_ERR_NOMEM;
  if (cudaMemcpy(dc.p, ctr, n * 16, cudaMemcpyHostToDevice) != cudaSuccess) return TWMC_ERR_CUDA;
  std::string err;
  if (!philox_launch(dc.as<uint32_t>(), n, key[0], key[1], dout.as<uint32_t>(), nullptr, &err)) return TWMC_ERR_CUDA;
  if (cudaMemcpy(out, dout.p, n * 16, cudaMemcpyDeviceToHost) != cudaSuccess) return TWMC_ERR_CUDA;
  return TWMC_OK;
}

int twmc_debug_wiener(int32_t precision, uint32_t seed, uint64_t id, uint32_t step0, int64_t n_steps,
                      int64_t n_sites, double* out) {
  if (precision != TWMC_PREC_F32 && precision != TWMC_PREC_F64) return TWMC_ERR_INVALID;
  if (n_steps < 0 || n_sites < 1 || (n_steps > 0 && !out)) return TWMC_ERR_INVALID;
  if (n_steps > (int64_t(1) << 40) / n_sites) return TWMC_ERR_INVALID;
  const size_t bytes = size_t(n_steps) * size_t(n_sites) * 16;
  if (bytes == 0) return TWMC_OK;
  DevBuf dout;
  if (!dout.ensure(bytes)) return TWMC_ERR_NOMEM;
  std::string err;
  if (!wiener_launch(precision == TWMC_PREC_F32 ? 0 : 1, seed, uint32_t(id), step0, n_steps, n_sites,
                     dout.as<double>(), nullptr, &err))
    return TWMC_ERR_CUDA;
  if (cudaMemcpy(out, dout.p, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) return TWMC_ERR_CUDA;
  return TWMC_OK;
}

}  // extern "C"
