// TWMC.cpp -- TWMCSystemData and the TWMCCuda solver plugin (see TWMC.hpp).
#include "TWMC.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <iostream>
#include <limits>

#include "twmc.h"

namespace pinco {

// ---------------------------------------------------------------------------
// TWMCSystemData (TWMCSystemData.cpp:14-115)
// ---------------------------------------------------------------------------
TWMCSystemData::TWMCSystemData(const Settings& s) {
  nx = s.getSize("nx");
  ny = s.getSize("ny");
  cellSz = s.getSize("cellSz", 1);
  latticeName = s.getString("lattice");
  if (latticeName == "lieb") cellSz = 3;
  nxy = nx * ny;
  PBC = s.getBool("PBC", false);
  if (s.getString("Manager") == "TWMCThread") PBC = true;  // TWMCManager.cpp:44-46
  if (nx == 1 && ny == 1) {
    dimension = D0;
  } else if (nx == 1 || ny == 1) {
    dimension = D1;
    if (ny == 1) { ny = nx; nx = 1; }
  } else {
    dimension = D2;
  }
  U = s.GetMatrix("U", nx, ny, cellSz);
  F = s.GetMatrix("F", nx, ny, cellSz);
  omega = s.GetMatrix("omega", nx, ny, cellSz);
  E = s.GetMatrix("E", nx, ny, cellSz);
  detuning = s.getDouble("detuning");
  J_AB_val = s.getDouble("J_AB");
  J_BC_val = s.getDouble("J_BC");
  J_val = s.getDouble("J");
  gamma_val = s.getDouble("gamma");
  beta_init = s.GetMatrix("beta_init", nx, ny, cellSz);
  beta_init_sigma = s.GetMatrix("beta_init_sigma", nx, ny, cellSz);

  const double obs_n_frames = double(s.getSize("n_frames"));
  t_start = s.getDouble("t_start");
  t_end = s.getDouble("t_end");
  frames_freq = s.getDouble("frames_freq");
  frames_period = s.getDouble("frames_period");
  if (frames_freq == 0 && frames_period == 0) {
    if (obs_n_frames == 0) throw ConfigError("Must have a non-zero, integer number of frames!");
    frames_freq = obs_n_frames / (t_end - t_start);
  } else if (frames_freq == 0 && frames_period != 0) {
    frames_freq = 1 / frames_period;
  }
  const double timestep = s.getDouble("timestep");
  if (!(timestep > 0)) throw ConfigError("timestep must be > 0");
  dt = timestep;
  frame_steps = std::max(size_t(1), size_t(std::ceil(1 / (frames_freq * timestep))));
  dt_obs = dt * double(frame_steps);
  nFramesTot = size_t(std::ceil((t_end - t_start) / dt_obs));
  t_end = double(nFramesTot) * dt_obs;
  size_t n_times = 0;
  for (double t = t_start; t <= t_end; t += timestep) ++n_times;
  n_dt = n_times;
  if (dt_obs < dt) { dt_obs = dt; frame_steps = 1; }
  precision = s.getString("precision", "f32");
  hop = s.getString("hop", "fft");
  integrator = s.getString("integrator", "euler");
  if (integrator != "euler" && integrator != "split")
    throw std::runtime_error("integrator must be \"euler\" or \"split\", not \"" + integrator + "\"");
  if (hop != "fft" && hop != "stencil")
    throw std::runtime_error("hop must be \"fft\" or \"stencil\", not \"" + hop + "\"");
  if (precision != "f32" && precision != "f64")
    throw std::runtime_error("precision must be \"f32\" or \"f64\", not \"" + precision + "\"");
}

size_t TWMCSystemData::ComputeNFrames(double ts, double te) const {
  return size_t(std::nearbyint((te - ts) / dt_obs));
}

std::vector<double> TWMCSystemData::GetStoredTimes() const {
  const size_t frames = nFramesTot + 1;
  std::vector<double> times(frames, 0.0);
  double t = t_start;
  size_t i_step = 0, i_frame = 1;
  times[0] = t_start;
  while (t <= t_end) {
    t += dt;
    ++i_step;
    if ((i_step % frame_steps == 0) && i_frame < frames) times[i_frame++] = t;
  }
  return times;
}

namespace {
// Gap-filled time table with slopes (NoisyMatrix.cpp:164-250) and its
// evaluation (NoisyMatrix.cpp:252-265).
struct TimeTable {
  std::vector<double> times;
  std::vector<cplx> vals, slopes;
  size_t n = 0;
  explicit TimeTable(const NoisyMatrix& m) {
    n = m.size();
    times = m.times();
    const size_t nrec = times.size();
    std::vector<cplx> v = m.time_values();
    for (size_t s = 0; s < n; ++s) {
      for (size_t pt = 0; pt < nrec; ++pt) {
        const cplx x = v[pt * n + s];
        if (!(std::isnan(x.real()) || std::isnan(x.imag()))) continue;
        cplx prev(NAN, NAN), next(NAN, NAN);
        long tp = long(pt) - 1;
        for (; tp >= 0 && std::isnan(prev.real()); --tp) prev = v[size_t(tp) * n + s];
        ++tp;
        size_t tn = pt + 1;
        for (; tn < nrec && std::isnan(next.real()); ++tn) next = v[tn * n + s];
        --tn;
        if (std::isnan(prev.real()) && std::isnan(next.real())) break;
        if (std::isnan(next.real())) v[pt * n + s] = prev;
        else if (std::isnan(prev.real())) v[pt * n + s] = next;
        else v[pt * n + s] = prev + (next - prev) / (times[tn] - times[size_t(tp)]) * (times[pt] - times[size_t(tp)]);
      }
    }
    vals = v;
    slopes.assign((nrec + 1) * n, cplx(0, 0));
    for (size_t i = 1; i < nrec; ++i)
      for (size_t s = 0; s < n; ++s)
        slopes[(i - 1) * n + s] = (v[i * n + s] - v[(i - 1) * n + s]) / (times[i] - times[i - 1]);
    vals.resize((nrec + 1) * n);
    for (size_t s = 0; s < n; ++s) vals[nrec * n + s] = v[(nrec - 1) * n + s];
    times.push_back(std::numeric_limits<double>::max());
  }
  std::vector<cplx> at(double t, size_t hint = 0) const {
    std::vector<cplx> out(n);
    if (t <= times[0]) { std::copy(vals.begin(), vals.begin() + long(n), out.begin()); return out; }
    size_t id;
    if (hint + 1 < times.size() && times[hint + 1] > t) id = hint;
    else id = size_t(std::lower_bound(times.begin(), times.end(), t) - times.begin()) - 1;
    for (size_t s = 0; s < n; ++s) out[s] = vals[id * n + s] + cplx(t - times[id], 0) * slopes[id * n + s];
    return out;
  }
};
}  // namespace

std::vector<std::vector<cplx>> TWMCSystemData::GetStoredVariableEvolution(const NoisyMatrix& mat) const {
  const size_t frames = nFramesTot + 1;
  std::vector<std::vector<cplx>> result(frames, std::vector<cplx>(n_sites()));
  if (!mat.HasTimeDependence()) return result;
  TimeTable tt(mat);
  double t = t_start;
  size_t i_step = 0, i_frame = 1;
  result[0] = tt.at(t);
  while (t <= t_end) {
    t += dt;
    ++i_step;
    if ((i_step % frame_steps == 0) && i_frame < frames) result[i_frame++] = tt.at(t);
  }
  return result;
}

// ---------------------------------------------------------------------------
// TWMCCuda solver
// ---------------------------------------------------------------------------
static SolverFactory::Registrator<TWMCCudaSolver> g_register_twmc_cuda("TWMCCuda");

TWMCCudaSolver::TWMCCudaSolver() { nTasksToRequest = size_t(1) << 24; }

TWMCCudaSolver::~TWMCCudaSolver() {
  if (h_) twmc_destroy(h_);
}

namespace {
int noise_kind(const NoisyMatrix& m) {
  switch (m.GetNoiseType()) {
    case NoisyMatrix::Gaussian: return TWMC_DISORDER_GAUSSIAN;
    case NoisyMatrix::Uniform: return TWMC_DISORDER_UNIFORM;
    default: return TWMC_DISORDER_NONE;  // Lorentzian / Poissonian draw nothing (NoisyMatrix.cpp:155-159)
  }
}
twmc_matrix to_c(const NoisyMatrix& m) {
  twmc_matrix c;
  c.base = m.base().empty() ? nullptr : reinterpret_cast<const double*>(m.base().data());
  c.noise_kind = noise_kind(m);
  c.noise_amp = c.noise_kind ? reinterpret_cast<const double*>(m.amp().data()) : nullptr;
  return c;
}
}  // namespace

void TWMCCudaSolver::SetupFor(const TWMCSystemData* d) {
  if (h_) { twmc_destroy(h_); h_ = nullptr; }
  last_ = d;
  twmc_system_desc desc;
  std::memset(&desc, 0, sizeof(desc));
  const bool lieb = d->latticeName == "lieb";
  desc.lattice = lieb ? TWMC_LATTICE_LIEB : TWMC_LATTICE_SQUARE;
  desc.nx = int64_t(d->nx);
  desc.ny = int64_t(d->ny);
  desc.pbc = d->PBC ? 1 : 0;
  desc.J = d->J_val;
  desc.J_AB = d->J_AB_val;
  desc.J_BC = d->J_BC_val;
  desc.gamma = d->gamma_val;
  desc.detuning = d->detuning;
  desc.dt = d->dt;
  desc.frame_steps = int64_t(d->frame_steps);
  desc.omega = to_c(lieb ? d->E : d->omega);
  desc.U = to_c(d->U);
  desc.F = to_c(d->F);
  desc.beta_init = to_c(d->beta_init);
  desc.beta_init_sigma = to_c(d->beta_init_sigma);
  if (d->F.HasTimeDependence()) {
    ft_times_ = d->F.times();
    ft_vals_.assign(reinterpret_cast<const double*>(d->F.time_values().data()),
                    reinterpret_cast<const double*>(d->F.time_values().data()) + 2 * d->F.time_values().size());
    desc.ft_nrec = int64_t(ft_times_.size());
    desc.ft_times = ft_times_.data();
    desc.ft_values = ft_vals_.data();
  }
  desc.precision = d->precision == "f64" ? TWMC_PREC_F64 : TWMC_PREC_F32;
  desc.noise_mode = TWMC_NOISE_PHILOX;
  desc.hop_mode = d->hop == "stencil" ? TWMC_HOP_STENCIL : TWMC_HOP_FFT;
  desc.integrator = d->integrator == "split" ? TWMC_INTEGRATOR_SPLIT : TWMC_INTEGRATOR_EULER;
  // the reference's manager runs a periodic lattice with F(t) on its Thermo
  // solver, which adds the work and area datasets (TWMCManager.cpp:47-58)
  thermo_ = !lieb && d->F.HasTimeDependence();
  desc.thermo = thermo_ ? 1 : 0;
  const int rc = twmc_create(&desc, &h_);
  if (rc != TWMC_OK) {
    err_ = std::string("twmc_create failed: ") + (h_ ? twmc_last_error(h_) : "");
    throw std::runtime_error(err_);
  }
}

std::vector<std::unique_ptr<TaskResults>> TWMCCudaSolver::Compute(const std::vector<std::unique_ptr<TaskData>>& tasks) {
  std::vector<std::unique_ptr<TaskResults>> out;
  size_t i0 = 0;
  while (i0 < tasks.size()) {
    // a run of tasks sharing one system
    auto* first = static_cast<TWMCTaskData*>(tasks[i0].get());
    const TWMCSystemData* d = first->systemData.get();
    size_t i1 = i0;
    while (i1 < tasks.size() && static_cast<TWMCTaskData*>(tasks[i1].get())->systemData.get() == d) ++i1;
    if (d != last_) SetupFor(d);
    const size_t n = i1 - i0, N = d->n_sites();
    std::vector<twmc_task_desc> td(n);
    size_t max_frames = 0;
    for (size_t k = 0; k < n; ++k) {
      auto* t = static_cast<TWMCTaskData*>(tasks[i0 + k].get());
      twmc_task_desc& c = td[k];
      std::memset(&c, 0, sizeof(c));
      c.id = t->id;
      c.seed = t->rngSeed;
      c.t_start = t->t_start;
      c.t_end = t->t_end;
      c.store_initial = t->storeInitialState ? 1 : 0;
      switch (t->initialCondition) {
        case TWMCTaskData::ReadFromSettings: c.ic_kind = TWMC_IC_SETTINGS; break;
        case TWMCTaskData::FixedPoint: c.ic_kind = TWMC_IC_FIXED; break;
        case TWMCTaskData::ReadFromPreviousData:
          c.ic_kind = TWMC_IC_GIVEN;
          c.init_field = reinterpret_cast<const double*>(t->prevField.data());
          if (!t->prevU.empty()) c.U_realization = reinterpret_cast<const double*>(t->prevU.data());
          if (!t->prevOmega.empty()) c.omega_realization = reinterpret_cast<const double*>(t->prevOmega.data());
          if (!t->prevF.empty()) c.F_realization = reinterpret_cast<const double*>(t->prevF.data());
          break;
      }
      max_frames = std::max(max_frames, d->ComputeNFrames(t->t_start, t->t_end) + (t->storeInitialState ? 1 : 0));
    }
    std::vector<cplx> frames(n * std::max<size_t>(max_frames, 1) * N);
    std::vector<cplx> ru(n * N), ro(n * N), rf(n * N);
    std::vector<int64_t> fw(n);
    std::vector<double> tf(n);
    std::vector<int32_t> st(n);
    std::vector<double> work(thermo_ ? frames.size() : 0), area(thermo_ ? frames.size() : 0);
    twmc_outputs o;
    std::memset(&o, 0, sizeof(o));
    o.frames = reinterpret_cast<double*>(frames.data());
    if (thermo_) {
      o.work = work.data();
      o.area = area.data();
    }
    o.U_realization = reinterpret_cast<double*>(ru.data());
    o.omega_realization = reinterpret_cast<double*>(ro.data());
    o.F_realization = reinterpret_cast<double*>(rf.data());
    o.frames_written = fw.data();
    o.t_final = tf.data();
    o.status = st.data();
    const int rc = twmc_run(h_, td.data(), n, &o);
    if (rc != TWMC_OK) {
      err_ = std::string("twmc_run failed: ") + twmc_last_error(h_);
      throw std::runtime_error(err_);
    }
    const bool lieb = d->latticeName == "lieb";
    const std::vector<size_t> dims = lieb ? std::vector<size_t>{d->nx, d->ny, 3} : std::vector<size_t>{d->nx, d->ny};
    for (size_t k = 0; k < n; ++k) {
      auto* t = static_cast<TWMCTaskData*>(tasks[i0 + k].get());
      auto r = std::make_unique<TWMCResults>();
      r->SetId(t->id);
      auto add_real = [&](const NoisyMatrix& m, const char* name, const std::vector<cplx>& src) {
        if (!m.HasNoise()) return;
        Dataset ds;
        ds.name = name;
        ds.frames = 1;
        ds.dims = dims;
        ds.data.assign(src.begin() + long(k * N), src.begin() + long((k + 1) * N));
        r->datasets.push_back(std::move(ds));
      };
      // dataset order of TWMCBaseSolver::Compute / TWMCLiebSolver::Compute
      add_real(d->U, "U_Realization", ru);
      add_real(lieb ? d->E : d->omega, "Omega_Realization", ro);
      add_real(d->F, "F_Realizatio", rf);
      Dataset traj;
      traj.name = "traj";
      traj.frames = size_t(fw[k]);
      traj.dims = dims;
      traj.data.assign(frames.begin() + long(k * max_frames * N), frames.begin() + long((k * max_frames + size_t(fw[k])) * N));
      r->datasets.push_back(std::move(traj));
      if (thermo_) {  // TWMCThermoSolver.cpp:280-282: traj, work, area
        for (int q = 0; q < 2; ++q) {
          const std::vector<double>& src = q ? area : work;
          Dataset ds;
          ds.name = q ? "area" : "work";
          ds.format = 11;
          ds.frames = size_t(fw[k]);
          ds.dims = dims;
          ds.rdata.assign(src.begin() + long(k * max_frames * N), src.begin() + long((k * max_frames + size_t(fw[k])) * N));
          r->datasets.push_back(std::move(ds));
        }
      }
      r->extra[0] = t->t_start;
      r->extra[1] = tf[k];
      r->status = st[k];
      out.push_back(std::move(r));
    }
    i0 = i1;
  }
  return out;
}

float TWMCCudaSolver::ApproximateComputationProgress() const {
  double f = 0.0;
  if (h_) twmc_progress(h_, &f);
  return float(f);
}

}  // namespace pinco
