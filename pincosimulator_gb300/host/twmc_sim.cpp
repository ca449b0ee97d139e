// twmc_sim.cpp -- the TWMC manager: `twmc_sim -i run.ini [-o out] [key value]...`
//
// Follows the reference's TWMCManager (src/TWMC/TWMCManager.cpp:38-204):
// builds TWMCSystemData from the settings, selects the solver by name
// (`solver` key, default "TWMCCuda"; an unknown name is the reference's
// NoEligibleSolver), dispatches n_traj trajectory tasks with seeds from
// mt19937(SEED), resumes trajectories already in the output archive whose
// stored end time plus one frame interval is before t_end (continuations
// start from the last stored frame with a fresh seed and without storing the
// initial state), and stores every result in the Pinco archive under
// <out>/data together with _t.dat (and _F_t.dat for a time-tabulated F).
//
// `twmc_sim --describe -i run.ini [key value]...` prints the resolved system
// as JSON instead of running it.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <filesystem>
#include <iostream>
#include <random>
#include <sstream>
#include <vector>

#include "PincoFormat.hpp"
#include "Settings.hpp"
#include "TWMC.hpp"

namespace fs = std::filesystem;
using namespace pinco;

namespace {

std::string json_cvec(const std::vector<cplx>& v) {
  std::ostringstream o;
  o.precision(17);
  o << "[";
  for (size_t i = 0; i < v.size(); ++i) o << (i ? "," : "") << "[" << v[i].real() << "," << v[i].imag() << "]";
  o << "]";
  return o.str();
}

std::string json_matrix(const NoisyMatrix& m) {
  std::ostringstream o;
  o << "{\"rows\":" << m.rows() << ",\"cols\":" << m.cols() << ",\"setup\":" << (m.IsSetup() ? "true" : "false")
    << ",\"noise\":" << int(m.GetNoiseType()) << ",\"base\":" << json_cvec(m.base())
    << ",\"amp\":" << json_cvec(m.amp()) << ",\"times\":[";
  o.precision(17);
  for (size_t i = 0; i < m.times().size(); ++i) o << (i ? "," : "") << m.times()[i];
  o << "],\"time_values\":" << json_cvec(m.time_values()) << "}";
  return o.str();
}

void describe(const Settings& s, const TWMCSystemData& d) {
  std::ostringstream o;
  o.precision(17);
  o << "{\"nx\":" << d.nx << ",\"ny\":" << d.ny << ",\"cellSz\":" << d.cellSz << ",\"lattice\":\"" << d.latticeName
    << "\",\"dimension\":" << int(d.dimension) << ",\"PBC\":" << (d.PBC ? "true" : "false") << ",\"J\":" << d.J_val
    << ",\"J_AB\":" << d.J_AB_val << ",\"J_BC\":" << d.J_BC_val << ",\"gamma\":" << d.gamma_val
    << ",\"detuning\":" << d.detuning << ",\"dt\":" << d.dt << ",\"t_start\":" << d.t_start
    << ",\"t_end\":" << d.t_end << ",\"frame_steps\":" << d.frame_steps << ",\"dt_obs\":" << d.dt_obs
    << ",\"nFramesTot\":" << d.nFramesTot << ",\"n_dt\":" << d.n_dt << ",\"n_traj\":" << s.getSize("n_traj")
    << ",\"seed\":" << s.GlobalSeed() << ",\"manager\":\"" << s.getString("Manager") << "\""
    << ",\"output\":\"" << s.GetOutputFolder() << "\""
    << ",\"precision\":\"" << d.precision << "\",\"hop\":\"" << d.hop << "\",\"integrator\":\"" << d.integrator << "\""
    << ",\"U\":" << json_matrix(d.U) << ",\"F\":" << json_matrix(d.F) << ",\"omega\":" << json_matrix(d.omega)
    << ",\"E\":" << json_matrix(d.E) << ",\"beta_init\":" << json_matrix(d.beta_init)
    << ",\"beta_init_sigma\":" << json_matrix(d.beta_init_sigma) << ",\"stored_times\":[";
  auto times = d.GetStoredTimes();
  for (size_t i = 0; i < times.size(); ++i) o << (i ? "," : "") << times[i];
  o << "]}";
  std::cout << o.str() << std::endl;
}

// The merge manager (MergeManager.cpp:54-102, registered as "merge"): every
// trajectory of oldArchive1, then of oldArchive2, is loaded whole
// (continuations joined) and stored in the archive under the output folder.
// An id present in both archives is stored twice, the second time as a
// continuation of the first, as the reference's saver does. The save-time
// tables (_t.dat, _F_t.dat) of the first archive are copied when present.
int merge(const Settings& s) {
  const fs::path out = fs::path(s.GetOutputFolder()) / "data";
  fs::create_directories(out);
  PincoArchive dst(out.string(), s.getDouble("chunk_size", 1.5));
  size_t n = 0;
  for (const char* key : {"oldArchive1", "oldArchive2"}) {
    const std::string root = s.getString(key);
    if (root.empty()) throw std::runtime_error(std::string("merge: missing key ") + key);
    const fs::path src = fs::path(root) / "data";
    if (!fs::exists(src / "_register.bin")) throw std::runtime_error("merge: no archive in " + src.string());
    PincoArchive a(src.string());
    std::cout << "Loading data from: " << root << " (" << a.UsedIds().size() << " trajectories)" << std::endl;
    for (size_t id : a.UsedIds()) {
      auto r = a.Load(id, false);
      if (!r) throw std::runtime_error("merge: cannot load trajectory " + std::to_string(id));
      dst.Store(*r);
      ++n;
    }
    if (std::string(key) == "oldArchive1")
      for (const char* f : {"_t.dat", "_F_t.dat"})
        if (fs::exists(src / f) && !fs::exists(out / f)) fs::copy_file(src / f, out / f);
  }
  std::cout << "Saved " << n << " items." << std::endl;
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  bool want_describe = false;
  std::vector<const char*> args;
  for (int i = 0; i < argc; ++i) {
    if (std::string(argv[i]) == "--describe") want_describe = true;
    else args.push_back(argv[i]);
  }
  try {
    Settings settings(int(args.size()), args.data());
    if (settings.getString("Manager") == "merge") return merge(settings);
    auto sys = std::make_shared<TWMCSystemData>(settings);
    if (want_describe) {
      describe(settings, *sys);
      return 0;
    }
    const std::string solver_name = settings.getString("solver", "TWMCCuda");
    std::unique_ptr<Solver> solver = SolverFactory::makeUniqueNewInstance(solver_name);
    if (!solver) {
      std::cerr << "ERROR: No solver available (" << solver_name << ")." << std::endl;
      return 2;
    }
    const fs::path out = settings.GetOutputFolder();
    const fs::path data = out / "data";
    PincoArchive archive(data.string(), settings.getDouble("chunk_size", 1.5));
    SaveRealColumn((data / "_t.dat").string(), sys->GetStoredTimes());
    if (sys->F.HasTimeDependence()) SaveComplexRows((data / "_F_t.dat").string(), sys->GetStoredVariableEvolution(sys->F));

    std::mt19937 seeds(settings.GlobalSeed());
    std::vector<std::unique_ptr<TaskData>> tasks;
    const std::set<size_t> used = archive.UsedIds();
    size_t n_traj = settings.getSize("n_traj");
    const double t_end = settings.getDouble("t_end");
    if (used.size() < n_traj) {
      size_t max_id = used.empty() ? 0 : *used.rbegin();
      for (size_t i = used.size(); i < n_traj; ++i) {
        auto t = std::make_unique<TWMCTaskData>();
        t->systemData = sys;
        t->t_start = sys->t_start;
        t->t_end = sys->t_end;
        t->initialCondition = TWMCTaskData::ReadFromSettings;
        t->rngSeed = seeds();
        t->storeInitialState = true;
        t->id = ++max_id;
        tasks.push_back(std::move(t));
      }
    }
    for (size_t id : used) {
      auto last = archive.Load(id, true);
      if (!last || !(last->extra[1] + sys->dt_obs < t_end)) continue;
      auto t = std::make_unique<TWMCTaskData>();
      t->systemData = sys;
      t->t_start = last->extra[1];
      t->t_end = t_end;
      t->initialCondition = TWMCTaskData::ReadFromPreviousData;
      t->rngSeed = seeds();
      t->id = id;
      t->storeInitialState = false;
      const Dataset* tr = last->find("traj");
      if (!tr || tr->data.size() < sys->n_sites()) { std::cerr << "trajectory " << id << " has no frame" << std::endl; return 3; }
      t->prevField.assign(tr->data.end() - long(sys->n_sites()), tr->data.end());
      if (auto* d = last->find("U_Realization")) t->prevU = d->data;
      if (auto* d = last->find("Omega_Realization")) t->prevOmega = d->data;
      if (auto* d = last->find("F_Realizatio")) t->prevF = d->data;
      tasks.push_back(std::move(t));
    }
    std::cout << "Enqueued " << tasks.size() << " tasks. " << std::endl;
    // batches bounded by host memory for the returned frames
    const double budget = settings.getDouble("batch_memory_gb", 4.0) * 1024.0 * 1024.0 * 1024.0;
    const double per_task = double(sys->nFramesTot + 2) * double(sys->n_sites()) * 16.0;
    const size_t batch = std::max<size_t>(1, std::min<size_t>(solver->nTasksToRequest, size_t(budget / per_task)));
    const auto t0 = std::chrono::steady_clock::now();
    size_t done = 0, bad = 0;
    for (size_t b = 0; b < tasks.size(); b += batch) {
      std::vector<std::unique_ptr<TaskData>> part;
      for (size_t k = b; k < std::min(tasks.size(), b + batch); ++k) part.push_back(std::move(tasks[k]));
      auto results = solver->Compute(part);
      for (auto& r : results) {
        auto* tr = static_cast<TWMCResults*>(r.get());
        if (tr->status != 0) ++bad;
        archive.Store(*tr);
      }
      done += results.size();
      const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      std::cout << "Completed " << done << "/" << tasks.size() << ", elapsed " << el << " s" << std::endl;
    }
    if (bad) std::cerr << bad << " trajectories became non-finite" << std::endl;
    return 0;
  } catch (const std::exception& e) {
    std::cerr << "ERROR: " << e.what() << std::endl;
    return 1;
  }
}
