// TWMC.hpp -- the TWMC system, task and result types, and the GPU solver
// plugin registered as "TWMCCuda".
//
//   TWMCSystemData   the reference's TWMCSystemData (src/TWMC/TWMCSystemData.cpp:14-189):
//                    lattice, 1-D swap, parameter matrices, frame grid,
//                    GetStoredTimes / GetStoredVariableEvolution.
//   TWMCTaskData     one trajectory (src/TWMC/TWMCTaskData.hpp:29-43).
//   TWMCResults      datasets of one trajectory with the reference's names
//                    and format ids (src/TWMC/TWMCResults.cpp:26-38) and the
//                    extra data [t_start, t_end].
//   TWMCCudaSolver   Solver plugin that runs a whole batch of tasks through
//                    the C ABI of libtwmc_cuda.so (include/twmc.h).
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "NoisyMatrix.hpp"
#include "Settings.hpp"
#include "Solver.hpp"

struct twmc_handle;

namespace pinco {

class TWMCSystemData {
 public:
  enum Dimension { D0, D1, D2 };
  explicit TWMCSystemData(const Settings& settings);
  TWMCSystemData() = default;

  std::vector<double> GetStoredTimes() const;
  // frames x sites of the time-tabulated F (complex), at the stored times
  std::vector<std::vector<cplx>> GetStoredVariableEvolution(const NoisyMatrix& mat) const;
  size_t ComputeNFrames(double t_start, double t_end) const;

  std::string latticeName;
  size_t nx = 0, ny = 0, nxy = 0, cellSz = 1;
  NoisyMatrix U, F, omega, E, beta_init, beta_init_sigma;
  double J_val = 0, detuning = 0, J_AB_val = 0, J_BC_val = 0, gamma_val = 0;
  double t_start = 0, t_end = 0, dt = 0, dt_obs = 0;
  double frames_freq = 0, frames_period = 0;
  size_t nFramesTot = 0, n_dt = 0, frame_steps = 1;
  bool PBC = false;
  Dimension dimension = D0;
  // engine options (keys absent from the reference's inputs)
  std::string precision = "f32";  // "f32" | "f64"
  std::string hop = "fft";        // "fft" | "stencil"
  std::string integrator = "euler";  // "euler" (the reference's step) | "split" (exact hopping over dt)
  size_t n_sites() const { return nx * ny * cellSz; }
};

class TWMCTaskData : public TaskData {
 public:
  enum InitialConditions { ReadFromSettings, FixedPoint, ReadFromPreviousData };
  std::shared_ptr<TWMCSystemData> systemData;
  size_t id = 0;
  double t_start = 0, t_end = 0;
  bool storeInitialState = true;
  InitialConditions initialCondition = ReadFromSettings;
  unsigned int rngSeed = 0;
  // ReadFromPreviousData: the last frame and the disorder realisations
  std::vector<cplx> prevField, prevU, prevOmega, prevF;
};

struct Dataset {
  std::string name;
  unsigned char format = 22;  // 22 = complex128, 11 = float64
  size_t frames = 1;          // elements in the frames dimension
  std::vector<size_t> dims;   // {nx, ny} or {nx, ny, 3}
  std::vector<cplx> data;     // format 22
  std::vector<double> rdata;  // format 11
};

class TWMCResults : public TaskResults {
 public:
  std::vector<Dataset> datasets;
  double extra[2] = {0, 0};  // t_start, t_end
  int status = 0;            // 0 or TWMC_ERR_NONFINITE
  const Dataset* find(const std::string& name) const {
    for (auto& d : datasets) if (d.name == name) return &d;
    return nullptr;
  }
};

class TWMCCudaSolver : public Solver {
 public:
  TWMCCudaSolver();
  ~TWMCCudaSolver() override;
  std::vector<std::unique_ptr<TaskResults>> Compute(const std::vector<std::unique_ptr<TaskData>>& tasks) override;
  float ApproximateComputationProgress() const override;
  const std::string& last_error() const { return err_; }

 private:
  void SetupFor(const TWMCSystemData* data);
  const TWMCSystemData* last_ = nullptr;
  twmc_handle* h_ = nullptr;
  bool thermo_ = false;  // work / area datasets (F(t) on a periodic lattice)
  std::string err_;
  std::vector<double> ft_times_, ft_vals_;
};

}  // namespace pinco
