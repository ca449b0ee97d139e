// NoisyMatrix.hpp -- a per-site parameter matrix with optional per-trajectory
// disorder and optional time table (the reference's NoisyMatrix,
// src/Base/NoisyMatrix.cpp:26-265).
//
// Storage is row-major over (nx, ny * cellSz), the memory order of the
// reference's MatrixCXd. Values read from a matrix file are column-major in
// the file and transposed on load (EigenUtils.cpp:61-96); time-table records
// are copied in memory order (NoisyMatrix.cpp:168-178). The disorder draw
// itself (Gaussian / Uniform on [0,1), NoisyMatrix.cpp:131-162) runs on the
// GPU from a Philox stream; here the matrix only carries base and amplitude.
#pragma once

#include <complex>
#include <map>
#include <string>
#include <vector>

namespace pinco {

using cplx = std::complex<double>;

class NoisyMatrix {
 public:
  enum NoiseType { None, Uniform, Gaussian, Lorentzian, Poissonian };

  NoisyMatrix() = default;
  NoisyMatrix(size_t nx, size_t ny, size_t cellSz = 1) : nx_(nx), ny_(ny * cellSz) {}

  size_t rows() const { return nx_; }
  size_t cols() const { return ny_; }
  size_t size() const { return nx_ * ny_; }

  void SetValue(cplx v) { base_.assign(size(), v); setup_ = true; }
  // N real values or 2N interleaved complex values, column-major
  bool SetValue(const std::vector<double>& values, std::string* why);
  void SetNoiseType(const std::string& type);
  NoiseType GetNoiseType() const { return noise_type_; }
  bool HasNoise() const { return noise_type_ != None; }
  void SetNoiseVal(cplx v) { amp_.assign(size(), v); }
  bool SetNoiseVal(const std::vector<double>& values, std::string* why);
  void SetTemporalValue(const std::map<double, std::vector<double>>& data);

  bool IsSetup() const { return setup_; }
  bool HasTimeDependence() const { return !times_.empty(); }
  const std::vector<cplx>& base() const { return base_; }
  const std::vector<cplx>& amp() const { return amp_; }
  const std::vector<double>& times() const { return times_; }
  const std::vector<cplx>& time_values() const { return tvals_; }  // records x size()

 private:
  size_t nx_ = 0, ny_ = 0;
  bool setup_ = false;
  NoiseType noise_type_ = None;
  std::vector<cplx> base_, amp_;
  std::vector<double> times_;
  std::vector<cplx> tvals_;
};

// column-major file values -> row-major matrix (EigenUtils.cpp InitMatrix)
bool init_matrix_from_values(size_t nx, size_t ny, const std::vector<double>& values, std::vector<cplx>* out,
                             std::string* why);

}  // namespace pinco
