// NoisyMatrix.cpp -- see NoisyMatrix.hpp.
#include "NoisyMatrix.hpp"

#include <iostream>

namespace pinco {

bool init_matrix_from_values(size_t nx, size_t ny, const std::vector<double>& values, std::vector<cplx>* out,
                             std::string* why) {
  const size_t n = nx * ny;
  out->assign(n, cplx(0, 0));
  if (values.size() == n) {
    for (size_t i = 0; i < nx; ++i)
      for (size_t j = 0; j < ny; ++j) (*out)[i * ny + j] = cplx(values[j * nx + i], 0.0);
    return true;
  }
  if (values.size() == 2 * n) {
    for (size_t i = 0; i < nx; ++i)
      for (size_t j = 0; j < ny; ++j)
        (*out)[i * ny + j] = cplx(values[2 * (j * nx + i)], values[2 * (j * nx + i) + 1]);
    return true;
  }
  if (why)
    *why = "matrix has " + std::to_string(n) + " elements but the data has " + std::to_string(values.size()) +
           " values";
  return false;
}

bool NoisyMatrix::SetValue(const std::vector<double>& values, std::string* why) {
  if (!init_matrix_from_values(nx_, ny_, values, &base_, why)) return false;
  setup_ = true;
  return true;
}

void NoisyMatrix::SetNoiseType(const std::string& type) {
  if (type == "Uniform" || type == "u") noise_type_ = Uniform;
  else if (type == "Gaussian" || type == "g") noise_type_ = Gaussian;
  else if (type == "Lorentzian" || type == "l") noise_type_ = Lorentzian;
  else if (type == "Poissonian" || type == "p") noise_type_ = Poissonian;
  else {
    noise_type_ = None;
    if (type != "None")
      std::cerr << "Unrecognized Noise Type " << type << ". Defaulting to: None." << std::endl;
  }
  if (amp_.empty()) amp_.assign(size(), cplx(0, 0));
}

bool NoisyMatrix::SetNoiseVal(const std::vector<double>& values, std::string* why) {
  return init_matrix_from_values(nx_, ny_, values, &amp_, why);
}

void NoisyMatrix::SetTemporalValue(const std::map<double, std::vector<double>>& data) {
  times_.clear();
  tvals_.clear();
  const size_t n = size();
  for (const auto& kv : data) {
    std::vector<cplx> rec(n, cplx(0, 0));
    if (kv.second.size() == n) {
      for (size_t i = 0; i < n; ++i) rec[i] = cplx(kv.second[i], 0.0);
    } else if (kv.second.size() == 2 * n) {
      for (size_t i = 0; i < n; ++i) rec[i] = cplx(kv.second[2 * i], kv.second[2 * i + 1]);
    } else {
      std::cerr << "Error in parsing a time-dependent matrix. Invalid number of elements." << std::endl;
    }
    times_.push_back(kv.first);
    tvals_.insert(tvals_.end(), rec.begin(), rec.end());
  }
  if (!tvals_.empty()) {
    base_.assign(tvals_.begin(), tvals_.begin() + long(n));
    setup_ = true;
  }
}

}  // namespace pinco
