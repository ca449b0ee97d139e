// Settings.hpp -- run configuration: the .ini (TOML subset) input, command-line
// key/value overrides, typed getters and parameter-matrix resolution.
//
// Mirrors the reference's Settings (src/Base/Settings.cpp:32-187, 211-573):
//   - `-i input.ini [-o output] [key value]...`; a folder input means
//     <folder>/_sim.ini with the folder as output; overrides are parsed as
//     `key = value` lines and merged over the file.
//   - Typed getters default to 0 / false / "" (or the given default);
//     floating getters accept integer values, integer getters do not.
//   - GetMatrix(name, nx, ny, cellSz) resolves name.data, name.file, name.t or
//     name_t (time table), name.real/.imag, a bare string (file relative to
//     the root folder) or a bare number, then name.Noise_Type /
//     name.Noise_Val_<i> (or the name_Noise_Type back-support keys).
// The TOML subset: `key = value` with bare, dotted or quoted keys, numbers,
// booleans, strings, flat numeric arrays, `[table]` headers (keys flattened as
// `table.key`) and `#` comments. Dotted keys are stored flat, so `U.Noise_Type`
// and `"U.Noise_Type"` name the same entry.
#pragma once

#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "NoisyMatrix.hpp"

namespace pinco {

struct TomlValue {
  enum Kind { Int, Float, Bool, String, Array } kind = Int;
  long long i = 0;
  double d = 0;
  bool b = false;
  std::string s;
  std::vector<double> arr;
};

class ConfigError : public std::runtime_error {
 public:
  using std::runtime_error::runtime_error;
};

// Parses TOML-subset text into flat key -> value entries (later keys win).
std::map<std::string, TomlValue> parse_toml(const std::string& text, const std::string& origin);

class Settings {
 public:
  // argv-style construction, like the reference's Settings(argc, argv).
  Settings(int argc, const char* const* argv);
  // Direct construction from a file and override pairs.
  Settings(const std::string& input_path, const std::vector<std::pair<std::string, std::string>>& overrides,
           const std::string& output_path = "");

  bool has(const std::string& key) const { return cfg_.count(key) != 0; }
  const TomlValue* find(const std::string& key) const;

  double getDouble(const std::string& key, double def = 0.0) const;
  long long getInt(const std::string& key, long long def = 0) const;
  size_t getSize(const std::string& key, size_t def = 0) const;
  bool getBool(const std::string& key, bool def = false) const;
  std::string getString(const std::string& key, const std::string& def = "") const;
  // number or name.real / name.imag pair; `ok` false when neither is set
  std::complex<double> getComplex(const std::string& key, bool* ok) const;

  NoisyMatrix GetMatrix(const std::string& name, size_t nx, size_t ny, size_t cellSz = 1) const;

  // SEED from the input (the reference adds time(0); that term is dropped
  // so that runs are reproducible unless `seed_time = true`).
  unsigned int GlobalSeed() const;

  std::string GetRootFolder() const;
  std::string GetOutputFolder() const { return output_; }
  std::string GetInputPath() const { return input_; }
  bool subsequentRun() const { return subsequent_; }

 private:
  void load(const std::string& input, const std::vector<std::pair<std::string, std::string>>& overrides,
            const std::string& output);
  std::map<std::string, TomlValue> cfg_;
  std::string input_, output_, input_parent_;
  bool subsequent_ = false;
};

// Whitespace-separated numbers of a matrix file (Settings.cpp:563-573).
std::vector<double> ReadCharFile(const std::string& path);
// Time-tabulated records: a time line, value lines, a blank line
// (Settings.cpp:530-561); `*` / `nan` entries are NaN.
std::map<double, std::vector<double>> ReadTemporalCharFile(const std::string& path);

}  // namespace pinco
