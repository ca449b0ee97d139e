// Settings.cpp -- see Settings.hpp.
#include "Settings.hpp"

#include <cctype>
#include <cmath>
#include <cstdlib>
#include <ctime>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <sstream>

namespace fs = std::filesystem;

namespace pinco {

namespace {

struct Cursor {
  const std::string& s;
  size_t i = 0;
  int line = 1;
  std::string origin;
  explicit Cursor(const std::string& t, std::string o) : s(t), origin(std::move(o)) {}
  bool eof() const { return i >= s.size(); }
  char peek() const { return eof() ? '\0' : s[i]; }
  [[noreturn]] void fail(const std::string& msg) const {
    throw ConfigError(origin + ":" + std::to_string(line) + ": " + msg);
  }
  void skip_ws() {
    while (!eof() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\r')) ++i;
  }
  // whitespace, newlines and comments
  void skip_all() {
    for (;;) {
      skip_ws();
      if (peek() == '#') { while (!eof() && s[i] != '\n') ++i; }
      if (peek() == '\n') { ++i; ++line; continue; }
      break;
    }
  }
  void end_of_line() {
    skip_ws();
    if (peek() == '#') while (!eof() && s[i] != '\n') ++i;
    if (eof()) return;
    if (s[i] != '\n') fail("unexpected text after value");
    ++i;
    ++line;
  }
};

std::string parse_quoted(Cursor& c) {
  const char q = c.peek();
  ++c.i;
  std::string out;
  while (!c.eof() && c.peek() != q) {
    char ch = c.s[c.i++];
    if (ch == '\n') c.fail("newline in string");
    if (q == '"' && ch == '\\') {
      if (c.eof()) c.fail("bad escape");
      char e = c.s[c.i++];
      switch (e) {
        case 'n': out += '\n'; break;
        case 't': out += '\t'; break;
        case '\\': out += '\\'; break;
        case '"': out += '"'; break;
        default: out += e;
      }
    } else {
      out += ch;
    }
  }
  if (c.eof()) c.fail("unterminated string");
  ++c.i;
  return out;
}

bool is_bare(char ch) { return std::isalnum(static_cast<unsigned char>(ch)) || ch == '_' || ch == '-'; }

std::string parse_key(Cursor& c) {
  std::string key;
  for (;;) {
    c.skip_ws();
    if (c.peek() == '"' || c.peek() == '\'') {
      key += parse_quoted(c);
    } else {
      size_t st = c.i;
      while (!c.eof() && is_bare(c.peek())) ++c.i;
      if (st == c.i) c.fail("expected a key");
      key += c.s.substr(st, c.i - st);
    }
    c.skip_ws();
    if (c.peek() == '.') { key += '.'; ++c.i; continue; }
    return key;
  }
}

bool parse_number(const std::string& tok, TomlValue* v) {
  std::string t;
  for (char ch : tok) if (ch != '_') t += ch;
  if (t.empty()) return false;
  const std::string low = [&] { std::string r = t; for (auto& ch : r) ch = char(std::tolower(ch)); return r; }();
  if (low == "inf" || low == "+inf" || low == "-inf" || low == "nan" || low == "+nan" || low == "-nan") {
    v->kind = TomlValue::Float;
    v->d = low.find("nan") != std::string::npos ? NAN : (low[0] == '-' ? -INFINITY : INFINITY);
    return true;
  }
  bool is_float = t.find_first_of(".eE") != std::string::npos;
  char* end = nullptr;
  if (!is_float) {
    errno = 0;
    long long x = std::strtoll(t.c_str(), &end, 10);
    if (end && *end == '\0' && errno == 0) { v->kind = TomlValue::Int; v->i = x; v->d = double(x); return true; }
    return false;
  }
  double x = std::strtod(t.c_str(), &end);
  if (end && *end == '\0') { v->kind = TomlValue::Float; v->d = x; return true; }
  return false;
}

TomlValue parse_value(Cursor& c) {
  c.skip_ws();
  TomlValue v;
  const char ch = c.peek();
  if (ch == '"' || ch == '\'') {
    v.kind = TomlValue::String;
    v.s = parse_quoted(c);
    return v;
  }
  if (ch == '[') {
    ++c.i;
    v.kind = TomlValue::Array;
    for (;;) {
      c.skip_all();
      if (c.peek() == ']') { ++c.i; break; }
      TomlValue e = parse_value(c);
      if (e.kind != TomlValue::Int && e.kind != TomlValue::Float) c.fail("only numeric arrays are supported");
      v.arr.push_back(e.d);
      c.skip_all();
      if (c.peek() == ',') { ++c.i; continue; }
      if (c.peek() == ']') { ++c.i; break; }
      c.fail("expected ',' or ']' in array");
    }
    return v;
  }
  size_t st = c.i;
  while (!c.eof() && !std::isspace(static_cast<unsigned char>(c.peek())) && c.peek() != ',' && c.peek() != ']' &&
         c.peek() != '#')
    ++c.i;
  const std::string tok = c.s.substr(st, c.i - st);
  if (tok == "true" || tok == "false") { v.kind = TomlValue::Bool; v.b = tok == "true"; return v; }
  if (!parse_number(tok, &v)) c.fail("cannot parse value '" + tok + "'");
  return v;
}

std::string read_file(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw ConfigError("cannot open " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  return ss.str();
}

}  // namespace

std::map<std::string, TomlValue> parse_toml(const std::string& text, const std::string& origin) {
  std::map<std::string, TomlValue> out;
  Cursor c(text, origin);
  std::string table;
  for (;;) {
    c.skip_all();
    if (c.eof()) break;
    if (c.peek() == '[') {
      ++c.i;
      table = parse_key(c);
      c.skip_ws();
      if (c.peek() != ']') c.fail("expected ']'");
      ++c.i;
      c.end_of_line();
      continue;
    }
    std::string key = parse_key(c);
    c.skip_ws();
    if (c.peek() != '=') c.fail("expected '=' after key '" + key + "'");
    ++c.i;
    TomlValue v = parse_value(c);
    out[table.empty() ? key : table + "." + key] = v;
    c.end_of_line();
  }
  return out;
}

Settings::Settings(int argc, const char* const* argv) {
  std::string input, output;
  std::vector<std::pair<std::string, std::string>> ov;
  std::vector<std::string> rest;
  for (int k = 1; k < argc; ++k) {
    const std::string a = argv[k];
    if ((a == "-i" || a == "--input") && k + 1 < argc) input = argv[++k];
    else if ((a == "-o" || a == "--output" || a == "-a" || a == "--append") && k + 1 < argc) output = argv[++k];
    else rest.push_back(a);
  }
  if (input.empty() && !rest.empty()) { input = rest.front(); rest.erase(rest.begin()); }
  if (input.empty()) throw ConfigError("an input file (-i) is required");
  if (rest.size() % 2 != 0) throw ConfigError("overridden parameters must have argument!");
  for (size_t k = 0; k < rest.size(); k += 2) ov.emplace_back(rest[k], rest[k + 1]);
  load(input, ov, output);
}

Settings::Settings(const std::string& input_path, const std::vector<std::pair<std::string, std::string>>& overrides,
                   const std::string& output_path) {
  load(input_path, overrides, output_path);
}

void Settings::load(const std::string& input, const std::vector<std::pair<std::string, std::string>>& overrides,
                    const std::string& output) {
  fs::path in = input;
  fs::path out = output;
  if (fs::is_directory(in)) {
    out = in;
    in = in / "_sim.ini";
    subsequent_ = fs::exists(in);
  } else if (!fs::exists(in)) {
    throw ConfigError("input file does not exist: " + input);
  }
  if (out.empty()) out = in.parent_path();
  if (out.empty()) out = ".";
  input_ = in.string();
  output_ = out.string();
  input_parent_ = in.parent_path().string();
  cfg_ = parse_toml(read_file(input_), input_);
  if (!overrides.empty()) {
    std::string text;
    for (auto& kv : overrides) text += kv.first + " = " + kv.second + "\n";
    for (auto& kv : parse_toml(text, "<command line>")) cfg_[kv.first] = kv.second;
  }
}

const TomlValue* Settings::find(const std::string& key) const {
  auto it = cfg_.find(key);
  return it == cfg_.end() ? nullptr : &it->second;
}

double Settings::getDouble(const std::string& key, double def) const {
  const TomlValue* v = find(key);
  if (!v || (v->kind != TomlValue::Int && v->kind != TomlValue::Float)) return def;
  return v->d;
}

long long Settings::getInt(const std::string& key, long long def) const {
  const TomlValue* v = find(key);
  return (v && v->kind == TomlValue::Int) ? v->i : def;
}

size_t Settings::getSize(const std::string& key, size_t def) const {
  const TomlValue* v = find(key);
  return (v && v->kind == TomlValue::Int && v->i >= 0) ? size_t(v->i) : def;
}

bool Settings::getBool(const std::string& key, bool def) const {
  const TomlValue* v = find(key);
  return (v && v->kind == TomlValue::Bool) ? v->b : def;
}

std::string Settings::getString(const std::string& key, const std::string& def) const {
  const TomlValue* v = find(key);
  return (v && v->kind == TomlValue::String) ? v->s : def;
}

std::complex<double> Settings::getComplex(const std::string& key, bool* ok) const {
  const TomlValue* v = find(key);
  if (v && (v->kind == TomlValue::Int || v->kind == TomlValue::Float)) { *ok = true; return {v->d, 0.0}; }
  const TomlValue* re = find(key + ".real");
  const TomlValue* im = find(key + ".imag");
  auto num = [](const TomlValue* x) { return x && (x->kind == TomlValue::Int || x->kind == TomlValue::Float); };
  if (num(re) || num(im)) { *ok = true; return {num(re) ? re->d : 0.0, num(im) ? im->d : 0.0}; }
  *ok = false;
  return {0.0, 0.0};
}

std::string Settings::GetRootFolder() const {
  std::string r = getString("rootFolder", input_parent_);
  return r.empty() ? "." : r;
}

unsigned int Settings::GlobalSeed() const {
  unsigned int s = unsigned(getInt("SEED", 0));
  if (getBool("seed_time", false)) s += unsigned(std::time(nullptr));
  return s;
}

NoisyMatrix Settings::GetMatrix(const std::string& path, size_t nx, size_t ny, size_t cellSz) const {
  NoisyMatrix m(nx, ny, cellSz);
  const fs::path root = GetRootFolder();
  std::string why;
  auto load_file = [&](const std::string& rel) {
    const fs::path p = root / rel;
    if (!fs::exists(p)) throw ConfigError("matrix " + path + ": file not found: " + p.string());
    if (!m.SetValue(ReadCharFile(p.string()), &why)) throw ConfigError("matrix " + path + ": " + why);
  };
  auto load_temporal = [&](const std::string& rel) {
    const fs::path p = root / rel;
    if (!fs::exists(p)) throw ConfigError("matrix " + path + ": time table not found: " + p.string());
    m.SetTemporalValue(ReadTemporalCharFile(p.string()));
  };
  if (has(path + ".data")) {
    const TomlValue* v = find(path + ".data");
    if (v->kind == TomlValue::Array) {
      if (!m.SetValue(v->arr, &why)) throw ConfigError("matrix " + path + ".data: " + why);
    } else {
      m.SetValue(cplx(getDouble(path + ".data"), 0.0));
    }
  } else if (has(path + ".file")) {
    load_file(getString(path + ".file"));
  } else if (has(path + ".t")) {
    load_temporal(getString(path + ".t"));
  } else if (has(path + "_t")) {
    load_temporal(getString(path + "_t"));
  } else if (has(path + ".real")) {
    m.SetValue(cplx(getDouble(path + ".real"), getDouble(path + ".imag")));
  } else {
    const TomlValue* v = find(path);
    bool ok = false;
    if (v && v->kind == TomlValue::String) {
      load_file(v->s);
    } else {
      cplx val = getComplex(path, &ok);
      if (ok) m.SetValue(val);
    }
  }
  // noise
  const bool dotted = has(path + ".Noise_Type");
  const std::string sep = dotted ? "." : "_";
  const std::string type = getString(path + sep + "Noise_Type", "xxx");
  if (type != "xxx") {
    m.SetNoiseType(type);
    if (m.HasNoise()) {
      const std::string key = path + sep + "Noise_Val_0";
      const TomlValue* nv = find(key);
      bool ok = false;
      if (nv && nv->kind == TomlValue::String && fs::exists(root / nv->s)) {
        if (!m.SetNoiseVal(ReadCharFile((root / nv->s).string()), &why)) throw ConfigError(key + ": " + why);
      } else {
        cplx val = getComplex(key, &ok);
        if (!ok) throw ConfigError("Variable " + key + " was not set, but was necessary.");
        m.SetNoiseVal(val);
      }
    }
  }
  return m;
}

std::vector<double> ReadCharFile(const std::string& path) {
  std::ifstream f(path);
  std::vector<double> v;
  double x;
  while (f >> x) v.push_back(x);
  return v;
}

std::map<double, std::vector<double>> ReadTemporalCharFile(const std::string& path) {
  std::map<double, std::vector<double>> result;
  std::ifstream in(path);
  std::string line;
  double time = 0.0;
  while (std::getline(in, line)) {
    std::istringstream iss(line);
    iss >> time;
    std::vector<double> arr;
    while (std::getline(in, line)) {
      if (line.empty() || line == "-" || line == " " || line == "\t" || line == "\r") break;
      std::istringstream ls(line);
      std::string st;
      while (ls >> st) {
        if (st == "*" || st == "nan" || st == "NAN" || st == "NaN") arr.push_back(NAN);
        else arr.push_back(double(std::stof(st)));  // values are read at float precision, as the reference does
      }
    }
    result.emplace(time, arr);
  }
  return result;
}

}  // namespace pinco
