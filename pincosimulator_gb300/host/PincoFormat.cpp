// PincoFormat.cpp -- see PincoFormat.hpp.
#include "PincoFormat.hpp"

#include <algorithm>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <stdexcept>

namespace fs = std::filesystem;

namespace pinco {

namespace {
const unsigned char kMagic[8] = {0x89, 'P', 'N', 'C', 0x0d, 0x0a, 0x1a, 0x0a};
const unsigned char kVersion = 1;
constexpr size_t kExtra = 2 * sizeof(double);

[[noreturn]] void fail(const std::string& m) { throw std::runtime_error("pinco archive: " + m); }

template <typename T>
void rd(FILE* f, T* v, const char* what) {
  if (std::fread(v, sizeof(T), 1, f) != 1) fail(std::string("truncated ") + what);
}
}  // namespace

PincoArchive::PincoArchive(const std::string& data_dir, double chunk_size_gb) : dir_(data_dir) {
  fs::create_directories(dir_);
  chunk_limit_ = chunk_size_gb > 0 ? size_t(chunk_size_gb * 1024.0 * 1024.0 * 1024.0) : size_t(1) << 30;
  const std::string path = dir_ + "/_register.bin";
  if (!fs::exists(path)) {
    reg_ = std::fopen(path.c_str(), "wb+");
    if (!reg_) fail("cannot create " + path);
    return;
  }
  reg_ = std::fopen(path.c_str(), "rb+");
  if (!reg_) fail("cannot open " + path);
  unsigned char magic[8], ver;
  if (std::fread(magic, 1, 8, reg_) != 8 || std::memcmp(magic, kMagic, 8) != 0) fail("bad magic in " + path);
  rd(reg_, &ver, "version");
  const int nd = std::fgetc(reg_);
  if (nd == EOF) fail("truncated header");
  names_.resize(size_t(nd));
  for (auto& nm : names_) {
    const int len = std::fgetc(reg_);
    if (len == EOF) fail("truncated name");
    nm.resize(size_t(len));
    if (len && std::fread(&nm[0], 1, size_t(len), reg_) != size_t(len)) fail("truncated name");
  }
  for (int i = 0; i < nd; ++i) {
    size_t D;
    rd(reg_, &D, "dims");
    if (D > 16) fail("implausible dimension count");
    std::vector<size_t> dv(D);
    if (D && std::fread(dv.data(), sizeof(size_t), D, reg_) != D) fail("truncated dims");
    dims_.push_back(dv);
  }
  for (int i = 0; i < nd; ++i) {
    const int f = std::fgetc(reg_);
    if (f == EOF) fail("truncated formats");
    formats_.push_back((unsigned char)f);
  }
  long extra_size;
  rd(reg_, &extra_size, "extra size");
  if (extra_size != long(kExtra)) fail("unexpected extra-data size");
  rd(reg_, &first_entry_, "entry offset");
  header_ = true;
  std::fseek(reg_, first_entry_, SEEK_SET);
  for (;;) {
    Entry e;
    e.register_pos = std::ftell(reg_);
    size_t w[4];
    if (std::fread(w, sizeof(size_t), 4, reg_) != 4) break;
    if (std::fread(e.extra, sizeof(double), 2, reg_) != 2) fail("truncated register entry");
    e.traj_id = w[0]; e.chunk_id = w[1]; e.chunk_offset = w[2]; e.continuation_offset = w[3];
    entries_.push_back(e);
    chunk_ids_.insert(e.chunk_id);
  }
  std::fseek(reg_, 0, SEEK_END);
}

PincoArchive::~PincoArchive() {
  if (cur_) close_chunk(cur_.get());
  if (reg_) std::fclose(reg_);
}

void PincoArchive::close_chunk(ChunkSet* c) {
  for (FILE* f : c->files) if (f) std::fclose(f);
  if (c->index) std::fclose(c->index);
  c->files.clear();
  c->index = nullptr;
}

std::set<size_t> PincoArchive::UsedIds() const {
  std::set<size_t> s;
  for (auto& e : entries_) s.insert(e.traj_id);
  return s;
}

void PincoArchive::write_header(const TWMCResults& r) {
  std::fseek(reg_, 0, SEEK_SET);
  std::fwrite(kMagic, 1, 8, reg_);
  std::fwrite(&kVersion, 1, 1, reg_);
  names_.clear();
  dims_.clear();
  formats_.clear();
  std::fputc(int(r.datasets.size()), reg_);
  for (auto& d : r.datasets) {
    names_.push_back(d.name);
    std::fputc(int(d.name.size()), reg_);
    std::fwrite(d.name.data(), 1, d.name.size(), reg_);
  }
  for (auto& d : r.datasets) {
    const size_t D = d.dims.size();
    std::fwrite(&D, sizeof(size_t), 1, reg_);
    std::fwrite(d.dims.data(), sizeof(size_t), D, reg_);
    dims_.push_back(d.dims);
  }
  for (auto& d : r.datasets) { std::fputc(d.format, reg_); formats_.push_back(d.format); }
  const long extra = long(kExtra);
  std::fwrite(&extra, sizeof(long), 1, reg_);
  first_entry_ = std::ftell(reg_) + long(sizeof(long));
  std::fwrite(&first_entry_, sizeof(long), 1, reg_);
  std::fflush(reg_);
  header_ = true;
}

PincoArchive::ChunkSet* PincoArchive::writable_chunk() {
  if (cur_ && cur_->total <= chunk_limit_) return cur_.get();
  if (cur_) close_chunk(cur_.get());
  // new id = largest used id + 1; an archive without chunks starts at 1
  const size_t id = chunk_ids_.empty() ? 1 : *chunk_ids_.rbegin() + 1;
  chunk_ids_.insert(id);
  cur_ = std::make_unique<ChunkSet>();
  cur_->id = id;
  for (size_t i = 0; i < names_.size(); ++i) {
    const std::string p = dir_ + "/variable" + std::to_string(i) + "_" + std::to_string(id) + ".cnk";
    FILE* f = std::fopen(p.c_str(), "wb+");
    if (!f) fail("cannot create " + p);
    cur_->files.push_back(f);
  }
  const std::string ip = dir_ + "/index_" + std::to_string(id) + ".bin";
  cur_->index = std::fopen(ip.c_str(), "wb+");
  if (!cur_->index) fail("cannot create " + ip);
  return cur_.get();
}

void PincoArchive::Store(const TWMCResults& r) {
  if (!header_) write_header(r);
  if (r.datasets.size() != names_.size()) fail("dataset count differs from the register");
  ChunkSet* c = writable_chunk();
  std::vector<size_t> row(1 + 2 * names_.size(), 0);
  row[0] = r.GetId();
  for (size_t i = 0; i < r.datasets.size(); ++i) {
    const Dataset& d = r.datasets[i];
    auto it = std::find(names_.begin(), names_.end(), d.name);
    if (it == names_.end()) fail("dataset " + d.name + " is not in the register");
    const size_t j = size_t(it - names_.begin());
    FILE* f = c->files[j];
    const long start = std::ftell(f);
    const bool real = formats_[j] == 11;
    const size_t bytes = real ? d.rdata.size() * sizeof(double) : d.data.size() * sizeof(cplx);
    std::fwrite(&bytes, sizeof(size_t), 1, f);
    if (real) std::fwrite(d.rdata.data(), 1, bytes, f);
    else std::fwrite(d.data.data(), 1, bytes, f);
    std::fflush(f);
    const long end = std::ftell(f);
    c->total += size_t(end - start + 1);  // the reference's size accounting
    row[1 + 2 * j] = d.frames;
    row[2 + 2 * j] = size_t(start);
  }
  std::fwrite(row.data(), sizeof(size_t), row.size(), c->index);
  std::fflush(c->index);
  const size_t chunk_row = c->rows++;
  // register entry; a continuation patches the previous final entry
  std::fseek(reg_, 0, SEEK_END);
  Entry e;
  e.traj_id = r.GetId();
  e.chunk_id = c->id;
  e.chunk_offset = chunk_row;
  e.continuation_offset = 0;
  e.extra[0] = r.extra[0];
  e.extra[1] = r.extra[1];
  e.register_pos = std::ftell(reg_);
  const size_t w[4] = {e.traj_id, e.chunk_id, e.chunk_offset, 0};
  std::fwrite(w, sizeof(size_t), 4, reg_);
  std::fwrite(e.extra, sizeof(double), 2, reg_);
  long prev = -1;
  for (size_t k = 0; k < entries_.size(); ++k)
    if (entries_[k].traj_id == e.traj_id) prev = long(k);
  if (prev >= 0) {
    entries_[size_t(prev)].continuation_offset = size_t(e.register_pos);
    std::fseek(reg_, entries_[size_t(prev)].register_pos + long(3 * sizeof(size_t)), SEEK_SET);
    const size_t co = size_t(e.register_pos);
    std::fwrite(&co, sizeof(size_t), 1, reg_);
    std::fseek(reg_, 0, SEEK_END);
  }
  std::fflush(reg_);
  entries_.push_back(e);
  chunk_ids_.insert(c->id);
}

std::unique_ptr<TWMCResults> PincoArchive::Load(size_t id, bool last_frame_only) const {
  std::vector<const Entry*> chain;
  for (auto& e : entries_) if (e.traj_id == id) chain.push_back(&e);
  if (chain.empty()) return nullptr;
  if (last_frame_only) { const Entry* last = chain.back(); chain.assign(1, last); }
  auto res = std::make_unique<TWMCResults>();
  res->SetId(id);
  res->extra[0] = chain.front()->extra[0];
  for (const Entry* e : chain) {
    const std::string ip = dir_ + "/index_" + std::to_string(e->chunk_id) + ".bin";
    FILE* fi = std::fopen(ip.c_str(), "rb");
    if (!fi) fail("missing " + ip);
    std::vector<size_t> row(1 + 2 * names_.size());
    std::fseek(fi, long(e->chunk_offset * row.size() * sizeof(size_t)), SEEK_SET);
    const size_t got = std::fread(row.data(), sizeof(size_t), row.size(), fi);
    std::fclose(fi);
    if (got != row.size()) fail("truncated index " + ip);
    for (size_t j = 0; j < names_.size(); ++j) {
      const std::string cp = dir_ + "/variable" + std::to_string(j) + "_" + std::to_string(e->chunk_id) + ".cnk";
      FILE* fc = std::fopen(cp.c_str(), "rb");
      if (!fc) fail("missing " + cp);
      size_t nel = row[1 + 2 * j];
      std::fseek(fc, long(row[2 + 2 * j]), SEEK_SET);
      size_t bytes = 0;
      if (std::fread(&bytes, sizeof(size_t), 1, fc) != 1) { std::fclose(fc); fail("truncated chunk " + cp); }
      if (last_frame_only && nel > 1) {
        const size_t el = bytes / nel;
        std::fseek(fc, long(el * (nel - 1)), SEEK_CUR);
        bytes = el;
        nel = 1;
      }
      const bool real = formats_[j] == 11;
      std::vector<cplx> data(real ? 0 : bytes / sizeof(cplx));
      std::vector<double> rdata(real ? bytes / sizeof(double) : 0);
      const size_t rb = bytes ? std::fread(real ? static_cast<void*>(rdata.data()) : static_cast<void*>(data.data()),
                                           1, bytes, fc)
                              : 0;
      std::fclose(fc);
      if (rb != bytes) fail("truncated chunk record in " + cp);
      Dataset* dst = nullptr;
      for (auto& d : res->datasets) if (d.name == names_[j]) dst = &d;
      if (!dst) {
        Dataset d;
        d.name = names_[j];
        d.format = formats_[j];
        d.dims = dims_[j];
        d.frames = 0;
        res->datasets.push_back(d);
        dst = &res->datasets.back();
      }
      const bool series = names_[j] == "traj" || names_[j] == "work" || names_[j] == "area";
      if (series) {  // frame series append across continuations, realisations are replaced
        dst->data.insert(dst->data.end(), data.begin(), data.end());
        dst->rdata.insert(dst->rdata.end(), rdata.begin(), rdata.end());
        dst->frames += nel;
      } else {
        dst->data = data;
        dst->rdata = rdata;
        dst->frames = nel;
      }
    }
    res->extra[1] = e->extra[1];
  }
  return res;
}

void SaveRealColumn(const std::string& path, const std::vector<double>& v) {
  std::ofstream f(path);
  f << "%\tformat:real\tcols:1\trows:" << v.size() << "\n";
  for (double x : v) f << x << "\n";
}

void SaveComplexRows(const std::string& path, const std::vector<std::vector<cplx>>& rows) {
  std::ofstream f(path);
  f << "%\tformat:complex\tcols:x\trows:" << rows.size() << "\n";
  for (auto& r : rows) {
    for (auto& x : r) f << x.real() << "\t" << x.imag() << "\t";
    f << "\n";
  }
}

}  // namespace pinco
