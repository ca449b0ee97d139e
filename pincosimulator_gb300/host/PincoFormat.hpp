// PincoFormat.hpp -- the reference's chunked binary results archive.
//
// Byte layout (src/Base/FileFormats/PincoFormat/ChunkRegister.cpp:152-233,
// 312-380; ChunkFileSet.cpp:58-224), all integers little-endian size_t /
// long (8 bytes):
//   data/_register.bin
//     magic 89 'P' 'N' 'C' 0D 0A 1A 0A, version byte 1,
//     dataset count (1 byte), per dataset: name length (1 byte) + name,
//     per dataset: D then D dims, per dataset: format id (1 byte;
//     22 = complex128, 11 = float64), long extra-data size (16),
//     long offset of the first entry,
//     entries {traj_id, chunk_id, chunk_offset, continuation_offset,
//              t_start, t_end (doubles)}
//   data/index_<c>.bin      rows {id, (elements, byte offset) per dataset}
//   data/variable<i>_<c>.cnk records [size_t bytes][payload]
// chunk_offset is the row of the index file; continuation_offset is the
// register position of the entry that continues a trajectory (0 if none).
// A new chunk set starts when the current one exceeds chunk_size GB.
#pragma once

#include <cstdio>
#include <map>
#include <memory>
#include <set>
#include <string>
#include <vector>

#include "TWMC.hpp"

namespace pinco {

class PincoArchive {
 public:
  struct Entry {
    size_t traj_id = 0, chunk_id = 0, chunk_offset = 0, continuation_offset = 0;
    double extra[2] = {0, 0};
    long register_pos = 0;
  };

  // Opens data_dir/_register.bin if it exists (reading every entry), else
  // prepares a new archive; the header is written with the first Store.
  explicit PincoArchive(const std::string& data_dir, double chunk_size_gb = 1.5);
  ~PincoArchive();

  void Store(const TWMCResults& r);
  // Last frame (last_frame_only) or the whole trajectory with continuations.
  std::unique_ptr<TWMCResults> Load(size_t id, bool last_frame_only) const;

  std::set<size_t> UsedIds() const;
  const std::vector<Entry>& entries() const { return entries_; }
  const std::vector<std::string>& dataset_names() const { return names_; }

 private:
  struct ChunkSet {
    size_t id = 0;
    std::vector<FILE*> files;
    FILE* index = nullptr;
    size_t rows = 0;
    size_t total = 0;
  };
  void write_header(const TWMCResults& r);
  ChunkSet* writable_chunk();
  void close_chunk(ChunkSet* c);
  std::string dir_;
  size_t chunk_limit_ = 0;
  FILE* reg_ = nullptr;
  bool header_ = false;
  std::vector<std::string> names_;
  std::vector<std::vector<size_t>> dims_;
  std::vector<unsigned char> formats_;
  long first_entry_ = 0;
  std::vector<Entry> entries_;
  std::set<size_t> chunk_ids_;
  std::unique_ptr<ChunkSet> cur_;
};

// Text side files (src/Base/FileFormats/DataStore.cpp:70-137).
void SaveRealColumn(const std::string& path, const std::vector<double>& v);
void SaveComplexRows(const std::string& path, const std::vector<std::vector<cplx>>& rows);

}  // namespace pinco
