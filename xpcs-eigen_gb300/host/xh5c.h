// The analysis file of `corr`: its datasets by absolute path, read from and
// written back to either
//   * an HDF5 file (h5lite.h), the reference's format: results are written
//     into the file they were read from, as the reference does; or
//   * an XH5C container, a flat stand-in with the same paths, types and
//     shapes.  Layout (little endian): "XH5C", u32 version (1), u32 record
//     count, then per record: u32 path length, path, u32 element type, u32
//     rank, u64 dims[rank], u64 byte count, payload.  Element types: 1 i32,
//     2 i64, 3 f32, 4 f64, 5 string, 6 u32, 7 i16, 8 u16.  Groups are
//     implicit.
#pragma once

#include <cstdint>
#include <map>
#include <set>
#include <string>
#include <vector>

namespace xh5c {

enum Type : uint32_t { I32 = 1, I64 = 2, F32 = 3, F64 = 4, STR = 5, U32 = 6, I16 = 7, U16 = 8 };

struct Dataset {
  uint32_t type = 0;
  std::vector<uint64_t> dims;
  std::vector<unsigned char> bytes;
  uint64_t count() const;
};

class File {
 public:
  // Reads an HDF5 file or an XH5C container (by its signature).
  bool load(const std::string &path);
  // Writes back in the format that was loaded: into the HDF5 file (only the
  // datasets put since loading), or a whole XH5C container.
  bool save(const std::string &path) const;
  // A new HDF5 file holding every dataset.
  void save_hdf5(const std::string &path) const;
  bool is_hdf5() const { return hdf5_; }
  const std::string &error() const { return error_; }
  bool has(const std::string &path) const;
  const Dataset *get(const std::string &path) const;
  std::string get_string(const std::string &path) const;  // throws if missing
  double get_scalar(const std::string &path) const;       // first element as double
  std::vector<int32_t> get_i32(const std::string &path) const;
  std::vector<double> get_f64(const std::string &path) const;
  template <class T>
  void put(const std::string &path, Type type, const std::vector<uint64_t> &dims, const T *data);

 private:
  std::map<std::string, Dataset> sets_;
  std::map<std::string, std::string> skipped_;  // HDF5 datasets not read, with the reason
  std::set<std::string> dirty_;                 // put since loading
  bool hdf5_ = false;
  mutable std::string error_;
};

template <class T>
void File::put(const std::string &path, Type type, const std::vector<uint64_t> &dims,
               const T *data) {
  Dataset d;
  d.type = type;
  d.dims = dims;
  uint64_t n = 1;
  for (uint64_t x : dims) n *= x;
  d.bytes.resize(n * sizeof(T));
  if (n) std::copy((const unsigned char *)data, (const unsigned char *)data + n * sizeof(T),
                   d.bytes.begin());
  sets_[path] = d;
  dirty_.insert(path);
}

}  // namespace xh5c
