// XH5C container: the flat stand-in for the HDF5 analysis file.
//
// Layout (little endian): "XH5C", u32 version (1), u32 record count, then per
// record: u32 path length, path, u32 element type, u32 rank, u64 dims[rank],
// u64 byte count, payload.  Element types: 1 i32, 2 i64, 3 f32, 4 f64,
// 5 string, 6 u32, 7 i16, 8 u16.  Datasets are addressed by absolute path
// ("/xpcs/dqmap"); groups are implicit.
#pragma once

#include <cstdint>
#include <map>
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
  bool load(const std::string &path);
  bool save(const std::string &path) const;
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
}

}  // namespace xh5c
