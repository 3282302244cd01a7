#include "xh5c.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <stdexcept>

#include "h5lite.h"

namespace xh5c {

namespace {

// HDF5 element kinds and sizes <-> container element types; kinds without a
// container type of their own widen (i8 -> i16, u8 -> u16, u64 -> i64).
Dataset from_h5(const h5lite::Data &d) {
  Dataset o;
  o.dims = d.dims.empty() ? std::vector<uint64_t>{1} : d.dims;
  const uint64_t n = d.count();
  auto widen = [&](uint32_t type, uint32_t to) {
    o.type = type;
    o.bytes.assign(n * to, 0);
    for (uint64_t i = 0; i < n; i++) {
      uint64_t u = 0;
      for (int k = (int)d.size - 1; k >= 0; k--) u = (u << 8) | d.bytes[i * d.size + k];
      if (d.kind == h5lite::Kind::Int && (u >> (8 * d.size - 1)) && d.size < 8)
        u |= ~0ull << (8 * d.size);
      memcpy(&o.bytes[i * to], &u, to);
    }
  };
  switch (d.kind) {
    case h5lite::Kind::String:
      o.type = STR;
      o.dims = {1};
      o.bytes = d.bytes;
      break;
    case h5lite::Kind::Float:
      o.type = d.size == 4 ? F32 : F64;
      o.bytes = d.bytes;
      break;
    case h5lite::Kind::Int:
      if (d.size == 4) {
        o.type = I32;
        o.bytes = d.bytes;
      } else if (d.size == 8) {
        o.type = I64;
        o.bytes = d.bytes;
      } else if (d.size == 2) {
        o.type = I16;
        o.bytes = d.bytes;
      } else {
        widen(I16, 2);
      }
      break;
    case h5lite::Kind::UInt:
      if (d.size == 4) {
        o.type = U32;
        o.bytes = d.bytes;
      } else if (d.size == 2) {
        o.type = U16;
        o.bytes = d.bytes;
      } else if (d.size == 8) {
        widen(I64, 8);
      } else {
        widen(U16, 2);
      }
      break;
  }
  return o;
}

h5lite::Data to_h5(const Dataset &d) {
  h5lite::Data o;
  o.dims = d.dims;
  o.bytes = d.bytes;
  switch (d.type) {
    case I32: o.kind = h5lite::Kind::Int; o.size = 4; break;
    case I64: o.kind = h5lite::Kind::Int; o.size = 8; break;
    case I16: o.kind = h5lite::Kind::Int; o.size = 2; break;
    case U32: o.kind = h5lite::Kind::UInt; o.size = 4; break;
    case U16: o.kind = h5lite::Kind::UInt; o.size = 2; break;
    case F32: o.kind = h5lite::Kind::Float; o.size = 4; break;
    case F64: o.kind = h5lite::Kind::Float; o.size = 8; break;
    case STR:  // one string: a scalar dataset as long as the string
      o.kind = h5lite::Kind::String;
      o.dims.clear();
      o.size = (uint32_t)std::max<size_t>(1, d.bytes.size());
      o.bytes.resize(o.size, 0);
      break;
    default: throw std::runtime_error("element type " + std::to_string(d.type));
  }
  return o;
}

}  // namespace

uint64_t Dataset::count() const {
  uint64_t n = 1;
  for (uint64_t x : dims) n *= x;
  return n;
}

static bool rd(FILE *f, void *p, size_t n) { return n == 0 || fread(p, 1, n, f) == n; }

bool File::load(const std::string &path) {
  if (h5lite::is_hdf5(path)) {
    std::map<std::string, h5lite::Data> sets;
    try {
      h5lite::read_all(path, sets, skipped_);
    } catch (const std::exception &e) {
      error_ = e.what();
      return false;
    }
    for (const auto &kv : sets) sets_[kv.first] = from_h5(kv.second);
    hdf5_ = true;
    dirty_.clear();
    return true;
  }
  FILE *f = fopen(path.c_str(), "rb");
  if (!f) return false;
  char magic[4];
  uint32_t version = 0, count = 0;
  bool ok = rd(f, magic, 4) && memcmp(magic, "XH5C", 4) == 0 && rd(f, &version, 4) &&
            rd(f, &count, 4);
  for (uint32_t r = 0; ok && r < count; r++) {
    uint32_t plen = 0, rank = 0;
    uint64_t nbytes = 0;
    Dataset d;
    ok = rd(f, &plen, 4);
    std::string name(plen, '\0');
    ok = ok && rd(f, &name[0], plen) && rd(f, &d.type, 4) && rd(f, &rank, 4);
    if (!ok) break;
    d.dims.resize(rank);
    ok = rd(f, d.dims.data(), 8 * rank) && rd(f, &nbytes, 8);
    if (!ok) break;
    d.bytes.resize(nbytes);
    ok = rd(f, d.bytes.data(), nbytes);
    if (ok) sets_[name] = std::move(d);
  }
  fclose(f);
  return ok;
}

void File::save_hdf5(const std::string &path) const {
  std::map<std::string, h5lite::Data> out;
  for (const auto &kv : sets_) out[kv.first] = to_h5(kv.second);
  h5lite::create(path);
  h5lite::write(path, out);
}

bool File::save(const std::string &path) const {
  if (hdf5_) {
    std::map<std::string, h5lite::Data> out;
    try {
      for (const std::string &p : dirty_) out[p] = to_h5(sets_.at(p));
      h5lite::write(path, out);
    } catch (const std::exception &e) {
      error_ = e.what();
      return false;
    }
    return true;
  }
  std::string tmp = path + ".tmp";
  FILE *f = fopen(tmp.c_str(), "wb");
  if (!f) return false;
  uint32_t version = 1, count = (uint32_t)sets_.size();
  bool ok = fwrite("XH5C", 1, 4, f) == 4 && fwrite(&version, 4, 1, f) == 1 &&
            fwrite(&count, 4, 1, f) == 1;
  for (const auto &kv : sets_) {
    uint32_t plen = (uint32_t)kv.first.size(), rank = (uint32_t)kv.second.dims.size();
    uint64_t nbytes = kv.second.bytes.size();
    ok = ok && fwrite(&plen, 4, 1, f) == 1 && fwrite(kv.first.data(), 1, plen, f) == plen &&
         fwrite(&kv.second.type, 4, 1, f) == 1 && fwrite(&rank, 4, 1, f) == 1 &&
         fwrite(kv.second.dims.data(), 8, rank, f) == rank && fwrite(&nbytes, 8, 1, f) == 1 &&
         fwrite(kv.second.bytes.data(), 1, nbytes, f) == nbytes;
  }
  ok = fclose(f) == 0 && ok;
  return ok && rename(tmp.c_str(), path.c_str()) == 0;
}

bool File::has(const std::string &path) const { return sets_.count(path) != 0; }

const Dataset *File::get(const std::string &path) const {
  auto it = sets_.find(path);
  if (it == sets_.end()) {
    auto sk = skipped_.find(path);
    if (sk != skipped_.end())
      throw std::runtime_error("dataset " + path + " is stored as " + sk->second +
                               ", which this reader does not handle");
    return nullptr;
  }
  return &it->second;
}

std::string File::get_string(const std::string &path) const {
  const Dataset *d = get(path);
  if (!d) throw std::runtime_error("missing dataset " + path);
  std::string s(d->bytes.begin(), d->bytes.end());
  size_t z = s.find('\0');
  return z == std::string::npos ? s : s.substr(0, z);
}

template <class T>
static double as_double(const unsigned char *p) {
  T v;
  memcpy(&v, p, sizeof(T));
  return (double)v;
}

static double elem(const Dataset &d, uint64_t i) {
  switch (d.type) {
    case I32: return as_double<int32_t>(d.bytes.data() + 4 * i);
    case I64: return as_double<int64_t>(d.bytes.data() + 8 * i);
    case F32: return as_double<float>(d.bytes.data() + 4 * i);
    case F64: return as_double<double>(d.bytes.data() + 8 * i);
    case U32: return as_double<uint32_t>(d.bytes.data() + 4 * i);
    case I16: return as_double<int16_t>(d.bytes.data() + 2 * i);
    case U16: return as_double<uint16_t>(d.bytes.data() + 2 * i);
    default: throw std::runtime_error("not a numeric dataset");
  }
}

double File::get_scalar(const std::string &path) const {
  const Dataset *d = get(path);
  if (!d || d->count() == 0) throw std::runtime_error("missing dataset " + path);
  return elem(*d, 0);
}

std::vector<int32_t> File::get_i32(const std::string &path) const {
  const Dataset *d = get(path);
  if (!d) throw std::runtime_error("missing dataset " + path);
  std::vector<int32_t> v(d->count());
  for (uint64_t i = 0; i < v.size(); i++) v[i] = (int32_t)elem(*d, i);
  return v;
}

std::vector<double> File::get_f64(const std::string &path) const {
  const Dataset *d = get(path);
  if (!d) throw std::runtime_error("missing dataset " + path);
  std::vector<double> v(d->count());
  for (uint64_t i = 0; i < v.size(); i++) v[i] = elem(*d, i);
  return v;
}

}  // namespace xh5c
