#include "xh5c.h"

#include <cstdio>
#include <cstring>
#include <stdexcept>

namespace xh5c {

uint64_t Dataset::count() const {
  uint64_t n = 1;
  for (uint64_t x : dims) n *= x;
  return n;
}

static bool rd(FILE *f, void *p, size_t n) { return n == 0 || fread(p, 1, n, f) == n; }

bool File::load(const std::string &path) {
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

bool File::save(const std::string &path) const {
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
  return it == sets_.end() ? nullptr : &it->second;
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
