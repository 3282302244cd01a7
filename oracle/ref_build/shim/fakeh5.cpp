/*
 * Test infrastructure (oracle build only): in-memory implementation of the
 * HDF5 subset declared in hdf5.h.
 *
 * Container format "XH5C" (little endian), read at the first H5Fopen of a path
 * and rewritten in place by every H5Fclose that follows a write:
 *
 *   char[4]  magic "XH5C"
 *   u32      version (1)
 *   u32      record count
 *   records: u32 path length, path bytes (absolute, '/'-separated),
 *            u32 element type (XH5C_* in hdf5.h), u32 rank,
 *            u64 dims[rank], u64 byte count, payload bytes (row major)
 *
 * Strings are stored as XH5C_STR with rank 1, dims {1} and the raw bytes.
 */
#include "hdf5.h"

#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace {

struct Dataset {
  uint32_t type = 0;
  std::vector<hsize_t> dims;
  std::vector<unsigned char> bytes;
};

struct Handle {
  int kind = 0;  // 1 file, 2 group, 3 dataset, 4 dataspace, 5 property list
  std::string path;
  std::vector<hsize_t> dims;
};

struct Store {
  std::map<std::string, Dataset> sets;
  bool dirty = false;
};

std::map<std::string, Store> g_files;
std::map<hid_t, Handle> g_handles;
std::map<hid_t, std::string> g_file_of;  // handle -> container file path
hid_t g_next = 100;

size_t elem_size(uint32_t t) {
  switch (t) {
    case XH5C_I16:
    case XH5C_U16:
      return 2;
    case XH5C_I32:
    case XH5C_F32:
    case XH5C_U32:
      return 4;
    case XH5C_I64:
    case XH5C_F64:
      return 8;
    default:
      return 1;
  }
}

bool read_exact(FILE *f, void *p, size_t n) { return n == 0 || fread(p, 1, n, f) == n; }

void load(const std::string &file, Store &st) {
  FILE *f = fopen(file.c_str(), "rb");
  if (!f) return;
  char magic[4];
  uint32_t version = 0, count = 0;
  if (!read_exact(f, magic, 4) || memcmp(magic, "XH5C", 4) != 0 || !read_exact(f, &version, 4) ||
      !read_exact(f, &count, 4)) {
    fclose(f);
    return;
  }
  for (uint32_t r = 0; r < count; r++) {
    uint32_t plen = 0, rank = 0;
    Dataset d;
    if (!read_exact(f, &plen, 4)) break;
    std::string path(plen, '\0');
    uint64_t nbytes = 0;
    if (!read_exact(f, &path[0], plen) || !read_exact(f, &d.type, 4) || !read_exact(f, &rank, 4))
      break;
    d.dims.resize(rank);
    if (!read_exact(f, d.dims.data(), 8 * rank) || !read_exact(f, &nbytes, 8)) break;
    d.bytes.resize(nbytes);
    if (!read_exact(f, d.bytes.data(), nbytes)) break;
    st.sets[path] = d;
  }
  fclose(f);
}

void save(const std::string &file, const Store &st) {
  std::string tmp = file + ".tmp";
  FILE *f = fopen(tmp.c_str(), "wb");
  if (!f) return;
  uint32_t version = 1, count = (uint32_t)st.sets.size();
  fwrite("XH5C", 1, 4, f);
  fwrite(&version, 4, 1, f);
  fwrite(&count, 4, 1, f);
  for (const auto &kv : st.sets) {
    uint32_t plen = (uint32_t)kv.first.size(), rank = (uint32_t)kv.second.dims.size();
    uint64_t nbytes = kv.second.bytes.size();
    fwrite(&plen, 4, 1, f);
    fwrite(kv.first.data(), 1, plen, f);
    fwrite(&kv.second.type, 4, 1, f);
    fwrite(&rank, 4, 1, f);
    fwrite(kv.second.dims.data(), 8, rank, f);
    fwrite(&nbytes, 8, 1, f);
    fwrite(kv.second.bytes.data(), 1, nbytes, f);
  }
  fclose(f);
  rename(tmp.c_str(), file.c_str());
}

std::string normalize(const std::string &p) {
  std::string out = "/";
  size_t i = 0;
  while (i < p.size()) {
    while (i < p.size() && p[i] == '/') i++;
    size_t j = i;
    while (j < p.size() && p[j] != '/') j++;
    if (j > i) {
      if (out.size() > 1) out += '/';
      out += p.substr(i, j - i);
    }
    i = j;
  }
  return out;
}

std::string resolve(hid_t loc, const char *name) {
  std::string n = name ? name : "";
  if (!n.empty() && n[0] == '/') return normalize(n);
  auto it = g_handles.find(loc);
  std::string base = it == g_handles.end() ? "/" : it->second.path;
  return normalize(base + "/" + n);
}

Store *store_of(hid_t h) {
  auto it = g_file_of.find(h);
  if (it == g_file_of.end()) return nullptr;
  return &g_files[it->second];
}

Dataset *dataset_of(hid_t h) {
  Store *st = store_of(h);
  auto it = g_handles.find(h);
  if (!st || it == g_handles.end() || it->second.kind != 3) return nullptr;
  auto ds = st->sets.find(it->second.path);
  return ds == st->sets.end() ? nullptr : &ds->second;
}

hid_t new_handle(int kind, const std::string &path, hid_t parent) {
  hid_t h = g_next++;
  Handle hd;
  hd.kind = kind;
  hd.path = path;
  g_handles[h] = hd;
  auto f = g_file_of.find(parent);
  if (f != g_file_of.end()) g_file_of[h] = f->second;
  return h;
}

double load_elem(const unsigned char *p, uint32_t t) {
  switch (t) {
    case XH5C_I16: { int16_t v; memcpy(&v, p, 2); return v; }
    case XH5C_U16: { uint16_t v; memcpy(&v, p, 2); return v; }
    case XH5C_I32: { int32_t v; memcpy(&v, p, 4); return v; }
    case XH5C_U32: { uint32_t v; memcpy(&v, p, 4); return v; }
    case XH5C_I64: { int64_t v; memcpy(&v, p, 8); return (double)v; }
    case XH5C_F32: { float v; memcpy(&v, p, 4); return v; }
    case XH5C_F64: { double v; memcpy(&v, p, 8); return v; }
    default: return 0.0;
  }
}

void store_elem(unsigned char *p, uint32_t t, double v) {
  switch (t) {
    case XH5C_I16: { int16_t x = (int16_t)v; memcpy(p, &x, 2); break; }
    case XH5C_U16: { uint16_t x = (uint16_t)v; memcpy(p, &x, 2); break; }
    case XH5C_I32: { int32_t x = (int32_t)v; memcpy(p, &x, 4); break; }
    case XH5C_U32: { uint32_t x = (uint32_t)v; memcpy(p, &x, 4); break; }
    case XH5C_I64: { int64_t x = (int64_t)v; memcpy(p, &x, 8); break; }
    case XH5C_F32: { float x = (float)v; memcpy(p, &x, 4); break; }
    case XH5C_F64: { memcpy(p, &v, 8); break; }
    default: break;
  }
}

hid_t create_dataset(hid_t loc, const char *name, hid_t type, hid_t space) {
  Store *st = store_of(loc);
  auto sp = g_handles.find(space);
  if (!st || sp == g_handles.end()) return -1;
  std::string path = resolve(loc, name);
  Dataset d;
  d.type = (uint32_t)type;
  d.dims = sp->second.dims;
  size_t n = 1;
  for (hsize_t x : d.dims) n *= (size_t)x;
  d.bytes.assign(n * elem_size(d.type), 0);
  st->sets[path] = d;
  st->dirty = true;
  return new_handle(3, path, loc);
}

}  // namespace

hid_t H5Fopen(const char *name, unsigned, hid_t) {
  std::string file = name ? name : "";
  if (!g_files.count(file)) load(file, g_files[file]);
  hid_t h = g_next++;
  Handle hd;
  hd.kind = 1;
  hd.path = "/";
  g_handles[h] = hd;
  g_file_of[h] = file;
  return h;
}

herr_t H5Fclose(hid_t file) {
  auto it = g_file_of.find(file);
  if (it == g_file_of.end()) return -1;
  Store &st = g_files[it->second];
  if (st.dirty) {
    save(it->second, st);
    st.dirty = false;
  }
  return 0;
}

hid_t H5Gopen2(hid_t loc, const char *name, hid_t) { return new_handle(2, resolve(loc, name), loc); }
hid_t H5Gcreate(hid_t loc, const char *name, hid_t, hid_t, hid_t) {
  return new_handle(2, resolve(loc, name), loc);
}
herr_t H5Gclose(hid_t) { return 0; }

hid_t H5Dopen(hid_t loc, const char *name, hid_t) {
  Store *st = store_of(loc);
  if (!st) return -1;
  std::string path = resolve(loc, name);
  if (!st->sets.count(path)) return -1;
  return new_handle(3, path, loc);
}
hid_t H5Dopen2(hid_t loc, const char *name, hid_t dapl) { return H5Dopen(loc, name, dapl); }
hid_t H5Dcreate(hid_t loc, const char *name, hid_t type, hid_t space, hid_t, hid_t, hid_t) {
  return create_dataset(loc, name, type, space);
}
hid_t H5Dcreate2(hid_t loc, const char *name, hid_t type, hid_t space, hid_t, hid_t, hid_t) {
  return create_dataset(loc, name, type, space);
}
herr_t H5Dclose(hid_t) { return 0; }

hid_t H5Dget_space(hid_t dset) {
  Dataset *d = dataset_of(dset);
  if (!d) return -1;
  hid_t h = g_next++;
  Handle hd;
  hd.kind = 4;
  hd.dims = d->dims;
  g_handles[h] = hd;
  return h;
}

hid_t H5Dget_type(hid_t dset) {
  Dataset *d = dataset_of(dset);
  return d ? (hid_t)d->type : -1;
}

hsize_t H5Dget_storage_size(hid_t dset) {
  Dataset *d = dataset_of(dset);
  return d ? (hsize_t)d->bytes.size() : 0;
}

herr_t H5Dread(hid_t dset, hid_t mem_type, hid_t, hid_t, hid_t, void *buf) {
  Dataset *d = dataset_of(dset);
  if (!d || !buf) return -1;
  if ((uint32_t)mem_type == d->type || d->type == XH5C_STR) {
    memcpy(buf, d->bytes.data(), d->bytes.size());
    return 0;
  }
  size_t es = elem_size(d->type), n = d->bytes.size() / es, ms = elem_size((uint32_t)mem_type);
  unsigned char *out = (unsigned char *)buf;
  for (size_t i = 0; i < n; i++)
    store_elem(out + i * ms, (uint32_t)mem_type, load_elem(d->bytes.data() + i * es, d->type));
  return 0;
}

herr_t H5Dwrite(hid_t dset, hid_t mem_type, hid_t, hid_t, hid_t, const void *buf) {
  Dataset *d = dataset_of(dset);
  Store *st = store_of(dset);
  if (!d || !st || !buf) return -1;
  if ((uint32_t)mem_type == d->type) {
    memcpy(d->bytes.data(), buf, d->bytes.size());
  } else {
    size_t es = elem_size(d->type), n = d->bytes.size() / es, ms = elem_size((uint32_t)mem_type);
    const unsigned char *in = (const unsigned char *)buf;
    for (size_t i = 0; i < n; i++)
      store_elem(d->bytes.data() + i * es, d->type, load_elem(in + i * ms, (uint32_t)mem_type));
  }
  st->dirty = true;
  return 0;
}

hid_t H5Screate_simple(int rank, const hsize_t *dims, const hsize_t *) {
  hid_t h = g_next++;
  Handle hd;
  hd.kind = 4;
  hd.dims.assign(dims, dims + rank);
  g_handles[h] = hd;
  return h;
}
herr_t H5Sclose(hid_t) { return 0; }

int H5Sget_simple_extent_dims(hid_t space, hsize_t *dims, hsize_t *maxdims) {
  auto it = g_handles.find(space);
  if (it == g_handles.end()) return -1;
  const std::vector<hsize_t> &v = it->second.dims;
  for (size_t i = 0; i < v.size(); i++) {
    if (dims) dims[i] = v[i];
    if (maxdims) maxdims[i] = v[i];
  }
  return (int)v.size();
}

int H5Sget_simple_extent_ndims(hid_t space) {
  auto it = g_handles.find(space);
  return it == g_handles.end() ? -1 : (int)it->second.dims.size();
}

herr_t H5Sselect_hyperslab(hid_t, int, const hsize_t *, const hsize_t *, const hsize_t *,
                           const hsize_t *) {
  return 0;
}

htri_t H5Tis_variable_str(hid_t) { return 0; }
hid_t H5Tget_native_type(hid_t type, int) { return type; }
htri_t H5Tequal(hid_t a, hid_t b) { return a == b ? 1 : 0; }
size_t H5Tget_size(hid_t type) { return elem_size((uint32_t)type); }

herr_t H5Eset_auto(int, void *, void *) { return 0; }

hid_t H5Pcreate(int) { return g_next++; }
herr_t H5Pset_chunk(hid_t, int, const hsize_t *) { return 0; }
herr_t H5Pset_deflate(hid_t, unsigned) { return 0; }
