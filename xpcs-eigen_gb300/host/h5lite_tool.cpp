// h5lite command line: inspect and write the HDF5 subset of h5lite.h.
//
//   h5lite_tool dump FILE            every dataset: path, kind, size, dims, values
//   h5lite_tool create FILE          a new file with an empty root group
//   h5lite_tool put FILE PATH KIND DIMS VALUE...
//                                    KIND i8..i64 u8..u64 f32 f64 str; DIMS "scalar"
//                                    or comma-separated; one value per element
//   h5lite_tool from-xh5c IN OUT     a new HDF5 file with every dataset of an
//                                    XH5C container
//
// dump prints one line per dataset: path, then kind and element size, then the
// dims, then the values (%.17g for numbers, strings in quotes); skipped
// datasets are printed as "skip PATH REASON".
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "h5lite.h"
#include "xh5c.h"

namespace {

int usage() {
  fprintf(stderr, "usage: h5lite_tool dump FILE | create FILE | put FILE PATH KIND DIMS VALUE... | "
                  "from-xh5c IN OUT\n");
  return 2;
}

double num(const h5lite::Data &d, uint64_t i) {
  const unsigned char *p = d.bytes.data() + i * d.size;
  if (d.kind == h5lite::Kind::Float) {
    if (d.size == 4) {
      float f;
      memcpy(&f, p, 4);
      return f;
    }
    double x;
    memcpy(&x, p, 8);
    return x;
  }
  uint64_t u = 0;
  for (int k = (int)d.size - 1; k >= 0; k--) u = (u << 8) | p[k];
  if (d.kind == h5lite::Kind::Int && d.size < 8 && (u >> (8 * d.size - 1)))
    u |= ~0ull << (8 * d.size);  // sign extension
  return d.kind == h5lite::Kind::Int ? (double)(int64_t)u : (double)u;
}

const char *kind_name(h5lite::Kind k) {
  switch (k) {
    case h5lite::Kind::Int: return "int";
    case h5lite::Kind::UInt: return "uint";
    case h5lite::Kind::Float: return "float";
    default: return "str";
  }
}

int dump(const std::string &path) {
  std::map<std::string, h5lite::Data> sets;
  std::map<std::string, std::string> skipped;
  h5lite::read_all(path, sets, skipped);
  for (const auto &kv : sets) {
    const h5lite::Data &d = kv.second;
    printf("%s %s%u ", kv.first.c_str(), kind_name(d.kind), d.size);
    if (d.dims.empty()) printf("scalar");
    for (size_t i = 0; i < d.dims.size(); i++) printf("%s%" PRIu64, i ? "," : "", d.dims[i]);
    for (uint64_t i = 0; i < d.count(); i++) {
      if (d.kind == h5lite::Kind::String) {
        const char *s = (const char *)d.bytes.data() + i * d.size;
        printf(" \"%.*s\"", (int)strnlen(s, d.size), s);
      } else {
        printf(" %.17g", num(d, i));
      }
    }
    printf("\n");
  }
  for (const auto &kv : skipped) printf("skip %s %s\n", kv.first.c_str(), kv.second.c_str());
  return 0;
}

bool parse_kind(const std::string &k, h5lite::Data &d) {
  if (k == "str") {
    d.kind = h5lite::Kind::String;
    return true;
  }
  if (k == "f32" || k == "f64") {
    d.kind = h5lite::Kind::Float;
    d.size = k == "f32" ? 4 : 8;
    return true;
  }
  if (k.size() >= 2 && (k[0] == 'i' || k[0] == 'u')) {
    d.kind = k[0] == 'i' ? h5lite::Kind::Int : h5lite::Kind::UInt;
    const int bits = atoi(k.c_str() + 1);
    if (bits != 8 && bits != 16 && bits != 32 && bits != 64) return false;
    d.size = (uint32_t)(bits / 8);
    return true;
  }
  return false;
}

int put(int argc, char **argv) {
  h5lite::Data d;
  if (argc < 7 || !parse_kind(argv[4], d)) return usage();
  const std::string dims = argv[5];
  if (dims != "scalar")
    for (const char *p = dims.c_str(); *p;) {
      char *e;
      d.dims.push_back(strtoull(p, &e, 10));
      p = *e == ',' ? e + 1 : e;
      if (e == p && *p) return usage();
    }
  const int nval = argc - 6;
  if ((uint64_t)nval != d.count()) {
    fprintf(stderr, "h5lite_tool: %d values for %" PRIu64 " elements\n", nval, d.count());
    return 2;
  }
  if (d.kind == h5lite::Kind::String) {
    size_t w = 1;
    for (int i = 0; i < nval; i++) w = std::max(w, strlen(argv[6 + i]));
    d.size = (uint32_t)w;
    d.bytes.assign((size_t)nval * w, 0);
    for (int i = 0; i < nval; i++) memcpy(&d.bytes[i * w], argv[6 + i], strlen(argv[6 + i]));
  } else {
    d.bytes.resize((size_t)nval * d.size);
    for (int i = 0; i < nval; i++) {
      unsigned char *p = &d.bytes[(size_t)i * d.size];
      if (d.kind == h5lite::Kind::Float) {
        const double x = strtod(argv[6 + i], nullptr);
        if (d.size == 4) {
          const float f = (float)x;
          memcpy(p, &f, 4);
        } else {
          memcpy(p, &x, 8);
        }
      } else {
        const uint64_t u = d.kind == h5lite::Kind::Int ? (uint64_t)strtoll(argv[6 + i], nullptr, 10)
                                                       : strtoull(argv[6 + i], nullptr, 10);
        for (uint32_t k = 0; k < d.size; k++) p[k] = (unsigned char)(u >> (8 * k));
      }
    }
  }
  h5lite::write(argv[2], {{argv[3], d}});
  return 0;
}

int from_xh5c(const std::string &in, const std::string &out) {
  xh5c::File f;
  if (!f.load(in)) {
    fprintf(stderr, "h5lite_tool: cannot read %s\n", in.c_str());
    return 1;
  }
  f.save_hdf5(out);
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc < 3) return usage();
  const std::string cmd = argv[1];
  try {
    if (cmd == "dump") return dump(argv[2]);
    if (cmd == "create") {
      h5lite::create(argv[2]);
      return 0;
    }
    if (cmd == "put") return put(argc, argv);
    if (cmd == "from-xh5c" && argc == 4) return from_xh5c(argv[2], argv[3]);
  } catch (const std::exception &e) {
    fprintf(stderr, "h5lite_tool: %s\n", e.what());
    return 1;
  }
  return usage();
}
