#include "imm.h"

#include <cstring>

namespace imm {

namespace {
constexpr size_t HDR = 1024;
constexpr size_t OFF_COMPRESSION = 4, OFF_ELAPSED = 128, OFF_DLEN = 152, OFF_CORECOTICK = 620;

template <class T>
T field(const unsigned char *h, size_t off) {
  T v;
  memcpy(&v, h + off, sizeof(T));
  return v;
}
}  // namespace

Reader::~Reader() {
  if (f_) fclose(f_);
}

bool Reader::open(const std::string &path) {
  f_ = fopen(path.c_str(), "rb");
  if (!f_) return false;
  unsigned char h[HDR];
  if (fread(h, 1, HDR, f_) != HDR) return false;
  compressed_ = field<int32_t>(h, OFF_COMPRESSION) != 0;
  rewind(f_);
  return true;
}

int Reader::next(int count, Block &out) {
  out.nnz.clear();
  out.idx.clear();
  out.val.clear();
  out.clock.clear();
  out.ticks.clear();
  unsigned char h[HDR];
  int done = 0;
  for (; done < count; done++) {
    if (fread(h, 1, HDR, f_) != HDR) break;
    const uint32_t n = field<uint32_t>(h, OFF_DLEN);
    const size_t i0 = out.val.size();
    if (compressed_) {
      out.idx.resize(i0 + n);
      if (n && fread(out.idx.data() + i0, 4, n, f_) != n) break;
    }
    out.val.resize(i0 + n);
    if (n && fread(out.val.data() + i0, 2, n, f_) != n) break;
    out.nnz.push_back(n);
    out.clock.push_back(field<double>(h, OFF_ELAPSED));
    out.ticks.push_back((double)field<int32_t>(h, OFF_CORECOTICK));
  }
  if ((int)out.nnz.size() < done) done = (int)out.nnz.size();
  return done;
}

int Reader::skip(int count) {
  unsigned char h[HDR];
  int done = 0;
  for (; done < count; done++) {
    if (fread(h, 1, HDR, f_) != HDR) break;
    const long bytes = (long)field<uint32_t>(h, OFF_DLEN) * (compressed_ ? 6 : 2);
    if (fseek(f_, bytes, SEEK_CUR) != 0) break;
  }
  return done;
}

}  // namespace imm
