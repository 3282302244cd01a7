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

bool Reader::check_dlen(uint32_t n) {
  if (pixels_ < 0) return true;
  if (compressed_ && (int64_t)n > pixels_) {
    error_ = "corrupt IMM frame " + std::to_string(frame_) + ": dlen " + std::to_string(n) +
             " exceeds the detector's " + std::to_string(pixels_) + " pixels";
    return false;
  }
  if (!compressed_ && (int64_t)n != pixels_) {
    error_ = "corrupt IMM frame " + std::to_string(frame_) + ": dense dlen " + std::to_string(n) +
             " differs from the detector's " + std::to_string(pixels_) + " pixels";
    return false;
  }
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
    const size_t got = fread(h, 1, HDR, f_);
    if (got == 0 && feof(f_)) break;  // clean end of file
    if (got != HDR) {
      error_ = "IMM file truncated in the header of frame " + std::to_string(frame_);
      return -1;
    }
    const uint32_t n = field<uint32_t>(h, OFF_DLEN);
    if (!check_dlen(n)) return -1;
    const size_t i0 = out.val.size();
    if (compressed_) {
      out.idx.resize(i0 + n);
      if (n && fread(out.idx.data() + i0, 4, n, f_) != n) {
        error_ = "IMM file truncated in the pixel indices of frame " + std::to_string(frame_);
        return -1;
      }
    }
    out.val.resize(i0 + n);
    if (n && fread(out.val.data() + i0, 2, n, f_) != n) {
      error_ = "IMM file truncated in the values of frame " + std::to_string(frame_);
      return -1;
    }
    out.nnz.push_back(n);
    out.clock.push_back(field<double>(h, OFF_ELAPSED));
    out.ticks.push_back((double)field<int32_t>(h, OFF_CORECOTICK));
    frame_++;
  }
  return done;
}

int Reader::skip(int count) {
  unsigned char h[HDR];
  int done = 0;
  for (; done < count; done++) {
    const size_t got = fread(h, 1, HDR, f_);
    if (got == 0 && feof(f_)) break;
    if (got != HDR) {
      error_ = "IMM file truncated in the header of frame " + std::to_string(frame_);
      return -1;
    }
    const uint32_t n = field<uint32_t>(h, OFF_DLEN);
    if (!check_dlen(n)) return -1;
    const long bytes = (long)n * (compressed_ ? 6 : 2);
    const long here = ftell(f_);
    if (fseek(f_, 0, SEEK_END) != 0) return -1;
    const long end = ftell(f_);
    if (here < 0 || end < 0 || end - here < bytes) {
      error_ = "IMM file truncated in frame " + std::to_string(frame_);
      return -1;
    }
    if (fseek(f_, here + bytes, SEEK_SET) != 0) return -1;
    frame_++;
  }
  return done;
}

}  // namespace imm
