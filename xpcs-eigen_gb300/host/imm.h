// IMM frame files (the detector stream of xpcs-eigen, src/xpcs/io/imm.h:63-144).
//
// Every frame is a 1024-byte header followed by its data.  Header fields used:
// compression (int32 @4, non-zero = sparse), elapsed (float64 @128, the
// frame's clock), dlen (uint32 @152, values in the frame), corecotick
// (int32 @620, the frame's tick).  Sparse frames carry int32 pixel indices
// then int16 values; dense frames carry int16 values only.  Values are read as
// signed 16-bit, as the reference reads them (imm.cpp:87-99).
//
// Unlike the reference (which trusts dlen and goes on after a short read,
// imm.cpp:70-118), the reader refuses a frame whose dlen exceeds the
// detector's pixel count (sparse) or differs from it (dense), and a file that
// ends inside a frame; next() and skip() then return -1 and error() says why.
#pragma once

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace imm {

struct Block {
  std::vector<uint32_t> nnz;       // values per frame
  std::vector<int32_t> idx;        // sparse: pixel indices, frames back to back
  std::vector<int16_t> val;        // values, frames back to back
  std::vector<double> clock, ticks;
};

class Reader {
 public:
  ~Reader();
  bool open(const std::string &path);
  bool compressed() const { return compressed_; }
  // The detector's pixel count (width * height): the bound on dlen.
  void set_frame_pixels(int64_t pixels) { pixels_ = pixels; }
  // Reads up to `count` frames; returns the number read (fewer only at the
  // end of the file), or -1 for a corrupt or truncated frame.
  int next(int count, Block &out);
  // Skips `count` frames (Imm::SkipFrames, imm.cpp:120-129); same returns.
  int skip(int count);
  // Frames read or skipped so far.
  int64_t position() const { return frame_; }
  const std::string &error() const { return error_; }

 private:
  bool check_dlen(uint32_t n);
  FILE *f_ = nullptr;
  bool compressed_ = false;
  int64_t pixels_ = -1;  // unknown: no bound
  int64_t frame_ = 0;
  std::string error_;
};

}  // namespace imm
