// IMM frame files (the detector stream of xpcs-eigen, src/xpcs/io/imm.h:63-144).
//
// Every frame is a 1024-byte header followed by its data.  Header fields used:
// compression (int32 @4, non-zero = sparse), elapsed (float64 @128, the
// frame's clock), dlen (uint32 @152, values in the frame), corecotick
// (int32 @620, the frame's tick).  Sparse frames carry int32 pixel indices
// then int16 values; dense frames carry int16 values only.  Values are read as
// signed 16-bit, as the reference reads them (imm.cpp:87-99).
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
  // Reads up to `count` frames; returns the number read (0 at end of file).
  int next(int count, Block &out);
  // Skips `count` frames (Imm::SkipFrames, imm.cpp:120-129).
  int skip(int count);

 private:
  FILE *f_ = nullptr;
  bool compressed_ = false;
};

}  // namespace imm
