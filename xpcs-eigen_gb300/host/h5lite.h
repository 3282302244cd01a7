// A reader and writer, written from the HDF5 File Format Specification
// (version 3.0), for the part of HDF5 that the XPCS analysis file uses
// (configuration.cpp:80-242 reads it, h5_result.cpp:56-347 writes into it).
//
// Reading: superblocks of versions 0-3 (with or without a user block),
// version 1 and 2 object headers with continuation blocks, groups stored as
// symbol tables (v1 B-tree + local heap) or as compact link messages, and
// datasets with compact or contiguous storage whose elements are
// little-endian integers, IEEE floats, fixed-length strings or
// variable-length strings (global heap).  Datasets stored in chunks (and so
// any compressed dataset) and groups whose links are in a fractal heap are
// listed as skipped, with the reason.
//
// Writing: into files with a version 0/1 superblock and symbol-table groups,
// the layout that the HDF5 library writes by default.  A dataset that exists
// with the same element type and shape is overwritten in place; otherwise a
// new dataset (version 1 object header, contiguous storage) is appended, with
// any missing groups, and each group that gains a link gets a new local-heap
// data segment, symbol-table nodes and B-tree appended, after which the
// addresses that point to them (the group's symbol-table message and the
// cached copies in the entries that lead to it) are updated in place.  The
// space the replaced structures held is left unused, as the library itself
// leaves freed space when a file is closed.  The file is rewritten through a
// temporary file and a rename.
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace h5lite {

enum class Kind { Int, UInt, Float, String };

struct Data {
  Kind kind = Kind::Int;
  uint32_t size = 0;                 // bytes per element (strings: bytes per string)
  std::vector<uint64_t> dims;        // empty: a scalar
  std::vector<unsigned char> bytes;  // row-major elements, little endian
  uint64_t count() const;
};

// True when the file holds an HDF5 superblock (at offset 0, 512, 1024, ...).
bool is_hdf5(const std::string &path);

// Every dataset of the file by absolute path ("/xpcs/dqmap").  Datasets and
// groups that this reader does not handle go to `skipped` (path -> reason).
// Throws std::runtime_error on a file it cannot parse.
void read_all(const std::string &path, std::map<std::string, Data> &sets,
              std::map<std::string, std::string> &skipped);

// A new file holding an empty root group (version 0 superblock).
void create(const std::string &path);

// Creates or overwrites the datasets `sets` (absolute paths) in the file.
// Throws std::runtime_error when the file's layout is outside what this
// writer handles, or when a dataset exists with another type or shape.
void write(const std::string &path, const std::map<std::string, Data> &sets);

}  // namespace h5lite
