// Read-only HDF5 reader for the files Fortnet writes (datasets, netstats, fnetout).
//
// Fortnet stores everything through the HDF5 Fortran high-level API, which produces files
// with superblock version 0, version-1 object headers and symbol-table groups (v1 B-tree +
// local heap).  This reader implements that subset of the published HDF5 file-format
// specification: superblock v0/v1, object header v1, symbol table message, SNOD/TREE/HEAP,
// dataspace v1/v2, fixed-point / IEEE float / fixed-length and variable-length string
// datatypes, contiguous / compact / unfiltered chunked layouts, attribute messages v1-v3.
// Fortran column-major arrays keep the file's dimension order reversed (coords(3, nAtom) has
// shape {nAtom, 3}), as h5py reports them.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace fnet {
namespace h5 {

struct Error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// A dataset or attribute value: numbers are widened to double (floats) or int64 (integers).
struct Value {
  enum Kind { kNone, kInt, kFloat, kString } kind = kNone;
  std::vector<uint64_t> shape;      // empty: scalar
  std::vector<int64_t> ints;
  std::vector<double> floats;
  std::vector<std::string> strings;

  size_t size() const;
  double as_double(size_t i = 0) const;  // any numeric kind
  int64_t as_int(size_t i = 0) const;
  std::vector<double> doubles() const;    // any numeric kind, flattened
  std::vector<int64_t> integers() const;
  std::string str(size_t i = 0) const;    // strings (whitespace-trimmed)
};

struct Node {
  std::string name;
  bool is_group = false;
  std::map<std::string, Value> attrs;
  std::map<std::string, std::unique_ptr<Node>> children;
  Value value;

  const Node &operator[](const std::string &path) const;  // "a/b/c"
  bool has(const std::string &path) const;
  const Value &attr(const std::string &name) const;
  bool has_attr(const std::string &name) const { return attrs.count(name) != 0; }
};

// Parse a whole file; throws h5::Error for malformed or unsupported content.
std::unique_ptr<Node> read(const std::string &path);
std::unique_ptr<Node> read_bytes(std::vector<uint8_t> data);

}  // namespace h5
}  // namespace fnet
