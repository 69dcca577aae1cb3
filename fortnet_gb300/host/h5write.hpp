// Minimal HDF5 writer for the files the fnet program writes (netstat, fnetout): groups,
// contiguous datasets and attributes of 32-bit integers, IEEE doubles and fixed-length ASCII
// strings.  The file uses the format's original structures (superblock version 0, version-1
// object headers, symbol-table groups with a version-1 B-tree and a local heap), which every
// HDF5 library version reads and which are what the reference's HDF5 library writes for these
// files by default.  No external library.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace h5w {

struct Value {
  enum Kind { I32, F64, STR } kind = I32;
  std::vector<uint64_t> dims;   // C order (slowest first), as the file lists them
  std::vector<int32_t> i;
  std::vector<double> d;
  std::string s;
};

struct Object {
  bool group = true;
  std::map<std::string, std::unique_ptr<Object>> children;  // sorted by name (strcmp order)
  std::vector<std::pair<std::string, Value>> attrs;          // in creation order
  Value data;                                                // datasets only
};

class File {
 public:
  // Groups on the path are created as needed ("a/b/c").
  Object &group(const std::string &path);
  // Fortran-shaped data written the way h5ltmake_dataset_f writes it: the file lists the
  // dimensions reversed (dims_c = Fortran dims reversed) and the data in Fortran order.
  void dataset_f64(const std::string &path, std::vector<uint64_t> dims_c, std::vector<double> data);
  void dataset_i32(const std::string &path, std::vector<uint64_t> dims_c, std::vector<int32_t> data);
  void attr_i32(const std::string &path, const std::string &name, std::vector<int32_t> v);
  void attr_f64(const std::string &path, const std::string &name, std::vector<double> v);
  void attr_str(const std::string &path, const std::string &name, const std::string &v);
  void write(const std::string &filename) const;

 private:
  Object root_;
  Object &leaf(const std::string &path, bool make_group);
};

}  // namespace h5w
