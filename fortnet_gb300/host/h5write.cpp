// Minimal HDF5 writer (see h5write.hpp).  Layout of one file, in write order: the superblock
// (version 0, 8-byte offsets and lengths, group K values 4 / 16), then every object depth
// first, children before their parent: a dataset's raw data and then its object header; a
// group's local heap (member names), its symbol-table nodes (up to 8 members each), its
// version-1 B-tree nodes (up to 32 children each) and then its object header holding the
// symbol-table message and the group's attributes.  The root group's header address and the
// end-of-file address are patched into the superblock last.
#include "h5write.hpp"

#include <cstring>
#include <fstream>
#include <stdexcept>

namespace h5w {

namespace {

constexpr uint64_t kUndef = ~uint64_t(0);
constexpr int kLeafK = 4;       // symbol-table node holds 2K = 8 entries
constexpr int kInternalK = 16;  // B-tree node holds 2K = 32 children
constexpr uint64_t kHeapFreeNull = 1;  // end of a local heap's free list

struct Bytes {
  std::vector<uint8_t> b;
  size_t size() const { return b.size(); }
  void u8(uint8_t v) { b.push_back(v); }
  void u16(uint16_t v) { put(&v, 2); }
  void u32(uint32_t v) { put(&v, 4); }
  void u64(uint64_t v) { put(&v, 8); }
  void put(const void *p, size_t n) {
    const uint8_t *c = static_cast<const uint8_t *>(p);
    b.insert(b.end(), c, c + n);  // the host is little-endian, as the format's fields are
  }
  void zeros(size_t n) { b.insert(b.end(), n, 0); }
  void pad8() { zeros((8 - b.size() % 8) % 8); }
  void set_u64(size_t pos, uint64_t v) { std::memcpy(&b[pos], &v, 8); }
};

static_assert(sizeof(double) == 8, "IEEE double expected");

size_t elem_size(const Value &v) { return v.kind == Value::STR ? v.s.size() + 1 : v.kind == Value::I32 ? 4 : 8; }

uint64_t count(const Value &v) {
  uint64_t n = 1;
  for (uint64_t d : v.dims) n *= d;
  return n;
}

// Datatype message body (version 1): 32-bit signed little-endian integer, IEEE double, or a
// null-terminated ASCII string of the value's length + 1.
Bytes datatype(const Value &v) {
  Bytes m;
  if (v.kind == Value::I32) {
    m.u8(0x10);  // class 0 (fixed point), version 1
    m.u8(0x08);  // little-endian, signed
    m.u8(0);
    m.u8(0);
    m.u32(4);
    m.u16(0);   // bit offset
    m.u16(32);  // precision
  } else if (v.kind == Value::F64) {
    m.u8(0x11);  // class 1 (floating point), version 1
    m.u8(0x20);  // little-endian, implied leading mantissa bit
    m.u8(63);    // sign bit position
    m.u8(0);
    m.u32(8);
    m.u16(0);
    m.u16(64);
    m.u8(52);  // exponent location
    m.u8(11);  // exponent size
    m.u8(0);   // mantissa location
    m.u8(52);  // mantissa size
    m.u32(1023);
  } else {
    m.u8(0x13);  // class 3 (string), version 1
    m.u8(0x00);  // null-terminated, ASCII
    m.u8(0);
    m.u8(0);
    m.u32((uint32_t)(v.s.size() + 1));
  }
  return m;
}

// Dataspace message body (version 1): scalar for strings, else the dimensions with equal
// maximum dimensions.
Bytes dataspace(const Value &v) {
  Bytes m;
  const bool scalar = v.kind == Value::STR;
  m.u8(1);
  m.u8(scalar ? 0 : (uint8_t)v.dims.size());
  m.u8(scalar ? 0 : 1);  // maximum dimensions present
  m.zeros(5);
  if (!scalar) {
    for (uint64_t d : v.dims) m.u64(d);
    for (uint64_t d : v.dims) m.u64(d);
  }
  return m;
}

void raw(Bytes &out, const Value &v) {
  if (v.kind == Value::I32) out.put(v.i.data(), 4 * v.i.size());
  else if (v.kind == Value::F64) out.put(v.d.data(), 8 * v.d.size());
  else out.put(v.s.c_str(), v.s.size() + 1);
}

struct Message {
  uint16_t type;
  uint8_t flags;
  Bytes body;
};

// Version-1 object header: 16-byte prefix, then every message with its 8-byte header and a
// body padded to 8 bytes.
uint64_t write_header(Bytes &f, const std::vector<Message> &msgs) {
  f.pad8();
  const uint64_t addr = f.size();
  uint32_t size = 0;
  for (const auto &m : msgs) size += 8 + (uint32_t)((m.body.size() + 7) / 8 * 8);
  f.u8(1);
  f.u8(0);
  f.u16((uint16_t)msgs.size());
  f.u32(1);  // reference count
  f.u32(size);
  f.zeros(4);
  for (const auto &m : msgs) {
    const size_t padded = (m.body.size() + 7) / 8 * 8;
    f.u16(m.type);
    f.u16((uint16_t)padded);
    f.u8(m.flags);
    f.zeros(3);
    f.put(m.body.b.data(), m.body.size());
    f.zeros(padded - m.body.size());
  }
  return addr;
}

Message attribute(const std::string &name, const Value &v) {
  Message m{0x000C, 0, {}};
  const Bytes dt = datatype(v), ds = dataspace(v);
  Bytes &a = m.body;
  a.u8(1);
  a.u8(0);
  a.u16((uint16_t)(name.size() + 1));
  a.u16((uint16_t)dt.size());
  a.u16((uint16_t)ds.size());
  a.put(name.c_str(), name.size() + 1);
  a.pad8();
  a.put(dt.b.data(), dt.size());
  a.pad8();
  a.put(ds.b.data(), ds.size());
  a.pad8();
  raw(a, v);
  return m;
}

struct Entry {
  uint64_t name_off;
  uint64_t header;
  bool group;
  uint64_t btree, heap;  // cached for groups
};

struct Written {
  uint64_t header, btree, heap;
};

Written write_object(Bytes &f, const Object &o);

Written write_group(Bytes &f, const Object &g) {
  std::vector<Entry> entries;
  std::vector<std::string> names;
  for (const auto &kv : g.children) {
    const Written w = write_object(f, *kv.second);
    entries.push_back(Entry{0, w.header, kv.second->group, w.btree, w.heap});
    names.push_back(kv.first);
  }
  // local heap: "" at offset 0, the names (each null-terminated, padded to 8), a free block
  Bytes data;
  data.zeros(8);
  for (size_t k = 0; k < names.size(); k++) {
    entries[k].name_off = data.size();
    data.put(names[k].c_str(), names[k].size() + 1);
    data.pad8();
  }
  const uint64_t free_off = data.size();
  data.u64(kHeapFreeNull);
  data.u64(16);
  f.pad8();
  const uint64_t heap = f.size();
  f.put("HEAP", 4);
  f.u8(0);
  f.zeros(3);
  f.u64(data.size());
  f.u64(free_off);
  f.u64(heap + 32);
  f.put(data.b.data(), data.size());
  // symbol-table nodes of up to 2 * kLeafK entries, each node sized for its full capacity
  struct Child {
    uint64_t addr;
    uint64_t last_name;  // heap offset of the node's largest name
  };
  std::vector<Child> level;
  for (size_t k0 = 0; k0 < entries.size() || (k0 == 0 && entries.empty()); k0 += 2 * kLeafK) {
    const size_t k1 = std::min(entries.size(), k0 + 2 * kLeafK);
    f.pad8();
    const uint64_t addr = f.size();
    f.put("SNOD", 4);
    f.u8(1);
    f.u8(0);
    f.u16((uint16_t)(k1 - k0));
    for (size_t k = k0; k < k1; k++) {
      const Entry &e = entries[k];
      f.u64(e.name_off);
      f.u64(e.header);
      f.u32(e.group ? 1 : 0);
      f.u32(0);
      if (e.group) {
        f.u64(e.btree);
        f.u64(e.heap);
      } else {
        f.zeros(16);
      }
    }
    f.zeros(40 * (2 * kLeafK - (k1 - k0)));
    level.push_back(Child{addr, k1 > k0 ? entries[k1 - 1].name_off : 0});
    if (entries.empty()) break;
  }
  // version-1 B-tree over the nodes: keys are heap offsets, key 0 the empty name and key
  // i + 1 the largest name under child i
  int height = 0;
  for (;;) {
    std::vector<Child> up;
    for (size_t c0 = 0; c0 < level.size(); c0 += 2 * kInternalK) {
      const size_t c1 = std::min(level.size(), c0 + 2 * kInternalK);
      f.pad8();
      const uint64_t addr = f.size();
      f.put("TREE", 4);
      f.u8(0);  // group node
      f.u8((uint8_t)height);
      f.u16((uint16_t)(entries.empty() ? 0 : c1 - c0));
      f.u64(kUndef);
      f.u64(kUndef);
      f.u64(0);
      for (size_t c = c0; c < c1; c++) {
        f.u64(level[c].addr);
        f.u64(level[c].last_name);
      }
      f.zeros(16 * (2 * kInternalK - (c1 - c0)));
      up.push_back(Child{addr, level[c1 - 1].last_name});
    }
    level.swap(up);
    height++;
    if (level.size() == 1) break;
  }
  const uint64_t btree = level[0].addr;
  std::vector<Message> msgs;
  Message st{0x0011, 0, {}};
  st.body.u64(btree);
  st.body.u64(heap);
  msgs.push_back(st);
  for (const auto &a : g.attrs) msgs.push_back(attribute(a.first, a.second));
  return Written{write_header(f, msgs), btree, heap};
}

Written write_dataset(Bytes &f, const Object &o) {
  const Value &v = o.data;
  f.pad8();
  const uint64_t data_addr = f.size();
  raw(f, v);
  const uint64_t bytes = count(v) * elem_size(v);
  std::vector<Message> msgs;
  msgs.push_back(Message{0x0001, 0, dataspace(v)});
  msgs.push_back(Message{0x0003, 1, datatype(v)});
  Message fill{0x0005, 1, {}};  // version 2: late allocation, write if set, default value
  fill.body.u8(2);
  fill.body.u8(2);
  fill.body.u8(2);
  fill.body.u8(1);
  fill.body.u32(0);
  msgs.push_back(fill);
  Message layout{0x0008, 0, {}};  // version 3, contiguous
  layout.body.u8(3);
  layout.body.u8(1);
  layout.body.u64(data_addr);
  layout.body.u64(bytes);
  msgs.push_back(layout);
  for (const auto &a : o.attrs) msgs.push_back(attribute(a.first, a.second));
  return Written{write_header(f, msgs), 0, 0};
}

Written write_object(Bytes &f, const Object &o) { return o.group ? write_group(f, o) : write_dataset(f, o); }

std::vector<std::string> split(const std::string &path) {
  std::vector<std::string> parts;
  size_t p = 0;
  while (p <= path.size()) {
    const size_t q = path.find('/', p);
    const std::string s = path.substr(p, q == std::string::npos ? std::string::npos : q - p);
    if (!s.empty()) parts.push_back(s);
    if (q == std::string::npos) break;
    p = q + 1;
  }
  return parts;
}

}  // namespace

Object &File::leaf(const std::string &path, bool make_group) {
  Object *o = &root_;
  const auto parts = split(path);
  for (size_t k = 0; k < parts.size(); k++) {
    if (!o->group) throw std::runtime_error("h5w: '" + path + "' passes through a dataset");
    auto &slot = o->children[parts[k]];
    if (!slot) {
      slot.reset(new Object());
      slot->group = make_group || k + 1 < parts.size();
    }
    o = slot.get();
  }
  return *o;
}

Object &File::group(const std::string &path) {
  Object &o = leaf(path, true);
  if (!o.group) throw std::runtime_error("h5w: '" + path + "' is a dataset");
  return o;
}

void File::dataset_f64(const std::string &path, std::vector<uint64_t> dims, std::vector<double> data) {
  Object &o = leaf(path, false);
  o.group = false;
  o.data.kind = Value::F64;
  o.data.dims = std::move(dims);
  o.data.d = std::move(data);
  if (count(o.data) != o.data.d.size()) throw std::runtime_error("h5w: size of '" + path + "'");
}

void File::dataset_i32(const std::string &path, std::vector<uint64_t> dims, std::vector<int32_t> data) {
  Object &o = leaf(path, false);
  o.group = false;
  o.data.kind = Value::I32;
  o.data.dims = std::move(dims);
  o.data.i = std::move(data);
  if (count(o.data) != o.data.i.size()) throw std::runtime_error("h5w: size of '" + path + "'");
}

void File::attr_i32(const std::string &path, const std::string &name, std::vector<int32_t> v) {
  Value x;
  x.kind = Value::I32;
  x.dims = {v.size()};
  x.i = std::move(v);
  leaf(path, true).attrs.emplace_back(name, std::move(x));
}

void File::attr_f64(const std::string &path, const std::string &name, std::vector<double> v) {
  Value x;
  x.kind = Value::F64;
  x.dims = {v.size()};
  x.d = std::move(v);
  leaf(path, true).attrs.emplace_back(name, std::move(x));
}

void File::attr_str(const std::string &path, const std::string &name, const std::string &v) {
  Value x;
  x.kind = Value::STR;
  x.s = v;
  leaf(path, true).attrs.emplace_back(name, std::move(x));
}

void File::write(const std::string &filename) const {
  Bytes f;
  const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
  f.put(sig, 8);
  f.u8(0);  // superblock version
  f.u8(0);  // free-space version
  f.u8(0);  // root symbol-table entry version
  f.u8(0);
  f.u8(0);  // shared-header-message version
  f.u8(8);  // size of offsets
  f.u8(8);  // size of lengths
  f.u8(0);
  f.u16(kLeafK);
  f.u16(kInternalK);
  f.u32(0);       // consistency flags
  f.u64(0);       // base address
  f.u64(kUndef);  // free-space info
  const size_t eof_pos = f.size();
  f.u64(0);       // end of file, patched
  f.u64(kUndef);  // driver information
  const size_t root_pos = f.size();
  f.zeros(40);    // root symbol-table entry, patched
  const Written root = write_group(f, root_);
  f.pad8();
  f.set_u64(eof_pos, f.size());
  f.set_u64(root_pos, 0);  // link name offset
  f.set_u64(root_pos + 8, root.header);
  const uint32_t cache = 1;
  std::memcpy(&f.b[root_pos + 16], &cache, 4);
  f.set_u64(root_pos + 24, root.btree);
  f.set_u64(root_pos + 32, root.heap);
  std::ofstream out(filename, std::ios::binary | std::ios::trunc);
  if (!out) throw std::runtime_error("h5w: cannot create " + filename);
  out.write(reinterpret_cast<const char *>(f.b.data()), (std::streamsize)f.size());
  if (!out) throw std::runtime_error("h5w: write failed for " + filename);
}

}  // namespace h5w
