// Read-only HDF5 subset reader (see hdf5lite.hpp for the supported structures).
#include "hdf5lite.hpp"

#include <algorithm>
#include <cstring>
#include <fstream>
#include <functional>
#include <iterator>

namespace fnet {
namespace h5 {

namespace {

constexpr uint64_t kUndef = ~uint64_t(0);

struct Datatype {
  int cls = -1;  // 0 fixed point, 1 float, 3 string, 9 variable length
  uint32_t size = 0;
  bool is_signed = false;
  bool big_endian = false;
};

class Reader {
 public:
  explicit Reader(std::vector<uint8_t> data) : b_(std::move(data)) {
    static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    if (b_.size() < 64 || std::memcmp(b_.data(), sig, 8) != 0)
      throw Error("not an HDF5 file (bad signature)");
    const int version = b_[8];
    if (version != 0 && version != 1) throw Error("unsupported superblock version");
    if (b_[13] != 8 || b_[14] != 8) throw Error("only 8-byte offsets and lengths are supported");
    size_t pos = 16 + 4 + 4;
    if (version == 1) pos += 4;
    pos += 4 * 8;  // base address, free space, end of file, driver information
    root_header_ = u(pos + 8, 8);
  }

  std::unique_ptr<Node> load_root() { return load("/", root_header_, 0); }

 private:
  std::vector<uint8_t> b_;
  uint64_t root_header_ = 0;

  void need(uint64_t pos, uint64_t n) const {
    if (pos > b_.size() || n > b_.size() - pos) throw Error("truncated HDF5 structure");
  }
  uint64_t u(uint64_t pos, int n) const {
    need(pos, n);
    uint64_t v = 0;
    for (int k = n - 1; k >= 0; k--) v = (v << 8) | b_[pos + k];
    return v;
  }
  bool sig(uint64_t pos, const char *s) const {
    need(pos, 4);
    return std::memcmp(b_.data() + pos, s, 4) == 0;
  }
  std::string cstr(uint64_t pos) const {
    std::string out;
    while (pos < b_.size() && b_[pos] != 0) out.push_back((char)b_[pos++]);
    return out;
  }

  // symbol-table group: v1 B-tree of SNOD nodes with names in the local heap
  std::vector<std::pair<std::string, uint64_t>> group_entries(uint64_t btree, uint64_t heap) {
    if (!sig(heap, "HEAP")) throw Error("bad local heap signature");
    const uint64_t seg = u(heap + 24, 8);
    std::vector<std::pair<std::string, uint64_t>> out;
    std::vector<uint64_t> stack{btree};
    while (!stack.empty()) {
      const uint64_t addr = stack.back();
      stack.pop_back();
      if (!sig(addr, "TREE")) throw Error("bad v1 B-tree signature");
      if (b_[addr + 4] != 0) throw Error("group B-tree expected");
      const int level = b_[addr + 5];
      const int used = (int)u(addr + 6, 2);
      uint64_t pos = addr + 8 + 16;
      std::vector<uint64_t> kids;
      for (int k = 0; k < used; k++) {
        pos += 8;  // key
        kids.push_back(u(pos, 8));
        pos += 8;
      }
      if (level > 0) {
        for (auto it = kids.rbegin(); it != kids.rend(); ++it) stack.push_back(*it);
        continue;
      }
      for (uint64_t snod : kids) {
        if (!sig(snod, "SNOD")) throw Error("bad symbol node signature");
        const int nsym = (int)u(snod + 6, 2);
        uint64_t p = snod + 8;
        for (int k = 0; k < nsym; k++) {
          out.emplace_back(cstr(seg + u(p, 8)), u(p + 8, 8));
          p += 40;
        }
      }
    }
    return out;
  }

  struct Msg {
    int type;
    uint64_t body;
  };
  std::vector<Msg> messages(uint64_t addr) {
    need(addr, 16);
    if (b_[addr] != 1) throw Error("unsupported object header version");
    const int nmsg = (int)u(addr + 2, 2);
    std::vector<std::pair<uint64_t, uint64_t>> blocks{{addr + 16, u(addr + 8, 4)}};
    std::vector<Msg> out;
    for (size_t bi = 0; bi < blocks.size() && (int)out.size() < nmsg; bi++) {
      const uint64_t start = blocks[bi].first, len = blocks[bi].second;
      uint64_t pos = start;
      while (pos + 8 <= start + len && (int)out.size() < nmsg) {
        const int mtype = (int)u(pos, 2);
        const uint64_t msize = u(pos + 2, 2);
        const uint64_t body = pos + 8;
        if (mtype == 0x10) blocks.emplace_back(u(body, 8), u(body + 8, 8));
        out.push_back({mtype, body});
        pos = body + msize;
      }
    }
    return out;
  }

  bool dataspace(uint64_t pos, std::vector<uint64_t> &shape) {
    const int version = b_[pos], ndim = b_[pos + 1];
    uint64_t p;
    if (version == 1) {
      p = pos + 8;
    } else if (version == 2) {
      p = pos + 4;
      if (b_[pos + 3] == 2) return false;  // null dataspace
    } else {
      throw Error("unsupported dataspace version");
    }
    shape.clear();
    for (int k = 0; k < ndim; k++) shape.push_back(u(p + 8 * k, 8));
    return true;
  }

  Datatype datatype(uint64_t pos) {
    Datatype t;
    t.cls = b_[pos] & 0x0f;
    const int bits0 = b_[pos + 1];
    t.size = (uint32_t)u(pos + 4, 4);
    t.big_endian = (t.cls == 0 || t.cls == 1) && (bits0 & 1);
    t.is_signed = t.cls == 0 && (bits0 & 0x08);
    if (t.cls != 0 && t.cls != 1 && t.cls != 3 && t.cls != 9)
      throw Error("unsupported datatype class");
    return t;
  }

  std::string global_heap_object(uint64_t coll, uint32_t index) {
    if (!sig(coll, "GCOL")) throw Error("bad global heap signature");
    const uint64_t csize = u(coll + 8, 8);
    uint64_t pos = coll + 16;
    while (pos < coll + csize) {
      const uint32_t oidx = (uint32_t)u(pos, 2);
      const uint64_t osize = u(pos + 8, 8);
      if (oidx == index) {
        need(pos + 16, osize);
        return std::string(b_.begin() + pos + 16, b_.begin() + pos + 16 + osize);
      }
      if (oidx == 0) break;
      pos += 16 + (osize + 7) / 8 * 8;
    }
    throw Error("global heap object not found");
  }

  std::vector<std::string> vlen_strings(const uint8_t *raw, size_t count) {
    std::vector<std::string> out;
    for (size_t k = 0; k < count; k++) {
      const uint8_t *r = raw + 16 * k;
      uint32_t len = 0;
      uint64_t coll = 0;
      uint32_t index = 0;
      for (int q = 3; q >= 0; q--) len = (len << 8) | r[q];
      for (int q = 11; q >= 4; q--) coll = (coll << 8) | r[q];
      for (int q = 15; q >= 12; q--) index = (index << 8) | r[q];
      out.push_back(global_heap_object(coll, index).substr(0, len));
    }
    return out;
  }

  static size_t count_of(const std::vector<uint64_t> &shape) {
    size_t c = 1;
    for (auto d : shape) c *= (size_t)d;
    return c;
  }

  // raw bytes of a dataset (zero-filled when never written)
  std::vector<uint8_t> read_raw(uint64_t lp, uint32_t esize, const std::vector<uint64_t> &shape) {
    const size_t count = count_of(shape), nbytes = count * esize;
    std::vector<uint8_t> raw(nbytes, 0);
    const int version = b_[lp];
    auto copy_from = [&](uint64_t addr, size_t n) {
      if (addr == kUndef) return;
      n = std::min(n, nbytes);
      need(addr, n);
      std::memcpy(raw.data(), b_.data() + addr, n);
    };
    if (version == 1 || version == 2) {
      const int ndim = b_[lp + 1], lclass = b_[lp + 2];
      uint64_t p = lp + 8;
      if (lclass == 1) {
        copy_from(u(p, 8), nbytes);
      } else if (lclass == 0) {
        p += 4 * ndim;
        const uint64_t csize = u(p, 4);
        copy_from(p + 4, csize);
      } else {
        throw Error("chunked layout v1/v2 unsupported");
      }
    } else if (version == 3) {
      const int lclass = b_[lp + 1];
      const uint64_t p = lp + 2;
      if (lclass == 0) {
        copy_from(p + 2, u(p, 2));
      } else if (lclass == 1) {
        copy_from(u(p, 8), nbytes);
      } else if (lclass == 2) {
        read_chunked(p, esize, shape, raw);
      } else {
        throw Error("unsupported layout class");
      }
    } else {
      throw Error("unsupported layout version");
    }
    return raw;
  }

  void read_chunked(uint64_t p, uint32_t esize, const std::vector<uint64_t> &shape,
                    std::vector<uint8_t> &out) {
    const int ndim = b_[p];  // dataset rank + 1 (element size dimension)
    const uint64_t btree = u(p + 1, 8);
    std::vector<uint64_t> cdims;
    for (int k = 0; k < ndim - 1; k++) cdims.push_back(u(p + 9 + 4 * k, 4));
    const int rank = ndim - 1;
    if ((int)shape.size() != rank) throw Error("chunk rank mismatch");
    std::vector<uint64_t> stack{btree};
    while (!stack.empty()) {
      const uint64_t addr = stack.back();
      stack.pop_back();
      if (!sig(addr, "TREE") || b_[addr + 4] != 1) throw Error("bad chunk B-tree");
      const int level = b_[addr + 5];
      const int used = (int)u(addr + 6, 2);
      uint64_t pos = addr + 24;
      for (int k = 0; k < used; k++) {
        const uint64_t csize = u(pos, 4), fmask = u(pos + 4, 4);
        std::vector<uint64_t> offs;
        for (int d = 0; d < ndim; d++) offs.push_back(u(pos + 8 + 8 * d, 8));
        pos += 8 + 8 * ndim;
        const uint64_t child = u(pos, 8);
        pos += 8;
        if (level > 0) {
          stack.push_back(child);
          continue;
        }
        if (fmask) throw Error("filtered chunks are unsupported");
        need(child, csize);
        // copy the chunk element by element into the row-major output
        size_t celems = 1;
        for (auto c : cdims) celems *= (size_t)c;
        std::vector<uint64_t> idx(rank, 0);
        for (size_t e = 0; e < celems; e++) {
          size_t rem = e;
          bool inside = true;
          size_t flat = 0;
          for (int d = rank - 1; d >= 0; d--) {
            idx[d] = rem % cdims[d];
            rem /= cdims[d];
          }
          for (int d = 0; d < rank; d++) {
            const uint64_t g = offs[d] + idx[d];
            if (g >= shape[d]) inside = false;
            flat = flat * (size_t)shape[d] + (size_t)g;
          }
          if (inside && (e + 1) * esize <= csize)
            std::memcpy(out.data() + flat * esize, b_.data() + child + e * esize, esize);
        }
      }
    }
  }

  Value decode(const Datatype &t, const std::vector<uint64_t> &shape, const uint8_t *raw,
               size_t count) {
    Value v;
    v.shape = shape;
    if (t.cls == 0 || t.cls == 1) {
      for (size_t k = 0; k < count; k++) {
        uint8_t tmp[8] = {0};
        const uint8_t *e = raw + k * t.size;
        for (uint32_t q = 0; q < t.size && q < 8; q++)
          tmp[q] = t.big_endian ? e[t.size - 1 - q] : e[q];
        if (t.cls == 1) {
          v.kind = Value::kFloat;
          if (t.size == 8) {
            double d;
            std::memcpy(&d, tmp, 8);
            v.floats.push_back(d);
          } else if (t.size == 4) {
            float f;
            std::memcpy(&f, tmp, 4);
            v.floats.push_back(f);
          } else {
            throw Error("unsupported float size");
          }
        } else {
          v.kind = Value::kInt;
          uint64_t x = 0;
          std::memcpy(&x, tmp, 8);
          int64_t s = (int64_t)x;
          if (t.is_signed && t.size < 8) {
            const int sh = 64 - 8 * (int)t.size;
            s = (int64_t)(x << sh) >> sh;
          }
          v.ints.push_back(s);
        }
      }
    } else if (t.cls == 3) {
      v.kind = Value::kString;
      for (size_t k = 0; k < count; k++) {
        std::string s(reinterpret_cast<const char *>(raw + k * t.size), t.size);
        s = s.substr(0, s.find('\0'));
        v.strings.push_back(s);
      }
    } else if (t.cls == 9) {
      v.kind = Value::kString;
      v.strings = vlen_strings(raw, count);
    }
    return v;
  }

  std::pair<std::string, Value> attribute(uint64_t pos) {
    const int version = b_[pos];
    const uint64_t name_size = u(pos + 2, 2), dt_size = u(pos + 4, 2), ds_size = u(pos + 6, 2);
    uint64_t p;
    std::string name;
    Datatype dt;
    std::vector<uint64_t> shape;
    if (version == 1) {
      p = pos + 8;
      name = cstr(p);
      p += (name_size + 7) / 8 * 8;
      dt = datatype(p);
      p += (dt_size + 7) / 8 * 8;
      if (!dataspace(p, shape)) shape.clear();
      p += (ds_size + 7) / 8 * 8;
    } else if (version == 2 || version == 3) {
      p = pos + 8 + (version == 3 ? 1 : 0);
      name = cstr(p);
      p += name_size;
      dt = datatype(p);
      p += dt_size;
      if (!dataspace(p, shape)) shape.clear();
      p += ds_size;
    } else {
      throw Error("unsupported attribute version");
    }
    const size_t count = count_of(shape);
    const size_t esize = dt.cls == 9 ? 16 : dt.size;
    need(p, count * esize);
    return {name, decode(dt, shape, b_.data() + p, count)};
  }

  std::unique_ptr<Node> load(const std::string &name, uint64_t header, int depth) {
    if (depth > 64) throw Error("group nesting too deep");
    auto node = std::make_unique<Node>();
    node->name = name;
    std::vector<uint64_t> shape;
    bool have_shape = false, have_type = false;
    Datatype dt;
    uint64_t layout = 0;
    bool have_layout = false;
    for (const Msg &m : messages(header)) {
      switch (m.type) {
        case 0x0011: {
          node->is_group = true;
          for (auto &e : group_entries(u(m.body, 8), u(m.body + 8, 8)))
            node->children[e.first] = load(e.first, e.second, depth + 1);
          break;
        }
        case 0x0001:
          have_shape = dataspace(m.body, shape);
          if (!have_shape) shape.clear();
          break;
        case 0x0003:
          dt = datatype(m.body);
          have_type = true;
          break;
        case 0x0008:
          layout = m.body;
          have_layout = true;
          break;
        case 0x000C: {
          auto a = attribute(m.body);
          node->attrs[a.first] = std::move(a.second);
          break;
        }
        case 0x0006:
          throw Error("link messages (new-style groups) are unsupported");
        default:
          break;
      }
    }
    if (have_layout && have_type) {
      const uint32_t esize = dt.cls == 9 ? 16 : dt.size;
      auto raw = read_raw(layout, esize, shape);
      node->value = decode(dt, shape, raw.data(), count_of(shape));
    }
    return node;
  }
};

std::string trim(const std::string &s) {
  size_t a = 0, b = s.size();
  while (a < b && (s[a] == ' ' || s[a] == '\0')) a++;
  while (b > a && (s[b - 1] == ' ' || s[b - 1] == '\0')) b--;
  return s.substr(a, b - a);
}

}  // namespace

size_t Value::size() const {
  return kind == kInt ? ints.size() : kind == kFloat ? floats.size() : strings.size();
}
double Value::as_double(size_t i) const {
  if (kind == kFloat) return floats.at(i);
  if (kind == kInt) return (double)ints.at(i);
  throw Error("value is not numeric");
}
int64_t Value::as_int(size_t i) const {
  if (kind == kInt) return ints.at(i);
  if (kind == kFloat) return (int64_t)floats.at(i);
  throw Error("value is not numeric");
}
std::vector<double> Value::doubles() const {
  std::vector<double> out;
  for (size_t k = 0; k < size(); k++) out.push_back(as_double(k));
  return out;
}
std::vector<int64_t> Value::integers() const {
  std::vector<int64_t> out;
  for (size_t k = 0; k < size(); k++) out.push_back(as_int(k));
  return out;
}
std::string Value::str(size_t i) const {
  if (kind != kString) throw Error("value is not a string");
  return trim(strings.at(i));
}

const Node &Node::operator[](const std::string &path) const {
  const Node *n = this;
  size_t pos = 0;
  while (pos <= path.size()) {
    const size_t next = path.find('/', pos);
    const std::string part = path.substr(pos, next == std::string::npos ? std::string::npos : next - pos);
    if (!part.empty() && part != ".") {
      auto it = n->children.find(part);
      if (it == n->children.end()) throw Error("'" + path + "': no member '" + part + "'");
      n = it->second.get();
    }
    if (next == std::string::npos) break;
    pos = next + 1;
  }
  return *n;
}

bool Node::has(const std::string &path) const {
  try {
    (void)(*this)[path];
    return true;
  } catch (const Error &) {
    return false;
  }
}

const Value &Node::attr(const std::string &name) const {
  auto it = attrs.find(name);
  if (it == attrs.end()) throw Error("no attribute '" + name + "' on '" + this->name + "'");
  return it->second;
}

std::unique_ptr<Node> read_bytes(std::vector<uint8_t> data) {
  Reader r(std::move(data));
  return r.load_root();
}

std::unique_ptr<Node> read(const std::string &path) {
  std::ifstream in(path, std::ios::binary);
  if (!in) throw Error("cannot open " + path);
  std::vector<uint8_t> data((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
  return read_bytes(std::move(data));
}

}  // namespace h5
}  // namespace fnet
