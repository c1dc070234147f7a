// h5lite.cpp -- HDF5 subset: see h5lite.h.  Field layouts follow the HDF5 file format
// specification (superblock, object headers and their messages, version-1 B-trees, symbol
// table nodes, local heaps); all offsets and lengths are 8 bytes.
#include "h5lite.h"

#include <algorithm>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>

namespace tlbm {
namespace h5 {

namespace {

constexpr uint64_t kUndef = ~uint64_t{0};
constexpr int kLeafK = 4;       // symbol table node: up to 2K entries
constexpr int kInternalK = 16;  // group B-tree node: up to 2K children
constexpr uint64_t kFreeNull = 1;  // a local heap's empty free list
constexpr size_t kSuperblock = 96;
constexpr size_t kBtreeNode = 24 + (2 * kInternalK + 1) * 8 + 2 * kInternalK * 8;
constexpr size_t kSymbolNode = 8 + 2 * kLeafK * 40;

uint64_t pad8(uint64_t v) { return (v + 7) & ~uint64_t{7}; }

// little-endian encoder into a growing byte image
struct Out {
  std::vector<uint8_t> b;
  void u8(unsigned v) { b.push_back(static_cast<uint8_t>(v)); }
  void le(uint64_t v, int n) {
    for (int i = 0; i < n; ++i) b.push_back(static_cast<uint8_t>(v >> (8 * i)));
  }
  void bytes(const void* p, size_t n) {
    const uint8_t* c = static_cast<const uint8_t*>(p);
    b.insert(b.end(), c, c + n);
  }
  void zeros(size_t n) { b.insert(b.end(), n, 0); }
};

// ---------------------------------------------------------------- writer

struct Node {
  std::string name;
  bool group = true;
  const Dataset* set = nullptr;
  std::map<std::string, std::unique_ptr<Node>> kids;  // sorted by name (byte order)
  // layout
  uint64_t header = 0, heap = 0, btree = 0, snod = 0, data = 0;
  std::vector<uint64_t> name_off;  // heap offsets of the children's names, in kids order
  uint64_t heap_data = 0;          // size of the heap's data segment
};

uint64_t header_size(const Node& n) {
  if (n.group) return 16 + 8 + 16;  // symbol table message
  const uint64_t r = n.set->dims.size();
  return 16 + (8 + 8 + 8 * r) + (8 + 24) + (8 + 8) + (8 + 24);
}

uint64_t count_of(const Dataset& d) {
  uint64_t c = 1;
  for (uint64_t e : d.dims) c *= e;
  return c;
}

void message(Out& o, unsigned type, uint64_t size) {
  o.le(type, 2);
  o.le(size, 2);
  o.u8(0);  // flags
  o.zeros(3);
}

void object_header(Out& o, const Node& n) {
  const uint64_t body = header_size(n) - 16;
  o.u8(1);  // version
  o.u8(0);
  o.le(n.group ? 1 : 4, 2);  // messages
  o.le(1, 4);                // reference count
  o.le(body, 4);
  o.zeros(4);
  if (n.group) {
    message(o, 0x0011, 16);  // symbol table: B-tree and local heap
    o.le(n.btree, 8);
    o.le(n.heap, 8);
    return;
  }
  const Dataset& d = *n.set;
  const uint64_t r = d.dims.size();
  message(o, 0x0001, 8 + 8 * r);  // dataspace, version 1, no maximum dimensions
  o.u8(1);
  o.u8(static_cast<unsigned>(r));
  o.u8(0);
  o.zeros(5);
  for (uint64_t e : d.dims) o.le(e, 8);
  message(o, 0x0003, 24);  // datatype, version 1, class 1 (floating point)
  o.u8(0x11);
  o.u8(0x20);  // little-endian, no padding, implied leading mantissa bit
  o.u8(31);    // sign bit position
  o.u8(0);
  o.le(4, 4);   // size in bytes
  o.le(0, 2);   // bit offset
  o.le(32, 2);  // bit precision
  o.u8(23);     // exponent location
  o.u8(8);      // exponent size
  o.u8(0);      // mantissa location
  o.u8(23);     // mantissa size
  o.le(127, 4);  // exponent bias
  o.zeros(4);
  message(o, 0x0005, 8);  // fill value, version 2: allocation late, write if set, undefined
  o.u8(2);
  o.u8(2);
  o.u8(2);
  o.u8(0);
  o.zeros(4);
  message(o, 0x0008, 24);  // data layout, version 3, contiguous
  o.u8(3);
  o.u8(1);
  o.le(n.data, 8);
  o.le(count_of(d) * 4, 8);
  o.zeros(6);
}

void group_structures(Out& o, const Node& n) {
  // local heap: header, then the data segment ("" at offset 0, then the children's names)
  o.bytes("HEAP", 4);
  o.u8(0);
  o.zeros(3);
  o.le(n.heap_data, 8);
  o.le(kFreeNull, 8);
  o.le(n.heap + 32, 8);
  o.zeros(8);
  for (const auto& kv : n.kids) {
    o.bytes(kv.first.data(), kv.first.size());
    o.zeros(pad8(kv.first.size() + 1) - kv.first.size());
  }
  // B-tree (one leaf level node, one child: the symbol table node)
  const size_t b0 = o.b.size();
  o.bytes("TREE", 4);
  o.u8(0);  // group node
  o.u8(0);  // level 0
  o.le(1, 2);
  o.le(kUndef, 8);
  o.le(kUndef, 8);
  o.le(0, 8);       // key 0: the empty string
  o.le(n.snod, 8);  // child 0
  o.le(n.name_off.empty() ? 0 : n.name_off.back(), 8);  // key 1: the last name
  o.zeros(kBtreeNode - (o.b.size() - b0));
  // symbol table node
  const size_t s0 = o.b.size();
  o.bytes("SNOD", 4);
  o.u8(1);
  o.u8(0);
  o.le(n.kids.size(), 2);
  size_t k = 0;
  for (const auto& kv : n.kids) {
    const Node& c = *kv.second;
    o.le(n.name_off[k++], 8);
    o.le(c.header, 8);
    o.le(c.group ? 1 : 0, 4);  // cache type 1: the group's B-tree and heap in the scratch pad
    o.zeros(4);
    o.le(c.group ? c.btree : 0, 8);
    o.le(c.group ? c.heap : 0, 8);
  }
  o.zeros(kSymbolNode - (o.b.size() - s0));
}

}  // namespace

bool write_f32(const std::string& file, const std::vector<Dataset>& sets, std::string* err) {
  Node root;
  for (const Dataset& d : sets) {
    Node* g = &root;
    size_t pos = 0;
    for (;;) {
      const size_t slash = d.path.find('/', pos);
      const std::string part =
          d.path.substr(pos, slash == std::string::npos ? slash : slash - pos);
      if (part.empty()) {
        *err = "empty name in " + d.path;
        return false;
      }
      auto& slot = g->kids[part];
      if (slash == std::string::npos) {
        if (slot) {
          *err = "duplicate object " + d.path;
          return false;
        }
        slot.reset(new Node);
        slot->name = part;
        slot->group = false;
        slot->set = &d;
        break;
      }
      if (!slot) {
        slot.reset(new Node);
        slot->name = part;
      } else if (!slot->group) {
        *err = part + " is a dataset, not a group, in " + d.path;
        return false;
      }
      g = slot.get();
      pos = slash + 1;
    }
  }
  // layout: superblock, then per group (depth first) its header, heap, B-tree and symbol table
  // node, each dataset's header; then every dataset's values
  std::vector<Node*> order;  // metadata objects in file order
  std::vector<Node*> stack = {&root};
  while (!stack.empty()) {
    Node* n = stack.back();
    stack.pop_back();
    order.push_back(n);
    if (n->group) {
      if (n->kids.size() > static_cast<size_t>(2 * kLeafK)) {
        *err = "more than " + std::to_string(2 * kLeafK) + " objects in one group";
        return false;
      }
      for (auto it = n->kids.rbegin(); it != n->kids.rend(); ++it)
        stack.push_back(it->second.get());
    }
  }
  uint64_t at = kSuperblock;
  for (Node* n : order) {
    n->header = at;
    at += header_size(*n);
    if (!n->group) continue;
    n->heap = at;
    uint64_t off = 8;
    for (const auto& kv : n->kids) {
      n->name_off.push_back(off);
      off += pad8(kv.first.size() + 1);
    }
    n->heap_data = off;
    at += 32 + off;
    n->btree = at;
    at += kBtreeNode;
    n->snod = at;
    at += kSymbolNode;
  }
  const uint64_t meta_end = at;
  for (Node* n : order) {
    if (n->group) continue;
    n->data = at;
    at += pad8(count_of(*n->set) * 4);
  }
  const uint64_t eof = at;

  Out o;
  o.bytes("\x89HDF\r\n\x1a\n", 8);
  o.u8(0);  // superblock version
  o.u8(0);  // free-space version
  o.u8(0);  // root symbol table entry version
  o.u8(0);
  o.u8(0);  // shared header message version
  o.u8(8);  // size of offsets
  o.u8(8);  // size of lengths
  o.u8(0);
  o.le(kLeafK, 2);
  o.le(kInternalK, 2);
  o.le(0, 4);  // consistency flags
  o.le(0, 8);  // base address
  o.le(kUndef, 8);
  o.le(eof, 8);
  o.le(kUndef, 8);
  o.le(0, 8);  // root entry: name offset, header, cache type 1 (B-tree, heap)
  o.le(root.header, 8);
  o.le(1, 4);
  o.zeros(4);
  o.le(root.btree, 8);
  o.le(root.heap, 8);
  for (Node* n : order) {
    object_header(o, *n);
    if (n->group) group_structures(o, *n);
  }
  if (o.b.size() != meta_end) {
    *err = "layout mismatch writing " + file;
    return false;
  }

  std::ofstream f(file, std::ios::binary | std::ios::trunc);
  if (!f.is_open()) {
    *err = "cannot open " + file + " for writing";
    return false;
  }
  f.write(reinterpret_cast<const char*>(o.b.data()), static_cast<std::streamsize>(o.b.size()));
  for (Node* n : order) {
    if (n->group) continue;
    if (static_cast<uint64_t>(f.tellp()) != n->data) {
      *err = "layout mismatch writing " + file;
      return false;
    }
    const uint64_t bytes = count_of(*n->set) * 4;
    f.write(reinterpret_cast<const char*>(n->set->data), static_cast<std::streamsize>(bytes));
    static const char zero[8] = {0};
    f.write(zero, static_cast<std::streamsize>(pad8(bytes) - bytes));
  }
  if (!f.good()) {
    *err = "write failed: " + file;
    return false;
  }
  return true;
}

// ---------------------------------------------------------------- reader

namespace {

struct Reader {
  std::ifstream f;
  uint64_t size = 0, base = 0;
  std::string err;

  bool read(uint64_t addr, void* dst, uint64_t n) {
    if (addr == kUndef || addr + base + n > size || addr + base + n < n) {
      err = "address out of the file";
      return false;
    }
    f.seekg(static_cast<std::streamoff>(addr + base));
    f.read(static_cast<char*>(dst), static_cast<std::streamsize>(n));
    if (!f.good()) {
      err = "read failed";
      return false;
    }
    return true;
  }
  bool bytes(uint64_t addr, uint64_t n, std::vector<uint8_t>* out) {
    out->resize(n);
    return n == 0 || read(addr, out->data(), n);
  }
};

uint64_t get(const uint8_t* p, int n) {
  uint64_t v = 0;
  for (int i = n - 1; i >= 0; --i) v = (v << 8) | p[i];
  return v;
}

struct Message {
  unsigned type;
  std::vector<uint8_t> data;
};

// the messages of the object header at `addr`, continuation blocks followed
bool header_messages(Reader& r, uint64_t addr, std::vector<Message>* out) {
  std::vector<uint8_t> b;
  if (!r.bytes(addr, 16, &b)) return false;
  struct Block {
    uint64_t addr, len;
    bool v2;
  };
  std::vector<Block> todo;
  if (b[0] == 1) {  // version 1: 16-byte prefix
    todo.push_back({addr + 16, get(&b[8], 4), false});
  } else if (std::memcmp(b.data(), "OHDR", 4) == 0 && b[4] == 2) {
    const unsigned flags = b[5];
    uint64_t p = 6;
    if (flags & 0x20) p += 16;  // access, modification, change, birth times
    if (flags & 0x10) p += 4;   // attribute storage phase change values
    const int w = 1 << (flags & 3);
    std::vector<uint8_t> h;
    if (!r.bytes(addr, p + w, &h)) return false;
    todo.push_back({addr + p + w, get(&h[p], w), true});
  } else {
    r.err = "unknown object header version";
    return false;
  }
  const bool order = b[0] != 1 && (b[5] & 0x04);  // v2: creation order fields present
  for (size_t t = 0; t < todo.size(); ++t) {
    const Block blk = todo[t];
    if (t > 200) {
      r.err = "too many header continuation blocks";
      return false;
    }
    std::vector<uint8_t> d;
    if (!r.bytes(blk.addr, blk.len, &d)) return false;
    uint64_t p = 0, end = blk.len;
    if (blk.v2 && t > 0) {  // continuation chunk: "OCHK", messages, checksum
      if (blk.len < 8 || std::memcmp(d.data(), "OCHK", 4) != 0) {
        r.err = "bad object header continuation chunk";
        return false;
      }
      p = 4;
      end = blk.len - 4;
    }
    const uint64_t hdr = blk.v2 ? (order ? 6 : 4) : 8;
    while (p + hdr <= end) {
      unsigned type;
      uint64_t size;
      if (blk.v2) {
        type = d[p];
        size = get(&d[p + 1], 2);
      } else {
        type = static_cast<unsigned>(get(&d[p], 2));
        size = get(&d[p + 2], 2);
      }
      p += hdr;
      if (p + size > end) {
        r.err = "truncated header message";
        return false;
      }
      Message m{type, std::vector<uint8_t>(d.begin() + p, d.begin() + p + size)};
      if (type == 0x0010) {  // continuation: address, length
        if (size < 16) {
          r.err = "bad continuation message";
          return false;
        }
        todo.push_back({get(&m.data[0], 8), get(&m.data[8], 8), blk.v2});
      } else if (type != 0) {
        out->push_back(std::move(m));
      }
      p += size;
    }
  }
  return true;
}

// null-terminated name at `off` of the local heap at `heap`
bool heap_name(Reader& r, uint64_t heap, uint64_t off, std::string* name) {
  std::vector<uint8_t> h;
  if (!r.bytes(heap, 32, &h)) return false;
  if (std::memcmp(h.data(), "HEAP", 4) != 0) {
    r.err = "bad local heap";
    return false;
  }
  const uint64_t size = get(&h[8], 8), data = get(&h[24], 8);
  if (off >= size) {
    r.err = "name offset outside the local heap";
    return false;
  }
  std::vector<uint8_t> s;
  if (!r.bytes(data + off, size - off, &s)) return false;
  const auto z = std::find(s.begin(), s.end(), 0);
  name->assign(s.begin(), z);
  return true;
}

// object header address of child `name` in the group B-tree rooted at `node`
bool btree_find(Reader& r, uint64_t node, uint64_t heap, const std::string& name, uint64_t* found,
                int depth) {
  if (depth > 64) {
    r.err = "group B-tree too deep";
    return false;
  }
  std::vector<uint8_t> h;
  if (!r.bytes(node, 24, &h)) return false;
  if (std::memcmp(h.data(), "TREE", 4) != 0 || h[4] != 0) {
    r.err = "bad group B-tree node";
    return false;
  }
  const int level = h[5];
  const uint64_t n = get(&h[6], 2);
  std::vector<uint8_t> kc;
  if (!r.bytes(node + 24, n * 16 + 8, &kc)) return false;
  for (uint64_t c = 0; c < n; ++c) {
    const uint64_t child = get(&kc[8 + 16 * c], 8);
    if (level > 0) {
      if (!btree_find(r, child, heap, name, found, depth + 1)) return false;
      if (*found != kUndef) return true;
      continue;
    }
    std::vector<uint8_t> s;
    if (!r.bytes(child, 8, &s)) return false;
    if (std::memcmp(s.data(), "SNOD", 4) != 0) {
      r.err = "bad symbol table node";
      return false;
    }
    const uint64_t entries = get(&s[6], 2);
    std::vector<uint8_t> e;
    if (!r.bytes(child + 8, entries * 40, &e)) return false;
    for (uint64_t k = 0; k < entries; ++k) {
      std::string nm;
      if (!heap_name(r, heap, get(&e[40 * k], 8), &nm)) return false;
      if (nm == name) {
        *found = get(&e[40 * k + 8], 8);
        return true;
      }
    }
  }
  return true;
}

// object header address of child `name` of the group whose header is at `group`
bool child(Reader& r, uint64_t group, const std::string& name, uint64_t* addr) {
  std::vector<Message> ms;
  if (!header_messages(r, group, &ms)) return false;
  *addr = kUndef;
  for (const Message& m : ms) {
    if (m.type == 0x0011 && m.data.size() >= 16) {  // symbol table
      if (!btree_find(r, get(&m.data[0], 8), get(&m.data[8], 8), name, addr, 0)) return false;
      if (*addr != kUndef) return true;
    } else if (m.type == 0x0006 && m.data.size() >= 2) {  // link
      const uint8_t* p = m.data.data();
      const uint8_t* e = p + m.data.size();
      const unsigned flags = p[1];
      p += 2;
      unsigned type = 0;
      if (flags & 0x08) type = *p++;
      if (flags & 0x04) p += 8;  // creation order
      if (flags & 0x10) p += 1;  // character set
      const int w = 1 << (flags & 3);
      if (p + w > e) continue;
      const uint64_t len = get(p, w);
      p += w;
      if (p + len > e) continue;
      const std::string nm(reinterpret_cast<const char*>(p), len);
      p += len;
      if (nm == name) {
        if (type != 0 || p + 8 > e) {
          r.err = "link " + name + " is not a hard link";
          return false;
        }
        *addr = get(p, 8);
        return true;
      }
    } else if (m.type == 0x0002 && m.data.size() >= 10) {  // link info: dense storage?
      const unsigned flags = m.data[1];
      const uint64_t heap = get(&m.data[(flags & 1) ? 10 : 2], 8);
      if (heap != kUndef) {
        r.err = "groups with dense link storage are not supported";
        return false;
      }
    }
  }
  r.err = "no object named " + name;
  return false;
}

}  // namespace

std::string read_f32(const std::string& file, const std::string& path, std::vector<float>* out,
                     std::vector<uint64_t>* dims) {
  Reader r;
  r.f.open(file, std::ios::binary | std::ios::ate);
  if (!r.f.is_open()) return "cannot open " + file;
  r.size = static_cast<uint64_t>(r.f.tellg());
  // the superblock sits at 0 or, after a user block, at 512, 1024, 2048, ...
  std::vector<uint8_t> sb;
  for (uint64_t at = 0;; at = at == 0 ? 512 : 2 * at) {
    if (at + 48 > r.size) return file + " is not an HDF5 file";
    if (!r.bytes(at, std::min<uint64_t>(r.size - at, 100), &sb)) return file + ": " + r.err;
    if (std::memcmp(sb.data(), "\x89HDF\r\n\x1a\n", 8) == 0) break;
  }
  uint64_t root = kUndef;
  const unsigned ver = sb[8];
  if (ver == 0 || ver == 1) {
    if (sb[13] != 8 || sb[14] != 8) return file + ": only 8-byte offsets and lengths are read";
    const size_t b = ver == 0 ? 24 : 28;  // version 1 adds the indexed-storage K
    if (sb.size() < b + 72) return file + ": truncated superblock";
    r.base = get(&sb[b], 8);
    root = get(&sb[b + 32 + 8], 8);  // root symbol table entry: its object header address
  } else if (ver == 2 || ver == 3) {
    if (sb[9] != 8 || sb[10] != 8) return file + ": only 8-byte offsets and lengths are read";
    r.base = get(&sb[12], 8);
    root = get(&sb[36], 8);
  } else {
    return file + ": unknown superblock version " + std::to_string(ver);
  }
  uint64_t obj = root;
  size_t pos = 0;
  while (pos < path.size()) {
    const size_t slash = path.find('/', pos);
    const std::string part = path.substr(pos, slash == std::string::npos ? slash : slash - pos);
    pos = slash == std::string::npos ? path.size() : slash + 1;
    if (part.empty()) continue;
    uint64_t next;
    if (!child(r, obj, part, &next)) return file + ": " + path + ": " + r.err;
    obj = next;
  }
  std::vector<Message> ms;
  if (!header_messages(r, obj, &ms)) return file + ": " + path + ": " + r.err;
  bool have_space = false, have_type = false, have_layout = false;
  unsigned elem = 0;
  uint64_t count = 1, addr = kUndef, stored = 0;
  std::vector<uint8_t> compact;
  dims->clear();
  for (const Message& m : ms) {
    const std::vector<uint8_t>& d = m.data;
    if (m.type == 0x0001 && d.size() >= 2) {  // dataspace
      const unsigned v = d[0], rank = d[1];
      const size_t at = v == 1 ? 8 : 4;
      if (d.size() < at + 8 * rank) return file + ": " + path + ": bad dataspace";
      for (unsigned k = 0; k < rank; ++k) {
        dims->push_back(get(&d[at + 8 * k], 8));
        count *= dims->back();
      }
      have_space = true;
    } else if (m.type == 0x0003 && d.size() >= 8) {  // datatype
      const unsigned cls = d[0] & 0x0F;
      elem = static_cast<unsigned>(get(&d[4], 4));
      if (cls != 1 || (d[1] & 1) != 0 || (elem != 4 && elem != 8))
        return file + ": " + path + ": only little-endian IEEE float32/float64 data is read";
      have_type = true;
    } else if (m.type == 0x0008 && d.size() >= 2) {  // data layout
      const unsigned v = d[0];
      if (v >= 3) {
        const unsigned cls = d[1];
        if (cls == 1 && d.size() >= 18) {
          addr = get(&d[2], 8);
          stored = get(&d[10], 8);
        } else if (cls == 0 && d.size() >= 4) {
          const uint64_t n = get(&d[2], 2);
          if (d.size() < 4 + n) return file + ": " + path + ": bad compact layout";
          compact.assign(d.begin() + 4, d.begin() + 4 + n);
          stored = n;
        } else {
          return file + ": " + path + ": chunked or virtual datasets are not supported";
        }
      } else if (v == 1 || v == 2) {
        const unsigned cls = d[2];
        if (cls != 1 || d.size() < 16) return file + ": " + path + ": unsupported layout";
        addr = get(&d[8], 8);
        stored = kUndef;
      } else {
        return file + ": " + path + ": unknown layout version";
      }
      have_layout = true;
    } else if (m.type == 0x000B) {
      return file + ": " + path + ": filtered (compressed) datasets are not supported";
    }
  }
  if (!have_space || !have_type || !have_layout) return file + ": " + path + " is not a dataset";
  const uint64_t bytes = count * elem;
  if (stored != kUndef && stored < bytes && compact.empty() && addr != kUndef)
    return file + ": " + path + ": stored size smaller than its dataspace";
  std::vector<uint8_t> raw;
  if (!compact.empty()) {
    if (compact.size() < bytes) return file + ": " + path + ": short compact data";
    raw.assign(compact.begin(), compact.begin() + bytes);
  } else if (addr == kUndef) {
    raw.assign(bytes, 0);  // never written: the default fill value
  } else if (!r.bytes(addr, bytes, &raw)) {
    return file + ": " + path + ": " + r.err;
  }
  out->resize(count);
  if (elem == 4) {
    std::memcpy(out->data(), raw.data(), bytes);
  } else {
    for (uint64_t k = 0; k < count; ++k) {
      double v;
      std::memcpy(&v, &raw[8 * k], 8);
      (*out)[k] = static_cast<float>(v);
    }
  }
  return "";
}

}  // namespace h5
}  // namespace tlbm
