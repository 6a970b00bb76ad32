// hdf5.cpp -- HDF5 file-format subset reader and writer (see hdf5.h).
//
// Written from the published HDF5 File Format Specification (superblock,
// object header, v1 B-tree, symbol table node, local heap and the message
// encodings of sections III and IV).  All multi-byte fields are little-endian;
// addresses are relative to the superblock's base address.
#include "hdf5.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <functional>
#include <memory>
#include <set>
#include <stdexcept>
#ifdef KNNG_HAVE_ZLIB
#include <zlib.h>
#endif

namespace knngio {
namespace h5 {
namespace {

const unsigned char kSig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
constexpr uint64_t kUndef = ~uint64_t(0);
constexpr int kMaxRank = 32;

[[noreturn]] void fail(const std::string& m) { throw std::runtime_error("HDF5: " + m); }

class File {
 public:
  File(const std::string& path, const char* mode) : path_(path), f_(std::fopen(path.c_str(), mode)) {
    if (!f_) fail("unable to open " + path);
  }
  ~File() {
    if (f_) std::fclose(f_);
  }
  File(const File&) = delete;
  File& operator=(const File&) = delete;
  uint64_t size() {
    if (fseeko(f_, 0, SEEK_END) != 0) fail("seek failed in " + path_);
    return uint64_t(ftello(f_));
  }
  void read_at(uint64_t off, void* p, size_t n) {
    if (fseeko(f_, off_t(off), SEEK_SET) != 0 || std::fread(p, 1, n, f_) != n)
      fail("truncated file " + path_ + " (reading " + std::to_string(n) + " bytes at " + std::to_string(off) + ")");
  }
  std::vector<uint8_t> read_vec(uint64_t off, size_t n) {
    std::vector<uint8_t> v(n);
    if (n) read_at(off, v.data(), n);
    return v;
  }
  void write(const void* p, size_t n) {
    if (n && std::fwrite(p, 1, n, f_) != n) fail("short write to " + path_);
  }
  void close() {
    FILE* f = f_;
    f_ = nullptr;
    if (std::fclose(f) != 0) fail("close failed for " + path_);
  }
  const std::string& path() const { return path_; }

 private:
  std::string path_;
  FILE* f_;
};

// Bounds-checked little-endian cursor over a decoded block.
struct Cur {
  const uint8_t* p;
  size_t n;
  size_t pos = 0;
  Cur(const uint8_t* p_, size_t n_) : p(p_), n(n_) {}
  explicit Cur(const std::vector<uint8_t>& v) : p(v.data()), n(v.size()) {}
  void need(size_t k) const {
    if (pos + k > n) fail("malformed file (record overrun)");
  }
  uint64_t u(int bytes) {
    need(size_t(bytes));
    uint64_t v = 0;
    for (int i = 0; i < bytes; ++i) v |= uint64_t(p[pos + size_t(i)]) << (8 * i);
    pos += size_t(bytes);
    return v;
  }
  uint8_t u8() { return uint8_t(u(1)); }
  void skip(size_t k) {
    need(k);
    pos += k;
  }
  const uint8_t* at() const { return p + pos; }
  size_t left() const { return n - pos; }
};

uint64_t addr_or_undef(Cur& c, int so) {
  const uint64_t v = c.u(so);
  return (so < 8 && v == (uint64_t(1) << (8 * so)) - 1) ? kUndef : v;
}

struct Message {
  int type;
  int flags;
  std::vector<uint8_t> data;
};

struct Dtype {
  int cls = -1;
  int size = 0;
  bool le = true;
  bool sgn = false;
  int str_pad = 0;
};

struct Space {
  bool null = false;
  std::vector<uint64_t> dims;  // empty for a scalar
  uint64_t count() const {
    uint64_t c = 1;
    for (uint64_t d : dims) c *= d;
    return null ? 0 : c;
  }
};

struct Filter {
  int id;
  std::vector<uint32_t> cd;
};

struct Layout {
  int cls = -1;             // 0 compact, 1 contiguous, 2 chunked
  uint64_t addr = kUndef;   // contiguous data / chunk index address
  uint64_t size = 0;        // contiguous bytes
  std::vector<uint8_t> compact;
  std::vector<uint64_t> chunk;  // chunk dims (dataset rank entries)
  int index = 0;            // chunk index: 0 v1 B-tree, 1 single, 2 implicit, 3 fixed array, ...
  uint64_t single_size = 0; // filtered single chunk: stored size
  uint32_t single_mask = 0;
  bool single_filtered = false;
};

struct Object {
  std::vector<Message> msgs;
  const Message* find(int type) const {
    for (const auto& m : msgs)
      if (m.type == type) return &m;
    return nullptr;
  }
};

class Reader {
 public:
  explicit Reader(const std::string& path) : f_(path, "rb") { open_super(); }

  uint64_t root() const { return root_; }

  // All messages of the object header at `addr` (versions 1 and 2), with
  // continuation blocks followed.
  Object object(uint64_t addr);

  Dtype dtype(const Message& m) const;
  Space space(const Message& m) const;
  Layout layout(const Message& m) const;
  std::vector<Filter> filters(const Message& m) const;
  // (name, object header address) of every link of a group object.
  std::vector<std::pair<std::string, uint64_t>> links(const Object& g);
  // Raw element bytes of a dataset, row-major, written into dst (count*size).
  void read_raw(const Object& o, const Dtype& t, const Space& s, uint8_t* dst);

  int so() const { return so_; }
  int sl() const { return sl_; }
  File& file() { return f_; }
  uint64_t abs(uint64_t a) const {
    if (a == kUndef) fail("undefined address in " + f_.path());
    return base_ + a;
  }

 private:
  void open_super();
  void parse_msgs_v1(const std::vector<uint8_t>& blk, Object& o, std::vector<std::pair<uint64_t, uint64_t>>& cont);
  void parse_msgs_v2(const std::vector<uint8_t>& blk, size_t start, size_t end, bool crt, Object& o,
                     std::vector<std::pair<uint64_t, uint64_t>>& cont);
  void symtab_links(uint64_t btree, uint64_t heap, std::vector<std::pair<std::string, uint64_t>>& out);
  void chunks_btree(uint64_t node, int ndims, int depth, const std::function<void(const uint64_t*, uint64_t, uint32_t, uint64_t)>& fn);

  File f_;
  int so_ = 8, sl_ = 8;
  uint64_t base_ = 0, root_ = kUndef;
};

void Reader::open_super() {
  const uint64_t fsize = f_.size();
  uint64_t at = 0;
  for (;;) {
    if (at + 8 > fsize) fail("no HDF5 superblock in " + f_.path());
    unsigned char sig[8];
    f_.read_at(at, sig, 8);
    if (std::memcmp(sig, kSig, 8) == 0) break;
    at = at ? at * 2 : 512;
  }
  const std::vector<uint8_t> sb = f_.read_vec(at, size_t(std::min<uint64_t>(fsize - at, 256)));
  Cur c(sb);
  c.skip(8);
  const int ver = c.u8();
  if (ver == 0 || ver == 1) {
    c.skip(3);  // free-space, root symbol table and reserved version bytes
    c.skip(1);  // shared header message format version
    so_ = c.u8();
    sl_ = c.u8();
    c.skip(1);
    c.skip(4);  // group leaf / internal node K
    c.skip(4);  // file consistency flags
    if (ver == 1) c.skip(4);
    if ((so_ != 2 && so_ != 4 && so_ != 8) || (sl_ != 2 && sl_ != 4 && sl_ != 8)) fail("bad offset/length sizes");
    base_ = c.u(so_);
    c.skip(size_t(3 * so_));  // free-space info, end of file, driver info
    c.skip(size_t(so_));      // root link name offset
    root_ = addr_or_undef(c, so_);
  } else if (ver == 2 || ver == 3) {
    so_ = c.u8();
    sl_ = c.u8();
    c.skip(1);
    if ((so_ != 2 && so_ != 4 && so_ != 8) || (sl_ != 2 && sl_ != 4 && sl_ != 8)) fail("bad offset/length sizes");
    base_ = c.u(so_);
    c.skip(size_t(2 * so_));  // superblock extension, end of file
    root_ = addr_or_undef(c, so_);
  } else {
    fail("superblock version " + std::to_string(ver) + " not supported");
  }
  // A file that was given a user block after it was written still stores its
  // old base address; the superblock's own position is authoritative.
  base_ = at;
  if (root_ == kUndef) fail("no root group in " + f_.path());
}

void Reader::parse_msgs_v1(const std::vector<uint8_t>& blk, Object& o, std::vector<std::pair<uint64_t, uint64_t>>& cont) {
  Cur c(blk);
  while (c.left() >= 8) {
    const int type = int(c.u(2));
    const size_t size = size_t(c.u(2));
    const int flags = c.u8();
    c.skip(3);
    c.need(size);
    Message m{type, flags, std::vector<uint8_t>(c.at(), c.at() + size)};
    c.skip(size);
    if (type == 0x10) {
      Cur d(m.data);
      const uint64_t a = d.u(so_), l = d.u(sl_);
      cont.emplace_back(a, l);
    } else if (type != 0) {
      o.msgs.push_back(std::move(m));
    }
  }
}

void Reader::parse_msgs_v2(const std::vector<uint8_t>& blk, size_t start, size_t end, bool crt, Object& o,
                           std::vector<std::pair<uint64_t, uint64_t>>& cont) {
  Cur c(blk.data(), end);
  c.pos = start;
  const size_t hdr = crt ? 6 : 4;
  while (c.left() >= hdr) {  // fewer bytes than a message header is the gap
    const int type = c.u8();
    const size_t size = size_t(c.u(2));
    const int flags = c.u8();
    if (crt) c.skip(2);
    c.need(size);
    Message m{type, flags, std::vector<uint8_t>(c.at(), c.at() + size)};
    c.skip(size);
    if (type == 0x10) {
      Cur d(m.data);
      const uint64_t a = d.u(so_), l = d.u(sl_);
      cont.emplace_back(a, l);
    } else if (type != 0) {
      o.msgs.push_back(std::move(m));
    }
  }
}

Object Reader::object(uint64_t addr) {
  Object o;
  std::vector<std::pair<uint64_t, uint64_t>> cont;
  const uint64_t at = abs(addr);
  uint8_t pre[40] = {0};
  const uint64_t fsize = f_.size();
  if (at >= fsize) fail("object header address out of file");
  f_.read_at(at, pre, size_t(std::min<uint64_t>(sizeof pre, fsize - at)));
  bool v2 = false, crt = false;
  if (std::memcmp(pre, "OHDR", 4) == 0) {
    v2 = true;
    if (pre[4] != 2) fail("object header version " + std::to_string(pre[4]) + " not supported");
    const int flags = pre[5];
    crt = (flags & 0x04) != 0;
    size_t p = 6;
    if (flags & 0x20) p += 16;
    if (flags & 0x10) p += 4;
    const int w = 1 << (flags & 3);
    Cur c(pre, sizeof pre);
    c.pos = p;
    const uint64_t size0 = c.u(w);
    p += size_t(w);
    const std::vector<uint8_t> blk = f_.read_vec(at, size_t(p + size0));
    parse_msgs_v2(blk, p, blk.size(), crt, o, cont);
  } else if (pre[0] == 1) {
    Cur c(pre, sizeof pre);
    c.skip(4);
    c.skip(4);  // reference count
    const uint64_t size0 = c.u(4);
    parse_msgs_v1(f_.read_vec(at + 16, size_t(size0)), o, cont);
  } else {
    fail("unknown object header at address " + std::to_string(addr));
  }
  std::set<uint64_t> seen;
  for (size_t i = 0; i < cont.size(); ++i) {
    const auto [a, l] = cont[i];
    if (!seen.insert(a).second || seen.size() > 65536 || l > (uint64_t(1) << 32)) fail("malformed object header continuation");
    const std::vector<uint8_t> blk = f_.read_vec(abs(a), size_t(l));
    if (v2) {
      if (blk.size() < 8 || std::memcmp(blk.data(), "OCHK", 4) != 0) fail("bad object header continuation block");
      parse_msgs_v2(blk, 4, blk.size() - 4, crt, o, cont);
    } else {
      parse_msgs_v1(blk, o, cont);
    }
  }
  return o;
}

Dtype Reader::dtype(const Message& m) const {
  if (m.flags & 0x02) fail("shared (committed) datatypes not supported");
  Cur c(m.data);
  const int b0 = c.u8();
  const uint32_t bits = uint32_t(c.u(3));
  Dtype t;
  t.cls = b0 & 0x0f;
  t.size = int(c.u(4));
  if (t.cls == 0) {
    t.le = (bits & 1) == 0;
    t.sgn = (bits & 8) != 0;
    const int off = int(c.u(2)), prec = int(c.u(2));
    if (off != 0 || prec != 8 * t.size || (t.size != 1 && t.size != 2 && t.size != 4 && t.size != 8))
      fail("fixed-point layout (size " + std::to_string(t.size) + ", precision " + std::to_string(prec) + ") not supported");
  } else if (t.cls == 1) {
    if (bits & 0x40) fail("VAX-order floating point not supported");
    t.le = (bits & 1) == 0;
    t.sgn = true;
    const int sign = int((bits >> 8) & 0xff);
    const int off = int(c.u(2)), prec = int(c.u(2));
    const int eloc = c.u8(), esz = c.u8(), mloc = c.u8(), msz = c.u8();
    const uint32_t bias = uint32_t(c.u(4));
    const bool ieee = off == 0 && prec == 8 * t.size && mloc == 0 && eloc == msz && sign == prec - 1 &&
                      ((t.size == 2 && esz == 5 && msz == 10 && bias == 15) ||
                       (t.size == 4 && esz == 8 && msz == 23 && bias == 127) ||
                       (t.size == 8 && esz == 11 && msz == 52 && bias == 1023));
    if (!ieee) fail("non-IEEE floating-point layout not supported");
  } else if (t.cls == 3) {
    t.str_pad = int(bits & 0x0f);
  }
  return t;
}

Space Reader::space(const Message& m) const {
  Cur c(m.data);
  const int ver = c.u8();
  const int rank = c.u8();
  c.u8();  // flags
  Space s;
  if (ver == 1) {
    c.skip(5);
  } else if (ver == 2) {
    const int type = c.u8();
    s.null = type == 2;
  } else {
    fail("dataspace version " + std::to_string(ver) + " not supported");
  }
  if (rank > kMaxRank) fail("dataspace rank too large");
  for (int i = 0; i < rank; ++i) s.dims.push_back(c.u(sl_));
  return s;
}

Layout Reader::layout(const Message& m) const {
  Cur c(m.data);
  const int ver = c.u8();
  Layout l;
  if (ver == 3 || ver == 4) {
    l.cls = c.u8();
    if (l.cls == 0) {
      const size_t n = size_t(c.u(2));
      c.need(n);
      l.compact.assign(c.at(), c.at() + n);
    } else if (l.cls == 1) {
      l.addr = addr_or_undef(c, so_);
      l.size = c.u(sl_);
    } else if (l.cls == 2 && ver == 3) {
      const int nd = c.u8();
      if (nd < 1 || nd > kMaxRank + 1) fail("bad chunk dimensionality");
      l.addr = addr_or_undef(c, so_);
      for (int i = 0; i < nd; ++i) l.chunk.push_back(c.u(4));
      l.chunk.pop_back();  // trailing entry is the element size
      l.index = 0;
    } else if (l.cls == 2) {
      const int flags = c.u8();
      const int nd = c.u8();
      const int w = c.u8();
      if (nd < 1 || nd > kMaxRank + 1 || w < 1 || w > 8) fail("bad chunk dimensionality");
      for (int i = 0; i < nd; ++i) l.chunk.push_back(c.u(w));
      l.chunk.pop_back();
      l.index = c.u8();
      if (l.index == 1) {
        if (flags & 0x02) {
          l.single_filtered = true;
          l.single_size = c.u(sl_);
          l.single_mask = uint32_t(c.u(4));
        }
      } else if (l.index == 3) {
        c.skip(1);  // page bits
      } else if (l.index != 2) {
        fail("chunk index type " + std::to_string(l.index) + " (extensible array / v2 B-tree) not supported");
      }
      l.addr = addr_or_undef(c, so_);
    } else {
      fail("layout class " + std::to_string(l.cls) + " not supported");
    }
  } else if (ver == 1 || ver == 2) {
    const int nd = c.u8();
    l.cls = c.u8();
    c.skip(5);
    if (l.cls != 0) l.addr = addr_or_undef(c, so_);
    std::vector<uint64_t> d;
    for (int i = 0; i < nd; ++i) d.push_back(c.u(4));
    if (l.cls == 1) {
      l.size = kUndef;  // implied by the dataspace and datatype
    } else if (l.cls == 2) {
      d.pop_back();
      l.chunk = d;
      l.index = 0;
    } else {
      const size_t n = size_t(c.u(4));
      c.need(n);
      l.compact.assign(c.at(), c.at() + n);
    }
  } else {
    fail("layout version " + std::to_string(ver) + " not supported");
  }
  return l;
}

std::vector<Filter> Reader::filters(const Message& m) const {
  Cur c(m.data);
  const int ver = c.u8();
  const int nf = c.u8();
  if (ver == 1) c.skip(6);
  else if (ver != 2) fail("filter pipeline version " + std::to_string(ver) + " not supported");
  std::vector<Filter> out;
  for (int i = 0; i < nf; ++i) {
    Filter f;
    f.id = int(c.u(2));
    size_t name_len = 0;
    if (ver == 1 || f.id >= 256) name_len = size_t(c.u(2));
    c.u(2);  // flags
    const int nv = int(c.u(2));
    if (ver == 1) name_len = (name_len + 7) & ~size_t(7);
    c.skip(name_len);
    for (int k = 0; k < nv; ++k) f.cd.push_back(uint32_t(c.u(4)));
    if (ver == 1 && (nv & 1)) c.skip(4);
    out.push_back(f);
  }
  return out;
}

void Reader::symtab_links(uint64_t btree, uint64_t heap, std::vector<std::pair<std::string, uint64_t>>& out) {
  const std::vector<uint8_t> hh = f_.read_vec(abs(heap), size_t(8 + 2 * sl_ + so_));
  if (std::memcmp(hh.data(), "HEAP", 4) != 0) fail("bad local heap signature");
  Cur hc(hh);
  hc.skip(8);
  const uint64_t seg_size = hc.u(sl_);
  hc.u(sl_);  // free list head
  const uint64_t seg_addr = hc.u(so_);
  if (seg_size > (uint64_t(1) << 32)) fail("local heap too large");
  const std::vector<uint8_t> seg = f_.read_vec(abs(seg_addr), size_t(seg_size));
  auto name_at = [&](uint64_t off) {
    if (off >= seg.size()) fail("link name outside the local heap");
    const char* s = reinterpret_cast<const char*>(seg.data() + off);
    return std::string(s, strnlen(s, seg.size() - size_t(off)));
  };
  std::set<uint64_t> seen;
  std::function<void(uint64_t, int)> walk = [&](uint64_t node, int depth) {
    if (depth > 64 || !seen.insert(node).second) fail("malformed group B-tree");
    const size_t hdr = size_t(8 + 2 * so_);
    const std::vector<uint8_t> h = f_.read_vec(abs(node), hdr);
    if (std::memcmp(h.data(), "TREE", 4) != 0 || h[4] != 0) fail("bad group B-tree node");
    const int level = h[5];
    const int n = int(h[6] | (h[7] << 8));
    const std::vector<uint8_t> body = f_.read_vec(abs(node) + hdr, size_t((n + 1) * sl_ + n * so_));
    Cur c(body);
    for (int i = 0; i < n; ++i) {
      c.skip(size_t(sl_));
      const uint64_t child = c.u(so_);
      if (level > 0) {
        walk(child, depth + 1);
        continue;
      }
      const std::vector<uint8_t> sh = f_.read_vec(abs(child), 8);
      if (std::memcmp(sh.data(), "SNOD", 4) != 0) fail("bad symbol table node");
      const int ns = int(sh[6] | (sh[7] << 8));
      const size_t esz = size_t(2 * so_ + 24);
      const std::vector<uint8_t> ents = f_.read_vec(abs(child) + 8, size_t(ns) * esz);
      Cur e(ents);
      for (int k = 0; k < ns; ++k) {
        const uint64_t name_off = e.u(so_);
        const uint64_t oh = e.u(so_);
        e.skip(24);
        out.emplace_back(name_at(name_off), oh);
      }
    }
  };
  walk(btree, 0);
}

std::vector<std::pair<std::string, uint64_t>> Reader::links(const Object& g) {
  std::vector<std::pair<std::string, uint64_t>> out;
  for (const auto& m : g.msgs) {
    if (m.type == 0x11) {
      Cur c(m.data);
      const uint64_t bt = c.u(so_), hp = c.u(so_);
      symtab_links(bt, hp, out);
    } else if (m.type == 0x02) {
      Cur c(m.data);
      c.u8();
      const int flags = c.u8();
      if (flags & 1) c.skip(8);
      if (addr_or_undef(c, so_) != kUndef) fail("dense group storage (fractal heap) not supported");
    } else if (m.type == 0x06) {
      Cur c(m.data);
      if (c.u8() != 1) fail("link message version not supported");
      const int flags = c.u8();
      int ltype = 0;
      if (flags & 0x08) ltype = c.u8();
      if (flags & 0x04) c.skip(8);
      if (flags & 0x10) c.u8();
      const size_t len = size_t(c.u(1 << (flags & 3)));
      c.need(len);
      std::string name(reinterpret_cast<const char*>(c.at()), len);
      c.skip(len);
      if (ltype == 0) out.emplace_back(name, c.u(so_));  // soft and external links are not followed
    }
  }
  return out;
}

void Reader::chunks_btree(uint64_t node, int ndims, int depth,
                          const std::function<void(const uint64_t*, uint64_t, uint32_t, uint64_t)>& fn) {
  if (depth > 64) fail("malformed chunk B-tree");
  const size_t hdr = size_t(8 + 2 * so_);
  const std::vector<uint8_t> h = f_.read_vec(abs(node), hdr);
  if (std::memcmp(h.data(), "TREE", 4) != 0 || h[4] != 1) fail("bad chunk B-tree node");
  const int level = h[5];
  const int n = int(h[6] | (h[7] << 8));
  const size_t ksz = size_t(8 + 8 * (ndims + 1));
  const std::vector<uint8_t> body = f_.read_vec(abs(node) + hdr, size_t(n + 1) * ksz + size_t(n * so_));
  Cur c(body);
  uint64_t off[kMaxRank + 1];
  for (int i = 0; i < n; ++i) {
    const uint64_t size = c.u(4);
    const uint32_t mask = uint32_t(c.u(4));
    for (int d = 0; d <= ndims; ++d) off[d] = c.u(8);
    const uint64_t child = c.u(so_);
    if (level > 0) chunks_btree(child, ndims, depth + 1, fn);
    else fn(off, size, mask, child);
  }
}

// Reverses the filter pipeline on one stored chunk.
std::vector<uint8_t> unfilter(std::vector<uint8_t> buf, const std::vector<Filter>& fl, uint32_t mask, size_t expect, int esz) {
  for (int i = int(fl.size()) - 1; i >= 0; --i) {
    if (mask & (1u << i)) continue;
    const Filter& f = fl[size_t(i)];
    if (f.id == 1) {
#ifdef KNNG_HAVE_ZLIB
      std::vector<uint8_t> out(std::max<size_t>(expect, 1));
      uLongf n = uLongf(out.size());
      const int rc = uncompress(out.data(), &n, buf.data(), uLong(buf.size()));
      if (rc != Z_OK) fail("deflate stream error " + std::to_string(rc));
      out.resize(size_t(n));
      buf.swap(out);
#else
      fail("deflate-compressed dataset needs a build with zlib");
#endif
    } else if (f.id == 2) {
      const size_t w = f.cd.empty() ? size_t(esz) : size_t(f.cd[0]);
      if (w > 1) {
        const size_t n = buf.size() / w;
        std::vector<uint8_t> out(buf.size());
        for (size_t b = 0; b < w; ++b)
          for (size_t k = 0; k < n; ++k) out[k * w + b] = buf[b * n + k];
        std::copy(buf.begin() + std::ptrdiff_t(n * w), buf.end(), out.begin() + std::ptrdiff_t(n * w));
        buf.swap(out);
      }
    } else if (f.id == 3) {
      if (buf.size() < 4) fail("fletcher32 chunk too short");
      buf.resize(buf.size() - 4);
    } else {
      fail("filter " + std::to_string(f.id) + " not supported (deflate, shuffle and fletcher32 are)");
    }
  }
  if (buf.size() != expect) fail("chunk decodes to " + std::to_string(buf.size()) + " bytes, expected " + std::to_string(expect));
  return buf;
}

void Reader::read_raw(const Object& o, const Dtype& t, const Space& s, uint8_t* dst) {
  const Message* lm = o.find(0x08);
  if (!lm) fail("dataset has no layout message");
  const Layout l = layout(*lm);
  const size_t esz = size_t(t.size);
  const uint64_t count = s.count();
  const uint64_t total = count * esz;
  if (l.cls == 0) {
    if (l.compact.size() < total) fail("compact data shorter than the dataspace");
    std::memcpy(dst, l.compact.data(), size_t(total));
    return;
  }
  if (l.cls == 1) {
    if (l.addr == kUndef) {
      std::memset(dst, 0, size_t(total));
      return;
    }
    if (l.size != kUndef && l.size < total) fail("contiguous storage shorter than the dataspace");
    f_.read_at(abs(l.addr), dst, size_t(total));
    return;
  }
  const int rank = int(s.dims.size());
  if (rank == 0 || int(l.chunk.size()) != rank) fail("chunk rank does not match the dataspace");
  std::vector<Filter> fl;
  if (const Message* pm = o.find(0x0B)) fl = filters(*pm);
  uint64_t cel = 1;
  for (uint64_t c : l.chunk) {
    if (c == 0) fail("zero chunk dimension");
    cel *= c;
  }
  const size_t cbytes = size_t(cel * esz);
  std::memset(dst, 0, size_t(total));
  // Copies one decoded chunk whose first element sits at `off` into dst.
  auto place = [&](const uint64_t* off, const std::vector<uint8_t>& ch) {
    for (int d = 0; d < rank; ++d)
      if (off[d] >= s.dims[size_t(d)]) return;
    const uint64_t run = std::min(l.chunk[size_t(rank - 1)], s.dims[size_t(rank - 1)] - off[rank - 1]);
    const uint64_t rows = cel / l.chunk[size_t(rank - 1)];
    for (uint64_t r = 0; r < rows; ++r) {
      uint64_t rem = r, dofs = 0, stride = 1;
      bool inside = true;
      for (int d = rank - 1; d >= 0; --d) {
        uint64_t idx = off[d];
        if (d < rank - 1) {
          idx += rem % l.chunk[size_t(d)];
          rem /= l.chunk[size_t(d)];
          if (idx >= s.dims[size_t(d)]) inside = false;
        }
        dofs += idx * stride;
        stride *= s.dims[size_t(d)];
      }
      if (inside) std::memcpy(dst + dofs * esz, ch.data() + r * l.chunk[size_t(rank - 1)] * esz, size_t(run * esz));
    }
  };
  if (l.addr == kUndef) return;  // no chunk was ever written
  // Chunk grid in row-major order (fixed-array and implicit indexes).
  std::vector<uint64_t> grid(static_cast<size_t>(rank));
  uint64_t nchunks = 1;
  for (int d = 0; d < rank; ++d) {
    grid[size_t(d)] = (s.dims[size_t(d)] + l.chunk[size_t(d)] - 1) / l.chunk[size_t(d)];
    nchunks *= grid[size_t(d)];
  }
  auto grid_offset = [&](uint64_t i, uint64_t* off) {
    for (int d = rank - 1; d >= 0; --d) {
      off[d] = (i % grid[size_t(d)]) * l.chunk[size_t(d)];
      i /= grid[size_t(d)];
    }
  };
  uint64_t off[kMaxRank + 1] = {0};
  if (l.index == 0) {
    chunks_btree(l.addr, rank, 0, [&](const uint64_t* o2, uint64_t size, uint32_t mask, uint64_t a) {
      place(o2, unfilter(f_.read_vec(abs(a), size_t(size)), fl, mask, cbytes, t.size));
    });
  } else if (l.index == 1) {
    const size_t sz = l.single_filtered ? size_t(l.single_size) : cbytes;
    place(off, unfilter(f_.read_vec(abs(l.addr), sz), fl, l.single_mask, cbytes, t.size));
  } else if (l.index == 2) {
    for (uint64_t i = 0; i < nchunks; ++i) {
      grid_offset(i, off);
      place(off, unfilter(f_.read_vec(abs(l.addr) + i * cbytes, cbytes), fl, 0, cbytes, t.size));
    }
  } else {
    const std::vector<uint8_t> hb = f_.read_vec(abs(l.addr), size_t(8 + sl_ + so_));
    if (std::memcmp(hb.data(), "FAHD", 4) != 0) fail("bad fixed array header");
    const int client = hb[5], entry = hb[6], page_bits = hb[7];
    Cur hc(hb);
    hc.skip(8);
    const uint64_t nel = hc.u(sl_);
    const uint64_t dblk = hc.u(so_);
    if (nel != nchunks) fail("fixed array length does not match the chunk grid");
    if (page_bits < 64 && nel > (uint64_t(1) << page_bits)) fail("paged fixed array chunk index not supported");
    const int csz = client == 1 ? entry - so_ - 4 : 0;
    if (csz < 0 || csz > 8) fail("bad fixed array entry size");
    const std::vector<uint8_t> db = f_.read_vec(abs(dblk), size_t(6 + so_) + size_t(nel) * size_t(entry));
    if (std::memcmp(db.data(), "FADB", 4) != 0) fail("bad fixed array data block");
    Cur dc(db);
    dc.skip(size_t(6 + so_));
    for (uint64_t i = 0; i < nel; ++i) {
      const uint64_t a = addr_or_undef(dc, so_);
      uint64_t size = cbytes;
      uint32_t mask = 0;
      if (client == 1) {
        size = dc.u(csz);
        mask = uint32_t(dc.u(4));
      }
      if (a == kUndef) continue;
      grid_offset(i, off);
      place(off, unfilter(f_.read_vec(abs(a), size_t(size)), fl, mask, cbytes, t.size));
    }
  }
}

float half_to_float(uint16_t h) {
  const uint32_t s = uint32_t(h >> 15) << 31, e = (h >> 10) & 0x1f;
  uint32_t m = h & 0x3ff, bits;
  if (e == 0) {
    if (m == 0) {
      bits = s;
    } else {  // subnormal half: normalise into a float
      int sh = 0;
      while (!(m & 0x400)) {
        m <<= 1;
        ++sh;
      }
      bits = s | (uint32_t(127 - 15 - sh + 1) << 23) | ((m & 0x3ff) << 13);
    }
  } else if (e == 31) {
    bits = s | 0x7f800000u | (m << 13);
  } else {
    bits = s | ((e + 127 - 15) << 23) | (m << 13);
  }
  float f;
  std::memcpy(&f, &bits, 4);
  return f;
}

uint64_t load(const uint8_t* p, int size, bool le) {
  uint64_t v = 0;
  for (int i = 0; i < size; ++i) v |= uint64_t(p[le ? i : size - 1 - i]) << (8 * i);
  return v;
}

int64_t as_int(uint64_t v, const Dtype& t) {
  if (t.sgn && t.size < 8 && (v >> (8 * t.size - 1)) & 1) v |= ~uint64_t(0) << (8 * t.size);
  return int64_t(v);
}

double as_double(const uint8_t* p, const Dtype& t) {
  const uint64_t v = load(p, t.size, t.le);
  if (t.cls == 0) return t.sgn ? double(as_int(v, t)) : double(v);
  if (t.size == 2) return half_to_float(uint16_t(v));
  if (t.size == 4) {
    const uint32_t b = uint32_t(v);
    float f;
    std::memcpy(&f, &b, 4);
    return f;
  }
  double d;
  std::memcpy(&d, &v, 8);
  return d;
}

bool is_dataset(const Object& o) { return o.find(0x01) && o.find(0x03) && o.find(0x08); }
bool is_group(const Object& o) { return o.find(0x11) || o.find(0x06) || o.find(0x02); }

std::string strip(const std::string& name) {
  size_t a = 0;
  while (a < name.size() && name[a] == '/') ++a;
  return name.substr(a);
}

// Object header address of the object at `path` ("" is the root group).
uint64_t lookup(Reader& r, const std::string& path) {
  uint64_t at = r.root();
  size_t pos = 0;
  const std::string p = strip(path);
  while (pos < p.size()) {
    size_t next = p.find('/', pos);
    if (next == std::string::npos) next = p.size();
    const std::string part = p.substr(pos, next - pos);
    pos = next + 1;
    if (part.empty()) continue;
    const Object g = r.object(at);
    bool found = false;
    for (const auto& [nm, a] : r.links(g)) {
      if (nm == part) {
        at = a;
        found = true;
        break;
      }
    }
    if (!found) throw std::runtime_error("dataset not found: /" + p);
  }
  return at;
}

struct Opened {
  Object obj;
  Dtype type;
  Space space;
};

Opened open_dataset(Reader& r, const std::string& name, DatasetInfo* info) {
  Opened d;
  d.obj = r.object(lookup(r, name));
  if (!is_dataset(d.obj)) throw std::runtime_error("not a dataset: /" + strip(name));
  d.type = r.dtype(*d.obj.find(0x03));
  d.space = r.space(*d.obj.find(0x01));
  if (d.type.cls != 0 && d.type.cls != 1)
    throw std::runtime_error("dataset /" + strip(name) + " has datatype class " + std::to_string(d.type.cls) +
                             " (only integer and floating-point data are read)");
  // Sizes come from the file: check them before anything is allocated.
  // Contiguous data must lie inside the file; compressed chunks may expand,
  // but not past 64 times the file's size.
  {
    const uint64_t fsize = r.file().size();
    long double bytes = d.type.size;
    for (uint64_t v : d.space.dims) bytes *= (long double)v;
    const Message* lm = d.obj.find(0x08);
    if (!lm) throw std::runtime_error("dataset /" + strip(name) + " has no layout message");
    const Layout l = r.layout(*lm);
    if (l.cls == 1 && l.addr != kUndef && (long double)r.abs(l.addr) + bytes > (long double)fsize)
      throw std::runtime_error("dataset /" + strip(name) + " extends past the end of the file");
    if (bytes > 64.0L * (long double)fsize + 65536.0L)
      throw std::runtime_error("dataset /" + strip(name) + " is implausibly large for its file");
  }
  if (info) {
    info->name = strip(name);
    info->type_class = d.type.cls;
    info->type_size = d.type.size;
    info->little_endian = d.type.le;
    info->is_signed = d.type.sgn;
    info->dims = d.space.dims;
  }
  return d;
}

// Bytes of one global heap object (variable-length data).
std::string global_heap_object(Reader& r, uint64_t coll, uint32_t index) {
  File& f = r.file();
  const int sl = r.sl();
  const std::vector<uint8_t> h = f.read_vec(r.abs(coll), size_t(8 + sl));
  if (std::memcmp(h.data(), "GCOL", 4) != 0) fail("bad global heap collection");
  Cur hc(h);
  hc.skip(8);
  const uint64_t size = hc.u(sl);
  if (size > (uint64_t(1) << 31)) fail("global heap collection too large");
  const std::vector<uint8_t> all = f.read_vec(r.abs(coll), size_t(size));
  Cur c(all);
  c.skip(size_t(8 + sl));
  while (c.left() >= size_t(8 + sl)) {
    const uint32_t idx = uint32_t(c.u(2));
    c.skip(6);
    const uint64_t n = c.u(sl);
    if (idx == 0) break;  // free space runs to the end of the collection
    c.need(size_t(n));
    if (idx == index) return std::string(reinterpret_cast<const char*>(c.at()), size_t(n));
    c.skip(std::min(c.left(), size_t((n + 7) & ~uint64_t(7))));
  }
  fail("global heap object not found");
}

std::string render_attr(Reader& r, const Message& m, std::string* name) {
  Cur c(m.data);
  const int ver = c.u8();
  const int flags = c.u8();
  const size_t nlen = size_t(c.u(2)), tlen = size_t(c.u(2)), slen = size_t(c.u(2));
  if (ver == 3) c.u8();
  if (ver < 1 || ver > 3) fail("attribute message version not supported");
  auto pad = [&](size_t n) { return ver == 1 ? (n + 7) & ~size_t(7) : n; };
  c.need(nlen);
  const char* np = reinterpret_cast<const char*>(c.at());
  *name = std::string(np, strnlen(np, nlen));
  c.skip(pad(nlen));
  if (flags & 0x03) return "<shared type>";
  c.need(tlen);
  const Message tm{0x03, 0, std::vector<uint8_t>(c.at(), c.at() + tlen)};
  c.skip(pad(tlen));
  c.need(slen);
  const Message sm{0x01, 0, std::vector<uint8_t>(c.at(), c.at() + slen)};
  c.skip(pad(slen));
  const int cls = tm.data.empty() ? -1 : (tm.data[0] & 0x0f);
  const Space s = r.space(sm);
  const uint64_t count = s.count();
  if (cls == 9 && tm.data.size() >= 4 && (tm.data[1] & 0x0f) == 1) {  // variable-length string
    std::string out;
    for (uint64_t i = 0; i < count; ++i) {
      const uint32_t len = uint32_t(c.u(4));
      const uint64_t coll = c.u(r.so());
      const uint32_t idx = uint32_t(c.u(4));
      std::string v = len ? global_heap_object(r, coll, idx) : std::string();
      if (i) out += ",";
      out += v.substr(0, std::min<size_t>(v.size(), len));
    }
    return out;
  }
  const Dtype t = r.dtype(tm);
  if (t.cls == 3) {
    c.need(size_t(count) * size_t(t.size));
    std::string v(reinterpret_cast<const char*>(c.at()), size_t(count) * size_t(t.size));
    v = v.substr(0, strnlen(v.c_str(), v.size()));
    if (t.str_pad == 2) v.erase(v.find_last_not_of(' ') + 1);
    return v;
  }
  if (t.cls != 0 && t.cls != 1) return "<type class " + std::to_string(t.cls) + ">";
  std::string out;
  for (uint64_t i = 0; i < count && i < 64; ++i) {
    c.need(size_t(t.size));
    char b[64];
    std::snprintf(b, sizeof b, t.cls == 1 ? "%.9g" : "%.0f", as_double(c.at(), t));
    c.skip(size_t(t.size));
    if (i) out += ",";
    out += b;
  }
  return out;
}

}  // namespace

bool is_hdf5(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  bool found = false;
  unsigned char sig[8];
  for (long at = 0; at <= (1L << 30) && !found; at = at ? at * 2 : 512) {
    if (fseeko(f, off_t(at), SEEK_SET) != 0 || std::fread(sig, 1, 8, f) != 8) break;
    found = std::memcmp(sig, kSig, 8) == 0;
  }
  std::fclose(f);
  return found;
}

std::vector<DatasetInfo> list_datasets(const std::string& path) {
  Reader r(path);
  std::vector<DatasetInfo> out;
  std::set<uint64_t> seen;
  std::function<void(uint64_t, const std::string&, int)> walk = [&](uint64_t at, const std::string& prefix, int depth) {
    if (depth > 64 || !seen.insert(at).second) return;
    const Object o = r.object(at);
    if (is_dataset(o)) {
      DatasetInfo d;
      d.name = prefix;
      const Dtype t = r.dtype(*o.find(0x03));
      d.type_class = t.cls;
      d.type_size = t.size;
      d.little_endian = t.le;
      d.is_signed = t.sgn;
      d.dims = r.space(*o.find(0x01)).dims;
      out.push_back(d);
    } else if (is_group(o)) {
      auto ls = r.links(o);
      std::sort(ls.begin(), ls.end());
      for (const auto& [nm, a] : ls) walk(a, prefix.empty() ? nm : prefix + "/" + nm, depth + 1);
    }
  };
  walk(r.root(), "", 0);
  return out;
}

std::vector<std::pair<std::string, std::string>> read_attributes(const std::string& path, const std::string& object) {
  Reader r(path);
  const Object o = r.object(lookup(r, object));
  std::vector<std::pair<std::string, std::string>> out;
  for (const auto& m : o.msgs) {
    if (m.type != 0x0C) continue;
    std::string name;
    std::string v = render_attr(r, m, &name);
    out.emplace_back(name, v);
  }
  return out;
}

std::vector<float> read_float(const std::string& path, const std::string& name, DatasetInfo* info) {
  Reader r(path);
  const Opened d = open_dataset(r, name, info);
  const uint64_t n = d.space.count();
  std::vector<float> out(static_cast<size_t>(n));
  if (d.type.cls == 1 && d.type.size == 4 && d.type.le) {
    r.read_raw(d.obj, d.type, d.space, reinterpret_cast<uint8_t*>(out.data()));
    return out;
  }
  std::vector<uint8_t> raw(size_t(n) * size_t(d.type.size));
  r.read_raw(d.obj, d.type, d.space, raw.data());
  for (uint64_t i = 0; i < n; ++i) out[size_t(i)] = float(as_double(raw.data() + i * uint64_t(d.type.size), d.type));
  return out;
}

std::vector<int32_t> read_int32(const std::string& path, const std::string& name, DatasetInfo* info) {
  Reader r(path);
  const Opened d = open_dataset(r, name, info);
  if (d.type.cls != 0) throw std::runtime_error("dataset /" + strip(name) + " is not an integer dataset");
  const uint64_t n = d.space.count();
  std::vector<uint8_t> raw(size_t(n) * size_t(d.type.size));
  r.read_raw(d.obj, d.type, d.space, raw.data());
  std::vector<int32_t> out(static_cast<size_t>(n));
  for (uint64_t i = 0; i < n; ++i) {
    const uint64_t v = load(raw.data() + i * uint64_t(d.type.size), d.type.size, d.type.le);
    const int64_t x = d.type.sgn ? as_int(v, d.type) : int64_t(v);
    if ((!d.type.sgn && v > uint64_t(INT32_MAX)) || x < INT32_MIN || x > INT32_MAX)
      throw std::runtime_error("dataset /" + strip(name) + " holds a value outside int32");
    out[size_t(i)] = int32_t(x);
  }
  return out;
}

// ---------------------------------------------------------------------------
// Writer.  Produces the structures libhdf5 writes with its default (earliest)
// format settings: superblock v0 with 8-byte offsets and lengths, group leaf
// K 4 / internal K 16, a symbol-table root group (one B-tree leaf, one local
// heap, one symbol table node of 2*4 entries), version 1 object headers,
// contiguous layout (message v3) and variable-length strings in one global
// heap collection.
namespace {

struct Out {
  std::vector<uint8_t> b;
  void u(uint64_t v, int n) {
    for (int i = 0; i < n; ++i) b.push_back(uint8_t(v >> (8 * i)));
  }
  void raw(const void* p, size_t n) {
    const uint8_t* q = static_cast<const uint8_t*>(p);
    b.insert(b.end(), q, q + n);
  }
  void zeros(size_t n) { b.insert(b.end(), n, 0); }
  void pad8() { zeros((8 - b.size() % 8) % 8); }
  size_t size() const { return b.size(); }
};

constexpr int kLeafK = 4, kInternalK = 16;
constexpr size_t kBtreeBytes = 24 + 2 * kInternalK * 8 + (2 * kInternalK + 1) * 8;
constexpr size_t kSnodBytes = 8 + 2 * kLeafK * 40;
constexpr size_t kGcolMin = 4096;

std::vector<uint8_t> type_i32() {
  Out o;
  o.u(0x10, 1);
  o.u(0x08, 1);  // little-endian, signed
  o.u(0, 2);
  o.u(4, 4);
  o.u(0, 2);
  o.u(32, 2);
  return o.b;
}

std::vector<uint8_t> type_f32() {
  Out o;
  o.u(0x11, 1);
  o.u(0x20, 1);  // little-endian, implied leading mantissa bit
  o.u(31, 1);    // sign bit position
  o.u(0, 1);
  o.u(4, 4);
  o.u(0, 2);
  o.u(32, 2);
  o.u(23, 1);
  o.u(8, 1);
  o.u(0, 1);
  o.u(23, 1);
  o.u(127, 4);
  return o.b;
}

std::vector<uint8_t> type_vlen_string() {
  Out o;
  o.u(0x19, 1);
  o.u(0x01, 1);  // string, null-terminated padding, ASCII
  o.u(0, 2);
  o.u(4 + 8 + 4, 4);
  o.u(0x10, 1);  // base type: unsigned 8-bit integer
  o.u(0, 3);
  o.u(1, 4);
  o.u(0, 2);
  o.u(8, 2);
  return o.b;
}

std::vector<uint8_t> space_v1(const std::vector<uint64_t>& dims) {
  Out o;
  o.u(1, 1);
  o.u(dims.size(), 1);
  o.u(0, 1);
  o.zeros(5);
  for (uint64_t d : dims) o.u(d, 8);
  return o.b;
}

void message_v1(Out& o, int type, const std::vector<uint8_t>& data, int flags = 0) {
  const size_t n = (data.size() + 7) & ~size_t(7);
  o.u(uint64_t(type), 2);
  o.u(n, 2);
  o.u(uint64_t(flags), 1);
  o.zeros(3);
  o.raw(data.data(), data.size());
  o.zeros(n - data.size());
}

std::vector<uint8_t> object_header_v1(const std::vector<std::pair<int, std::vector<uint8_t>>>& msgs) {
  Out body;
  for (const auto& [t, d] : msgs) message_v1(body, t, d, (t == 0x03 || t == 0x11) ? 1 : 0);  // constant
  Out o;
  o.u(1, 1);
  o.u(0, 1);
  o.u(msgs.size(), 2);
  o.u(1, 4);  // reference count
  o.u(body.size(), 4);
  o.zeros(4);
  o.raw(body.b.data(), body.size());
  return o.b;
}

std::vector<uint8_t> attribute_v1(const std::string& name, const std::vector<uint8_t>& type,
                                  const std::vector<uint8_t>& data) {
  const std::vector<uint8_t> sp = space_v1({});
  Out o;
  o.u(1, 1);
  o.u(0, 1);
  o.u(name.size() + 1, 2);
  o.u(type.size(), 2);
  o.u(sp.size(), 2);
  o.raw(name.c_str(), name.size() + 1);
  o.pad8();
  o.raw(type.data(), type.size());
  o.pad8();
  o.raw(sp.data(), sp.size());
  o.pad8();
  o.raw(data.data(), data.size());
  return o.b;
}

}  // namespace

namespace {

std::vector<uint8_t> type_f16() {
  Out o;
  o.u(0x11, 1);
  o.u(0x20, 1);  // little-endian, implied leading mantissa bit
  o.u(15, 1);    // sign bit position
  o.u(0, 1);
  o.u(2, 4);
  o.u(0, 2);
  o.u(16, 2);
  o.u(10, 1);
  o.u(5, 1);
  o.u(0, 1);
  o.u(10, 1);
  o.u(15, 4);
  return o.b;
}

size_t elem_bytes(int type_class) { return type_class == 2 ? 2 : 4; }

// Local heap data segment of a symbol-table group: "" at offset 0, the link
// names, then one free block (its "next" field 1 ends the free list).
struct HeapSeg {
  Out seg;
  std::vector<uint64_t> off;
  uint64_t free_off = 0;
};
HeapSeg heap_seg(const std::vector<std::string>& names) {
  HeapSeg h;
  h.seg.zeros(8);
  for (const auto& nm : names) {
    h.off.push_back(h.seg.size());
    h.seg.raw(nm.c_str(), nm.size() + 1);
    h.seg.pad8();
  }
  h.free_off = h.seg.size();
  h.seg.u(1, 8);
  h.seg.u(64, 8);
  h.seg.zeros(48);
  return h;
}

size_t group_image_bytes(const std::vector<std::string>& names) {
  return kBtreeBytes + 32 + heap_seg(names).seg.size() + kSnodBytes;
}

// [B-tree leaf][heap header][heap data][symbol node] of one group at address
// `at`; entries are (name, object header address), sorted by name.
void group_image(Out& m, uint64_t at, const std::vector<std::pair<std::string, uint64_t>>& entries, uint64_t* a_bt,
                 uint64_t* a_heap) {
  std::vector<std::string> names;
  for (const auto& e : entries) names.push_back(e.first);
  const HeapSeg h = heap_seg(names);
  *a_bt = at;
  *a_heap = at + kBtreeBytes;
  const uint64_t a_seg = *a_heap + 32, a_snod = a_seg + h.seg.size();
  const size_t bt0 = m.size();
  m.raw("TREE", 4);
  m.u(0, 1);
  m.u(0, 1);
  m.u(1, 2);
  m.u(kUndef, 8);
  m.u(kUndef, 8);
  m.u(0, 8);
  m.u(a_snod, 8);
  m.u(entries.empty() ? 0 : h.off.back(), 8);
  m.zeros(kBtreeBytes - (m.size() - bt0));
  m.raw("HEAP", 4);
  m.u(0, 1);
  m.zeros(3);
  m.u(h.seg.size(), 8);
  m.u(h.free_off, 8);
  m.u(a_seg, 8);
  m.raw(h.seg.b.data(), h.seg.size());
  const size_t sn0 = m.size();
  m.raw("SNOD", 4);
  m.u(1, 1);
  m.u(0, 1);
  m.u(entries.size(), 2);
  for (size_t i = 0; i < entries.size(); ++i) {
    m.u(h.off[i], 8);
    m.u(entries[i].second, 8);
    m.u(0, 4);
    m.u(0, 4);
    m.zeros(16);
  }
  m.zeros(kSnodBytes - (m.size() - sn0));
}

}  // namespace

void write_file(const std::string& path, const std::vector<WriteDataset>& ds_in, const std::vector<WriteAttr>& attrs) {
  std::vector<WriteDataset> ds(ds_in);
  std::sort(ds.begin(), ds.end(), [](const WriteDataset& a, const WriteDataset& b) { return a.name < b.name; });
  // one level of groups: "group/name"
  std::vector<std::string> groups;
  std::vector<std::string> leaf(ds.size()), grp(ds.size());
  for (size_t i = 0; i < ds.size(); ++i) {
    const std::string& nm = ds[i].name;
    const size_t s = nm.find('/');
    if (nm.empty() || s == 0 || s + 1 == nm.size() || (s != std::string::npos && nm.find('/', s + 1) != std::string::npos))
      fail("bad dataset name '" + nm + "' (one optional group level)");
    if (i && nm == ds[i - 1].name) fail("duplicate dataset name " + nm);
    if (ds[i].type_class < 0 || ds[i].type_class > 2) fail("datasets are written as int32, float32 or float16");
    grp[i] = s == std::string::npos ? "" : nm.substr(0, s);
    leaf[i] = s == std::string::npos ? nm : nm.substr(s + 1);
    if (!grp[i].empty() && (groups.empty() || groups.back() != grp[i])) groups.push_back(grp[i]);
  }
  std::sort(groups.begin(), groups.end());
  groups.erase(std::unique(groups.begin(), groups.end()), groups.end());
  for (const auto& g : groups)
    for (size_t i = 0; i < ds.size(); ++i)
      if (grp[i].empty() && leaf[i] == g) fail("name " + g + " is both a dataset and a group");
  // root entries and each group's entries, sorted by name (libhdf5 binary-searches symbol nodes)
  std::vector<std::string> root_names;
  for (size_t i = 0; i < ds.size(); ++i)
    if (grp[i].empty()) root_names.push_back(leaf[i]);
  for (const auto& g : groups) root_names.push_back(g);
  std::sort(root_names.begin(), root_names.end());
  if (root_names.size() > size_t(2 * kLeafK)) fail("at most 8 entries per group are written");
  std::vector<std::vector<size_t>> members(groups.size());
  for (size_t i = 0; i < ds.size(); ++i)
    if (!grp[i].empty())
      members[size_t(std::lower_bound(groups.begin(), groups.end(), grp[i]) - groups.begin())].push_back(i);
  for (const auto& mem : members)
    if (mem.size() > size_t(2 * kLeafK)) fail("at most 8 entries per group are written");

  // Global heap objects for the string attributes.
  std::vector<uint32_t> gidx(attrs.size(), 0);
  Out gobj;
  uint32_t nobj = 0;
  for (size_t i = 0; i < attrs.size(); ++i) {
    if (!attrs[i].is_string || attrs[i].s.empty()) continue;
    gidx[i] = ++nobj;
    gobj.u(nobj, 2);
    gobj.u(0, 2);
    gobj.zeros(4);
    gobj.u(attrs[i].s.size(), 8);
    gobj.raw(attrs[i].s.data(), attrs[i].s.size());
    gobj.pad8();
  }
  const uint64_t gsize = nobj ? std::max<uint64_t>(kGcolMin, (16 + gobj.size() + 16 + 4095) & ~uint64_t(4095)) : 0;

  auto symtab_msg = [](uint64_t bt, uint64_t heap) {
    Out st;
    st.u(bt, 8);
    st.u(heap, 8);
    return st.b;
  };
  auto root_header = [&](uint64_t bt, uint64_t heap, uint64_t gcol) {
    std::vector<std::pair<int, std::vector<uint8_t>>> msgs;
    msgs.emplace_back(0x11, symtab_msg(bt, heap));
    for (size_t i = 0; i < attrs.size(); ++i) {
      Out v;
      if (attrs[i].is_string) {
        v.u(attrs[i].s.size(), 4);
        v.u(gidx[i] ? gcol : 0, 8);
        v.u(gidx[i], 4);
        msgs.emplace_back(0x0C, attribute_v1(attrs[i].name, type_vlen_string(), v.b));
      } else {
        v.raw(&attrs[i].f, 4);
        msgs.emplace_back(0x0C, attribute_v1(attrs[i].name, type_f32(), v.b));
      }
    }
    return object_header_v1(msgs);
  };
  auto dataset_header = [&](const WriteDataset& d, uint64_t addr, uint64_t bytes) {
    Out lay;
    lay.u(3, 1);
    lay.u(1, 1);
    lay.u(addr, 8);
    lay.u(bytes, 8);
    const std::vector<uint8_t> t = d.type_class == 0 ? type_i32() : d.type_class == 1 ? type_f32() : type_f16();
    return object_header_v1({{0x01, space_v1(d.dims)}, {0x03, t}, {0x08, lay.b}});
  };
  std::vector<uint64_t> bytes;
  for (const auto& d : ds) {
    uint64_t n = elem_bytes(d.type_class);
    for (uint64_t v : d.dims) n *= v;
    bytes.push_back(n);
  }
  // Addresses: superblock, root header, root group image, each group's header
  // and image, global heap, dataset headers, raw data.
  const uint64_t a_root = 96;
  const uint64_t a_rimg = a_root + root_header(0, 0, 0).size();
  uint64_t at = a_rimg + group_image_bytes(root_names);
  std::vector<uint64_t> a_ghdr(groups.size()), a_gimg(groups.size());
  const size_t ghdr_bytes = object_header_v1({{0x11, symtab_msg(0, 0)}}).size();
  for (size_t g = 0; g < groups.size(); ++g) {
    std::vector<std::string> names;
    for (size_t i : members[g]) names.push_back(leaf[i]);
    a_ghdr[g] = at;
    a_gimg[g] = at + ghdr_bytes;
    at = a_gimg[g] + group_image_bytes(names);
  }
  const uint64_t a_gcol = at;
  at += gsize;
  std::vector<uint64_t> a_hdr(ds.size()), a_data(ds.size());
  for (size_t i = 0; i < ds.size(); ++i) {
    a_hdr[i] = at;
    at += dataset_header(ds[i], 0, 0).size();
  }
  const uint64_t meta_end = at;
  for (size_t i = 0; i < ds.size(); ++i) {
    at = (at + 7) & ~uint64_t(7);
    a_data[i] = at;
    at += bytes[i];
  }
  const uint64_t eof = at;

  // root entries with their object header addresses
  std::vector<std::pair<std::string, uint64_t>> root_entries;
  for (const auto& nm : root_names) {
    uint64_t a = 0;
    for (size_t i = 0; i < ds.size(); ++i)
      if (grp[i].empty() && leaf[i] == nm) a = a_hdr[i];
    for (size_t g = 0; g < groups.size(); ++g)
      if (groups[g] == nm) a = a_ghdr[g];
    root_entries.emplace_back(nm, a);
  }
  uint64_t r_bt = 0, r_heap = 0;
  {
    Out probe;
    group_image(probe, a_rimg, root_entries, &r_bt, &r_heap);
  }

  Out m;
  m.raw(kSig, 8);
  m.u(0, 1);  // superblock version
  m.u(0, 1);  // free-space storage version
  m.u(0, 1);  // root group symbol table entry version
  m.u(0, 1);
  m.u(0, 1);  // shared header message format version
  m.u(8, 1);
  m.u(8, 1);
  m.u(0, 1);
  m.u(kLeafK, 2);
  m.u(kInternalK, 2);
  m.u(0, 4);
  m.u(0, 8);       // base address
  m.u(kUndef, 8);  // free-space info
  m.u(eof, 8);
  m.u(kUndef, 8);  // driver info
  m.u(0, 8);       // root link name offset
  m.u(a_root, 8);
  m.u(1, 4);  // cache type: symbol table
  m.u(0, 4);
  m.u(r_bt, 8);
  m.u(r_heap, 8);
  const std::vector<uint8_t> rh = root_header(r_bt, r_heap, a_gcol);
  m.raw(rh.data(), rh.size());
  group_image(m, a_rimg, root_entries, &r_bt, &r_heap);
  for (size_t g = 0; g < groups.size(); ++g) {
    std::vector<std::pair<std::string, uint64_t>> entries;
    for (size_t i : members[g]) entries.emplace_back(leaf[i], a_hdr[i]);
    uint64_t bt = 0, heap = 0;
    {
      Out probe;
      group_image(probe, a_gimg[g], entries, &bt, &heap);
    }
    const std::vector<uint8_t> gh = object_header_v1({{0x11, symtab_msg(bt, heap)}});
    m.raw(gh.data(), gh.size());
    group_image(m, a_gimg[g], entries, &bt, &heap);
  }
  if (nobj) {
    const size_t g0 = m.size();
    m.raw("GCOL", 4);
    m.u(1, 1);
    m.zeros(3);
    m.u(gsize, 8);
    m.raw(gobj.b.data(), gobj.size());
    const uint64_t free_bytes = gsize - (m.size() - g0);
    m.u(0, 2);  // object 0: the free space
    m.u(0, 2);
    m.zeros(4);
    m.u(free_bytes, 8);
    m.zeros(size_t(free_bytes - 16));
  }
  for (size_t i = 0; i < ds.size(); ++i) {
    const std::vector<uint8_t> h = dataset_header(ds[i], a_data[i], bytes[i]);
    m.raw(h.data(), h.size());
  }
  if (m.size() != meta_end) fail("internal layout error while writing " + path);
  File f(path, "wb");
  f.write(m.b.data(), m.size());
  uint64_t pos = m.size();
  static const uint8_t zero[8] = {0};
  for (size_t i = 0; i < ds.size(); ++i) {
    f.write(zero, size_t(a_data[i] - pos));
    f.write(ds[i].data, size_t(bytes[i]));
    pos = a_data[i] + bytes[i];
  }
  f.close();
}

}  // namespace h5
}  // namespace knngio
