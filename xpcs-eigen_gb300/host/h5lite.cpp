#include "h5lite.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <set>
#include <stdexcept>

namespace h5lite {

uint64_t Data::count() const {
  uint64_t n = 1;
  for (uint64_t d : dims) n *= d;
  return n;
}

namespace {

const unsigned char SIG[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
constexpr uint64_t UNDEF = ~0ull;  // the undefined address (all bits set)
constexpr int MAX_DEPTH = 64;

[[noreturn]] void fail(const std::string &m) { throw std::runtime_error("HDF5: " + m); }

std::vector<unsigned char> slurp(const std::string &path) {
  FILE *f = fopen(path.c_str(), "rb");
  if (!f) fail("cannot open " + path);
  std::vector<unsigned char> b;
  unsigned char buf[1 << 16];
  size_t n;
  while ((n = fread(buf, 1, sizeof buf, f)) > 0) b.insert(b.end(), buf, buf + n);
  fclose(f);
  return b;
}

void spill(const std::string &path, const std::vector<unsigned char> &b) {
  const std::string tmp = path + ".tmp";
  FILE *f = fopen(tmp.c_str(), "wb");
  if (!f) fail("cannot write " + tmp);
  const bool ok = b.empty() || fwrite(b.data(), 1, b.size(), f) == b.size();
  if (fclose(f) != 0 || !ok || rename(tmp.c_str(), path.c_str()) != 0) fail("cannot write " + path);
}

uint64_t round8(uint64_t x) { return (x + 7) & ~(uint64_t)7; }

// The file image with its superblock facts.  File addresses are relative to
// the base address (the superblock's position when a user block precedes it).
struct Image {
  std::vector<unsigned char> b;
  uint64_t sb = 0, base = 0;
  int version = 0;
  int so = 8, sl = 8;          // sizes of offsets and lengths
  int leafK = 4, nodeK = 16;   // symbol-table node and group B-tree node ranks
  uint64_t root_entry = 0;     // position of the root symbol-table entry (v0/v1)
  uint64_t root = UNDEF;       // root group object header address
  uint64_t eof_field = 0;      // position of the end-of-file address

  void need(uint64_t pos, uint64_t n) const {
    if (pos > b.size() || n > b.size() - pos) fail("a structure runs past the end of the file");
  }
  uint64_t get(uint64_t pos, int n) const {
    need(pos, (uint64_t)n);
    uint64_t v = 0;
    for (int i = n - 1; i >= 0; i--) v = (v << 8) | b[pos + i];
    return v;
  }
  uint64_t addr(uint64_t pos) const { return get(pos, so); }  // UNDEF stays all ones (so = 8)
  uint64_t at(uint64_t rel) const {
    if (rel == UNDEF) fail("undefined address");
    if (rel > b.size() - base) fail("address past the end of the file");
    return base + rel;
  }
  bool sig(uint64_t pos, const char *s) const {
    need(pos, 4);
    return memcmp(&b[pos], s, 4) == 0;
  }
  void put(uint64_t pos, uint64_t v, int n) {
    need(pos, (uint64_t)n);
    for (int i = 0; i < n; i++) {
      b[pos + i] = (unsigned char)(v & 0xff);
      v >>= 8;
    }
  }
  // appends bytes at the next 8-byte boundary; returns their file address
  uint64_t append(const std::vector<unsigned char> &x) {
    while ((b.size() - base) % 8) b.push_back(0);
    const uint64_t rel = b.size() - base;
    b.insert(b.end(), x.begin(), x.end());
    return rel;
  }
};

void le(std::vector<unsigned char> &o, uint64_t v, int n) {
  for (int i = 0; i < n; i++) {
    o.push_back((unsigned char)(v & 0xff));
    v >>= 8;
  }
}

void parse_superblock(Image &im) {
  bool found = false;
  for (uint64_t off = 0; off + 8 <= im.b.size(); off = off ? 2 * off : 512) {
    if (memcmp(&im.b[off], SIG, 8) == 0) {
      im.sb = off;
      found = true;
      break;
    }
  }
  if (!found) fail("no superblock");
  const uint64_t s = im.sb;
  im.version = (int)im.get(s + 8, 1);
  if (im.version == 0 || im.version == 1) {
    im.so = (int)im.get(s + 13, 1);
    im.sl = (int)im.get(s + 14, 1);
    if (im.so != 8 || im.sl != 8) fail("sizes of offsets and lengths other than 8 bytes");
    im.leafK = (int)im.get(s + 16, 2);
    im.nodeK = (int)im.get(s + 18, 2);
    if (im.leafK <= 0 || im.nodeK <= 0) fail("bad B-tree ranks");
    const uint64_t p = s + 24 + (im.version == 1 ? 4 : 0);
    im.base = im.get(p, 8);
    im.eof_field = p + 16;
    im.root_entry = p + 32;
    im.root = im.get(im.root_entry + 8, 8);
  } else if (im.version == 2 || im.version == 3) {
    im.so = (int)im.get(s + 9, 1);
    im.sl = (int)im.get(s + 10, 1);
    if (im.so != 8 || im.sl != 8) fail("sizes of offsets and lengths other than 8 bytes");
    im.base = im.get(s + 12, 8);
    im.eof_field = s + 12 + 16;
    im.root = im.get(s + 12 + 24, 8);
  } else {
    fail("superblock version " + std::to_string(im.version));
  }
  if (im.base > im.b.size()) fail("base address past the end of the file");
}

// ------------------------------------------------------------- object headers

struct Msg {
  int type;
  uint64_t pos;   // position of the message data
  uint64_t size;  // bytes of message data
  int flags;
};

enum : int {
  M_NIL = 0x00, M_SPACE = 0x01, M_LINFO = 0x02, M_TYPE = 0x03, M_LINK = 0x06, M_LAYOUT = 0x08,
  M_FILTER = 0x0b, M_CONT = 0x10, M_STAB = 0x11
};

std::vector<Msg> messages(const Image &im, uint64_t rel) {
  std::vector<Msg> out;
  const uint64_t p = im.at(rel);
  std::vector<std::pair<uint64_t, uint64_t>> chunks;
  if (im.get(p, 1) == 1) {  // version 1: 16-byte prefix, messages aligned to 8 bytes
    const uint64_t nmsg = im.get(p + 2, 2);
    chunks.push_back({p + 16, im.get(p + 8, 4)});
    for (size_t c = 0; c < chunks.size() && out.size() < nmsg; c++) {
      if (c > 4096) fail("too many object header chunks");
      uint64_t q = chunks[c].first;
      const uint64_t end = q + chunks[c].second;
      im.need(q, chunks[c].second);
      while (q + 8 <= end && out.size() < nmsg) {
        const int type = (int)im.get(q, 2);
        const uint64_t sz = im.get(q + 2, 2);
        const int fl = (int)im.get(q + 4, 1);
        if (q + 8 + sz > end) fail("a header message runs past its chunk");
        if (type == M_CONT) chunks.push_back({im.at(im.addr(q + 8)), im.get(q + 16, 8)});
        out.push_back({type, q + 8, sz, fl});
        q += 8 + sz;
      }
    }
  } else if (im.sig(p, "OHDR")) {  // version 2
    const int fl = (int)im.get(p + 5, 1);
    uint64_t q = p + 6 + ((fl & 0x20) ? 16 : 0) + ((fl & 0x10) ? 4 : 0);
    const int w = 1 << (fl & 3);
    const uint64_t size0 = im.get(q, w);
    chunks.push_back({q + w, size0});
    const int hdr = 4 + ((fl & 0x04) ? 2 : 0);
    for (size_t c = 0; c < chunks.size(); c++) {
      if (c > 4096) fail("too many object header chunks");
      uint64_t r = chunks[c].first;
      const uint64_t end = r + chunks[c].second;
      im.need(r, chunks[c].second);
      while (r + hdr <= end) {
        const int type = (int)im.get(r, 1);
        const uint64_t sz = im.get(r + 1, 2);
        const int mf = (int)im.get(r + 3, 1);
        r += hdr;
        if (r + sz > end) fail("a header message runs past its chunk");
        if (type == M_CONT) {
          const uint64_t a = im.at(im.addr(r)), len = im.get(r + 8, 8);
          if (len < 8 || !im.sig(a, "OCHK")) fail("bad continuation block");
          chunks.push_back({a + 4, len - 8});  // signature and checksum around the messages
        }
        out.push_back({type, r, sz, mf});
        r += sz;
      }
    }
  } else {
    fail("unknown object header");
  }
  return out;
}

const Msg *find(const std::vector<Msg> &ms, int type) {
  for (const Msg &m : ms)
    if (m.type == type) return &m;
  return nullptr;
}

// ------------------------------------------------------------------ datasets

struct Type {
  Kind kind = Kind::Int;
  uint32_t size = 0;   // element size in the file
  bool vlstr = false;  // variable-length string: (length, heap address, index) per element
  std::string why;     // non-empty: not handled
};

Type parse_type(const Image &im, const Msg &m) {
  Type t;
  if (m.flags & 0x02) {
    t.why = "shared datatype";
    return t;
  }
  const uint64_t d = m.pos;
  const int cls = (int)(im.get(d, 1) & 0x0f);
  const int bits = (int)im.get(d + 1, 1);
  t.size = (uint32_t)im.get(d + 4, 4);
  switch (cls) {
    case 0:
      t.kind = (bits & 0x08) ? Kind::Int : Kind::UInt;
      if (bits & 1) t.why = "big-endian integers";
      if (t.size != 1 && t.size != 2 && t.size != 4 && t.size != 8) t.why = "integer size";
      break;
    case 1:
      t.kind = Kind::Float;
      if ((bits & 1) || (bits & 0x40)) t.why = "float byte order";
      if (t.size != 4 && t.size != 8) t.why = "float size";
      break;
    case 3:
      t.kind = Kind::String;
      break;
    case 9:
      if ((bits & 0x0f) == 1) {
        t.kind = Kind::String;
        t.vlstr = true;
        t.size = 4 + 8 + 4;
      } else {
        t.why = "variable-length sequence";
      }
      break;
    default:
      t.why = "datatype class " + std::to_string(cls);
  }
  return t;
}

bool parse_space(const Image &im, const Msg &m, std::vector<uint64_t> &dims, std::string &why) {
  const uint64_t d = m.pos;
  const int ver = (int)im.get(d, 1), rank = (int)im.get(d + 1, 1);
  uint64_t q;
  if (ver == 1) {
    q = d + 8;
  } else if (ver == 2) {
    if (im.get(d + 3, 1) == 2) {  // null dataspace: no elements
      dims.assign(1, 0);
      return true;
    }
    q = d + 4;
  } else {
    why = "dataspace version " + std::to_string(ver);
    return false;
  }
  dims.clear();
  for (int i = 0; i < rank; i++) dims.push_back(im.get(q + 8 * (uint64_t)i, 8));
  return true;
}

// Where a dataset's elements are: compact (in the layout message) or
// contiguous (an address, possibly undefined before any write).
struct Layout {
  bool compact = false;
  uint64_t pos = 0;        // compact: data position; contiguous: position of the address field
  uint64_t size = 0;       // compact: data bytes
  uint64_t addr = UNDEF;   // contiguous
  std::string why;
};

Layout parse_layout(const Image &im, const Msg &m) {
  Layout L;
  const uint64_t d = m.pos;
  const int ver = (int)im.get(d, 1);
  if (ver == 3 || ver == 4) {
    const int cls = (int)im.get(d + 1, 1);
    if (cls == 0) {
      L.compact = true;
      L.size = im.get(d + 2, 2);
      L.pos = d + 4;
    } else if (cls == 1) {
      L.pos = d + 2;
      L.addr = im.addr(d + 2);
    } else {
      L.why = cls == 2 ? "chunked storage" : "storage class " + std::to_string(cls);
    }
  } else if (ver == 1 || ver == 2) {
    const int rank = (int)im.get(d + 1, 1), cls = (int)im.get(d + 2, 1);
    uint64_t q = d + 8;
    if (cls == 1) {
      L.pos = q;
      L.addr = im.addr(q);
    } else if (cls == 0) {
      q += 4 * (uint64_t)rank;
      L.compact = true;
      L.size = im.get(q, 4);
      L.pos = q + 4;
    } else {
      L.why = "chunked storage";
    }
  } else {
    L.why = "layout version " + std::to_string(ver);
  }
  return L;
}

// A variable-length string: the element (length, global heap collection
// address, object index) resolved in its collection.
std::string vl_string(const Image &im, const unsigned char *e) {
  auto rd = [e](int off, int n) {
    uint64_t v = 0;
    for (int i = n - 1; i >= 0; i--) v = (v << 8) | e[off + i];
    return v;
  };
  const uint64_t len = rd(0, 4), coll = rd(4, 8), idx = rd(12, 4);
  if (len == 0 || coll == UNDEF) return std::string();
  const uint64_t g = im.at(coll);
  if (!im.sig(g, "GCOL")) fail("bad global heap collection");
  const uint64_t end = g + im.get(g + 8, 8);
  uint64_t q = g + 16;
  for (int guard = 0; q + 16 <= end && guard < (1 << 20); guard++) {
    const uint64_t h = im.get(q, 2), osz = im.get(q + 8, 8);
    if (h == 0) break;  // the collection's free space
    if (h == idx) {
      if (len > osz) fail("variable-length string longer than its heap object");
      im.need(q + 16, len);
      return std::string((const char *)&im.b[q + 16], (size_t)len);
    }
    q += 16 + round8(osz);
  }
  fail("variable-length string not found in its heap collection");
}

// The dataset whose header messages are ms, or its reason for being skipped.
bool read_dataset(const Image &im, const std::vector<Msg> &ms, Data &out, std::string &why) {
  const Msg *mt = find(ms, M_TYPE), *msp = find(ms, M_SPACE), *ml = find(ms, M_LAYOUT);
  if (!mt || !msp || !ml) {
    why = "dataset without a datatype, dataspace or layout";
    return false;
  }
  const Type t = parse_type(im, *mt);
  if (!t.why.empty()) {
    why = t.why;
    return false;
  }
  std::vector<uint64_t> dims;
  if (!parse_space(im, *msp, dims, why)) return false;
  const Layout L = parse_layout(im, *ml);
  if (!L.why.empty()) {
    why = L.why;
    return false;
  }
  if (const Msg *mf = find(ms, M_FILTER)) {
    if (im.get(mf->pos + 1, 1) > 0) {
      why = "filtered storage";
      return false;
    }
  }
  // the size, checked against the file before anything is allocated
  constexpr uint64_t MAX_UNWRITTEN = 1ull << 30;  // bytes of zeros for a never-written dataset
  uint64_t n = 1;
  for (uint64_t x : dims) {
    if (x && n > (~0ull >> 1) / x) fail("dataspace too large");
    n *= x;
  }
  if (t.size && n > (~0ull >> 1) / t.size) fail("dataspace too large");
  const uint64_t nbytes = n * t.size;
  if (L.compact) {
    if (L.size < nbytes) fail("compact data shorter than its dataspace");
    im.need(L.pos, nbytes);
  } else if (L.addr != UNDEF) {
    im.need(im.at(L.addr), nbytes);
  } else if (nbytes > MAX_UNWRITTEN) {
    why = "storage never allocated";
    return false;
  }
  std::vector<unsigned char> raw(nbytes, 0);
  if (nbytes) {
    if (L.compact)
      memcpy(raw.data(), &im.b[L.pos], nbytes);
    else if (L.addr != UNDEF)  // an undefined address: never written, zeros
      memcpy(raw.data(), &im.b[im.at(L.addr)], nbytes);
  }
  out.dims = dims;
  out.kind = t.kind;
  if (t.vlstr) {  // to fixed-length strings as wide as the longest
    std::vector<std::string> s(n);
    size_t w = 1;
    for (uint64_t i = 0; i < n; i++) {
      s[i] = vl_string(im, &raw[16 * i]);
      w = std::max(w, s[i].size());
    }
    if (n * w > (1ull << 31)) fail("strings too large");
    out.size = (uint32_t)w;
    out.bytes.assign(n * w, 0);
    for (uint64_t i = 0; i < n; i++) memcpy(&out.bytes[i * w], s[i].data(), s[i].size());
  } else {
    out.size = t.size;
    out.bytes.swap(raw);
  }
  return true;
}

// ------------------------------------------------------------------- groups

struct Entry {
  std::string name;
  uint64_t ohdr = UNDEF;
  uint64_t pos = 0;  // position of the symbol-table entry (0: a link message)
  std::vector<unsigned char> raw;  // the 40-byte symbol-table entry
};

struct Heap {
  uint64_t hdr = 0, seg = 0, size = 0;  // header position, data segment position and size
};

Heap open_heap(const Image &im, uint64_t rel) {
  Heap h;
  h.hdr = im.at(rel);
  if (!im.sig(h.hdr, "HEAP")) fail("bad local heap");
  h.size = im.get(h.hdr + 8, 8);
  h.seg = im.at(im.addr(h.hdr + 24));
  im.need(h.seg, h.size);
  return h;
}

std::string heap_name(const Image &im, const Heap &h, uint64_t off) {
  if (off >= h.size) fail("link name outside its local heap");
  const char *p = (const char *)&im.b[h.seg + off];
  const size_t n = strnlen(p, (size_t)(h.size - off));
  if (n == h.size - off) fail("unterminated link name");
  return std::string(p, n);
}

constexpr int ENTRY = 40;  // symbol-table entry: name offset, header address, cache type, reserved, scratch

void btree_entries(const Image &im, uint64_t rel, const Heap &h, std::vector<Entry> &out,
                   int depth) {
  if (depth > MAX_DEPTH) fail("B-tree too deep");
  const uint64_t n = im.at(rel);
  if (!im.sig(n, "TREE") || im.get(n + 4, 1) != 0) fail("bad group B-tree node");
  const int level = (int)im.get(n + 5, 1);
  const uint64_t used = im.get(n + 6, 2);
  const uint64_t q = n + 24;
  for (uint64_t i = 0; i < used; i++) {
    const uint64_t child = im.addr(q + 8 + 16 * i);
    if (level > 0) {
      btree_entries(im, child, h, out, depth + 1);
      continue;
    }
    const uint64_t s = im.at(child);
    if (!im.sig(s, "SNOD")) fail("bad symbol-table node");
    const uint64_t nsym = im.get(s + 6, 2);
    for (uint64_t k = 0; k < nsym; k++) {
      const uint64_t e = s + 8 + ENTRY * k;
      im.need(e, ENTRY);
      Entry en;
      en.name = heap_name(im, h, im.get(e, 8));
      en.ohdr = im.addr(e + 8);
      en.pos = e;
      en.raw.assign(im.b.begin() + e, im.b.begin() + e + ENTRY);
      out.push_back(std::move(en));
    }
  }
}

// Links of a group given its header messages; false with a reason when the
// group's links are not readable here.
bool group_links(const Image &im, const std::vector<Msg> &ms, std::vector<Entry> &out,
                 std::string &why) {
  if (const Msg *st = find(ms, M_STAB)) {
    const Heap h = open_heap(im, im.addr(st->pos + 8));
    btree_entries(im, im.addr(st->pos), h, out, 0);
    return true;
  }
  if (const Msg *li = find(ms, M_LINFO)) {
    const int fl = (int)im.get(li->pos + 1, 1);
    const uint64_t fh = im.addr(li->pos + 2 + ((fl & 1) ? 8 : 0));
    if (fh != UNDEF) {
      why = "links in a fractal heap";
      return false;
    }
  }
  for (const Msg &m : ms) {
    if (m.type != M_LINK) continue;
    const uint64_t d = m.pos;
    const int fl = (int)im.get(d + 1, 1);
    uint64_t q = d + 2;
    int ltype = 0;
    if (fl & 0x08) ltype = (int)im.get(q++, 1);
    if (fl & 0x04) q += 8;
    if (fl & 0x10) q += 1;
    const int w = 1 << (fl & 3);
    const uint64_t nlen = im.get(q, w);
    q += w;
    im.need(q, nlen);
    Entry en;
    en.name.assign((const char *)&im.b[q], (size_t)nlen);
    q += nlen;
    if (ltype != 0) continue;  // soft and external links are not followed
    en.ohdr = im.addr(q);
    out.push_back(std::move(en));
  }
  return true;
}

bool is_group(const std::vector<Msg> &ms) {
  return find(ms, M_STAB) || find(ms, M_LINFO) || find(ms, M_LINK);
}

void walk(const Image &im, uint64_t rel, const std::string &path, int depth,
          std::set<uint64_t> &seen, std::map<std::string, Data> &sets,
          std::map<std::string, std::string> &skipped) {
  if (depth > MAX_DEPTH || !seen.insert(rel).second) return;
  const std::vector<Msg> ms = messages(im, rel);
  std::vector<Entry> links;
  std::string why;
  if (!group_links(im, ms, links, why)) {
    skipped[path.empty() ? "/" : path] = why;
    return;
  }
  for (const Entry &e : links) {
    const std::string p = path + "/" + e.name;
    if (e.ohdr == UNDEF) continue;
    const std::vector<Msg> cm = messages(im, e.ohdr);
    if (find(cm, M_LAYOUT)) {
      Data d;
      std::string w;
      if (read_dataset(im, cm, d, w))
        sets[p] = std::move(d);
      else
        skipped[p] = w;
    } else if (is_group(cm)) {
      walk(im, e.ohdr, p, depth + 1, seen, sets, skipped);
    }
  }
}

// ------------------------------------------------------------------- writing

// A group of a version 0/1 file as the writer sees it: where its symbol-table
// message is and which entry (superblock or parent's node) caches its
// B-tree and heap addresses.
struct Group {
  uint64_t ohdr = UNDEF, stab = 0, btree = UNDEF, heap = UNDEF, entry = 0;
  std::vector<Entry> links;
};

Group open_group(const Image &im, uint64_t rel, uint64_t entry) {
  const std::vector<Msg> ms = messages(im, rel);
  const Msg *st = find(ms, M_STAB);
  if (!st) fail("a group without a symbol table cannot be written by this writer");
  Group g;
  g.ohdr = rel;
  g.stab = st->pos;
  g.btree = im.addr(st->pos);
  g.heap = im.addr(st->pos + 8);
  g.entry = entry;
  const Heap h = open_heap(im, g.heap);
  btree_entries(im, g.btree, h, g.links, 0);
  return g;
}

std::vector<unsigned char> v1_header(const std::vector<std::pair<int, std::vector<unsigned char>>> &msgs) {
  std::vector<unsigned char> body;
  for (const auto &m : msgs) {
    const uint64_t sz = round8(m.second.size());
    le(body, (uint64_t)m.first, 2);
    le(body, sz, 2);
    le(body, 0, 4);  // flags and reserved
    body.insert(body.end(), m.second.begin(), m.second.end());
    body.resize(body.size() + (sz - m.second.size()), 0);
  }
  std::vector<unsigned char> h;
  le(h, 1, 1);  // version
  le(h, 0, 1);
  le(h, msgs.size(), 2);
  le(h, 1, 4);  // reference count
  le(h, body.size(), 4);
  le(h, 0, 4);  // to the 8-byte boundary
  h.insert(h.end(), body.begin(), body.end());
  return h;
}

std::vector<unsigned char> heap_header(uint64_t size, uint64_t free_head, uint64_t seg) {
  std::vector<unsigned char> h = {'H', 'E', 'A', 'P', 0, 0, 0, 0};
  le(h, size, 8);
  le(h, free_head, 8);
  le(h, seg, 8);
  return h;
}

// A free block of 16 bytes closing a heap data segment (next free block: 1,
// meaning none).
void free_block(std::vector<unsigned char> &seg) {
  le(seg, 1, 8);
  le(seg, 16, 8);
}

uint64_t btree_node_bytes(const Image &im) { return 24 + (2 * (uint64_t)im.nodeK + 1) * 8 + 2 * (uint64_t)im.nodeK * 8; }
uint64_t snod_bytes(const Image &im) { return 8 + 2 * (uint64_t)im.leafK * ENTRY; }

// Adds the link name -> rel to group g: a new heap data segment (the old one
// plus the name), new symbol-table nodes and B-tree, and the addresses that
// point to them updated in place.
void insert_link(Image &im, const Group &g, const std::string &name, uint64_t rel) {
  if (name.empty() || name.find('/') != std::string::npos) fail("bad link name '" + name + "'");
  Heap h = open_heap(im, g.heap);
  std::vector<unsigned char> seg(im.b.begin() + h.seg, im.b.begin() + h.seg + h.size);
  const uint64_t name_off = seg.size();
  seg.insert(seg.end(), name.begin(), name.end());
  seg.resize(round8(seg.size() + 1), 0);
  const uint64_t free_off = seg.size();
  free_block(seg);
  const uint64_t seg_rel = im.append(seg);
  im.put(h.hdr + 8, seg.size(), 8);
  im.put(h.hdr + 16, free_off, 8);
  im.put(h.hdr + 24, seg_rel, 8);
  h = open_heap(im, g.heap);

  struct Item {
    std::string name;
    uint64_t off;
    std::vector<unsigned char> raw;
  };
  std::vector<Item> items;
  for (const Entry &e : g.links) {
    if (e.name == name) fail("link '" + name + "' exists");
    items.push_back({e.name, im.get(e.pos, 8), e.raw});
  }
  std::vector<unsigned char> raw;
  le(raw, name_off, 8);
  le(raw, rel, 8);
  le(raw, 0, 4);  // no cached scratch-pad
  le(raw, 0, 4);
  raw.resize(ENTRY, 0);
  items.push_back({name, name_off, raw});
  std::sort(items.begin(), items.end(),
            [](const Item &a, const Item &b) { return strcmp(a.name.c_str(), b.name.c_str()) < 0; });

  // symbol-table nodes of up to 2K entries
  const size_t cap = 2 * (size_t)im.leafK;
  std::vector<uint64_t> snods, last;  // node addresses and the heap offset of each node's last name
  for (size_t i = 0; i < items.size(); i += cap) {
    const size_t n = std::min(cap, items.size() - i);
    std::vector<unsigned char> s = {'S', 'N', 'O', 'D', 1, 0};
    le(s, n, 2);
    for (size_t k = 0; k < n; k++) s.insert(s.end(), items[i + k].raw.begin(), items[i + k].raw.end());
    s.resize(snod_bytes(im), 0);
    snods.push_back(im.append(s));
    last.push_back(items[i + n - 1].off);
  }
  // B-tree: level-0 nodes over the symbol-table nodes, and a level-1 node over
  // those when one node cannot hold them all
  const size_t fan = 2 * (size_t)im.nodeK;
  auto build = [&](int level, const std::vector<uint64_t> &kids, const std::vector<uint64_t> &keys,
                   std::vector<uint64_t> &nodes, std::vector<uint64_t> &node_last) {
    const size_t nn = (kids.size() + fan - 1) / fan;
    const uint64_t sz = btree_node_bytes(im);
    // the nodes' addresses first, for the sibling links
    while ((im.b.size() - im.base) % 8) im.b.push_back(0);
    const uint64_t first = im.b.size() - im.base;
    for (size_t j = 0; j < nn; j++) nodes.push_back(first + j * sz);
    for (size_t j = 0; j < nn; j++) {
      const size_t a = j * fan, n = std::min(fan, kids.size() - a);
      std::vector<unsigned char> t = {'T', 'R', 'E', 'E', 0, (unsigned char)level};
      le(t, n, 2);
      le(t, j > 0 ? nodes[j - 1] : UNDEF, 8);
      le(t, j + 1 < nn ? nodes[j + 1] : UNDEF, 8);
      le(t, a > 0 ? keys[a - 1] : 0, 8);  // key 0: the empty name at offset 0, or the previous node's last
      for (size_t k = 0; k < n; k++) {
        le(t, kids[a + k], 8);
        le(t, keys[a + k], 8);
      }
      t.resize(sz, 0);
      im.b.insert(im.b.end(), t.begin(), t.end());
      node_last.push_back(keys[a + n - 1]);
    }
  };
  std::vector<uint64_t> l0, l0_last;
  build(0, snods, last, l0, l0_last);
  uint64_t root = l0[0];
  if (l0.size() > 1) {
    if (l0.size() > fan) fail("group too large for this writer");
    std::vector<uint64_t> l1, l1_last;
    build(1, l0, l0_last, l1, l1_last);
    root = l1[0];
  }
  im.put(g.stab, root, 8);
  if (g.entry && im.get(g.entry + 16, 4) == 1) im.put(g.entry + 24, root, 8);  // cached B-tree address
}

// A new, empty group: heap ("" at offset 0), empty B-tree node and header.
uint64_t new_group(Image &im, uint64_t *btree_out = nullptr, uint64_t *heap_out = nullptr) {
  std::vector<unsigned char> seg(8, 0);
  free_block(seg);
  const uint64_t seg_rel = im.append(seg);
  const uint64_t heap = im.append(heap_header(seg.size(), 8, seg_rel));
  std::vector<unsigned char> t = {'T', 'R', 'E', 'E', 0, 0, 0, 0};
  le(t, UNDEF, 8);
  le(t, UNDEF, 8);
  t.resize(btree_node_bytes(im), 0);
  const uint64_t btree = im.append(t);
  std::vector<unsigned char> st;
  le(st, btree, 8);
  le(st, heap, 8);
  if (btree_out) *btree_out = btree;
  if (heap_out) *heap_out = heap;
  return im.append(v1_header({{M_STAB, st}}));
}

std::vector<unsigned char> type_message(const Data &d) {
  std::vector<unsigned char> m;
  switch (d.kind) {
    case Kind::Int:
    case Kind::UInt:
      le(m, 0x10, 1);  // version 1, fixed-point
      le(m, d.kind == Kind::Int ? 0x08 : 0x00, 1);
      le(m, 0, 2);
      le(m, d.size, 4);
      le(m, 0, 2);           // bit offset
      le(m, 8 * d.size, 2);  // precision
      break;
    case Kind::Float:
      le(m, 0x11, 1);  // version 1, floating point
      le(m, 0x20, 1);  // implied leading mantissa bit
      le(m, d.size == 8 ? 63 : 31, 1);  // sign bit position
      le(m, 0, 1);
      le(m, d.size, 4);
      le(m, 0, 2);
      le(m, 8 * d.size, 2);
      le(m, d.size == 8 ? 52 : 23, 1);  // exponent location, size
      le(m, d.size == 8 ? 11 : 8, 1);
      le(m, 0, 1);  // mantissa location, size
      le(m, d.size == 8 ? 52 : 23, 1);
      le(m, d.size == 8 ? 1023 : 127, 4);
      break;
    case Kind::String:
      le(m, 0x13, 1);  // version 1, string
      le(m, 0x01, 1);  // null-padded ASCII
      le(m, 0, 2);
      le(m, d.size, 4);
      break;
  }
  return m;
}

bool same_type(const Image &im, const std::vector<Msg> &ms, const Data &d) {
  const Msg *mt = find(ms, M_TYPE), *msp = find(ms, M_SPACE);
  if (!mt || !msp) return false;
  const Type t = parse_type(im, *mt);
  std::vector<uint64_t> dims;
  std::string why;
  if (!t.why.empty() || t.vlstr || !parse_space(im, *msp, dims, why)) return false;
  return t.kind == d.kind && t.size == d.size && dims == d.dims;
}

void write_one(Image &im, const std::string &path, const Data &d) {
  if (path.size() < 2 || path[0] != '/') fail("dataset path must be absolute: " + path);
  if (d.size == 0 || d.bytes.size() != d.count() * d.size) fail("bad data for " + path);
  std::vector<std::string> parts;
  for (size_t a = 1; a <= path.size();) {
    const size_t b = path.find('/', a);
    const size_t e = b == std::string::npos ? path.size() : b;
    if (e == a) fail("empty path component in " + path);
    parts.push_back(path.substr(a, e - a));
    a = e + 1;
  }
  // walk (and create) the groups; every change moves the group's structures,
  // so the walk restarts from the root after each one
  for (int pass = 0; pass < 2 * (int)parts.size() + 2; pass++) {
    Group g = open_group(im, im.root, im.root_entry);
    size_t k = 0;
    bool changed = false;
    for (; k + 1 < parts.size(); k++) {
      const Entry *e = nullptr;
      for (const Entry &x : g.links)
        if (x.name == parts[k]) e = &x;
      if (!e) {
        insert_link(im, g, parts[k], new_group(im));
        changed = true;
        break;
      }
      g = open_group(im, e->ohdr, e->pos);
    }
    if (changed) continue;
    const std::string &name = parts.back();
    for (const Entry &x : g.links) {
      if (x.name != name) continue;
      const std::vector<Msg> ms = messages(im, x.ohdr);
      const Msg *ml = find(ms, M_LAYOUT);
      if (!ml || !same_type(im, ms, d))
        fail(path + " exists with another type or shape");
      const Layout L = parse_layout(im, *ml);
      if (!L.why.empty()) fail(path + ": " + L.why);
      if (L.compact) {
        if (L.size < d.bytes.size()) fail(path + ": compact storage too small");
        im.need(L.pos, d.bytes.size());
        memcpy(&im.b[L.pos], d.bytes.data(), d.bytes.size());
      } else if (!d.bytes.empty()) {
        uint64_t a = L.addr;
        if (a == UNDEF) {  // storage never allocated
          a = im.append(d.bytes);
          im.put(L.pos, a, 8);
          im.put(L.pos + 8, d.bytes.size(), 8);  // version 3 size field
        } else {
          const uint64_t p = im.at(a);
          im.need(p, d.bytes.size());
          memcpy(&im.b[p], d.bytes.data(), d.bytes.size());
        }
      }
      return;
    }
    // a new dataset: its elements, then its header
    const uint64_t data = d.bytes.empty() ? UNDEF : im.append(d.bytes);
    std::vector<unsigned char> space = {1, (unsigned char)d.dims.size(), 0, 0, 0, 0, 0, 0};
    for (uint64_t x : d.dims) le(space, x, 8);
    const std::vector<unsigned char> fill = {2, 2, 2, 0};  // fill value message, version 2, none defined
    std::vector<unsigned char> layout = {3, 1};            // version 3, contiguous
    le(layout, data, 8);
    le(layout, d.bytes.size(), 8);
    const uint64_t oh =
        im.append(v1_header({{M_SPACE, space}, {M_TYPE, type_message(d)}, {0x05, fill},
                             {M_LAYOUT, layout}}));
    insert_link(im, g, name, oh);
    return;
  }
  fail("could not create the groups of " + path);
}

}  // namespace

bool is_hdf5(const std::string &path) {
  FILE *f = fopen(path.c_str(), "rb");
  if (!f) return false;
  bool hit = false;
  unsigned char s[8];
  for (long off = 0; !hit && off <= (1l << 24); off = off ? 2 * off : 512) {
    if (fseek(f, off, SEEK_SET) != 0 || fread(s, 1, 8, f) != 8) break;
    hit = memcmp(s, SIG, 8) == 0;
  }
  fclose(f);
  return hit;
}

void read_all(const std::string &path, std::map<std::string, Data> &sets,
              std::map<std::string, std::string> &skipped) {
  Image im;
  im.b = slurp(path);
  parse_superblock(im);
  std::set<uint64_t> seen;
  walk(im, im.root, "", 0, seen, sets, skipped);
}

void create(const std::string &path) {
  Image im;
  im.b.assign(96, 0);
  memcpy(im.b.data(), SIG, 8);
  im.b[13] = 8;  // sizes of offsets and lengths
  im.b[14] = 8;
  im.put(16, (uint64_t)im.leafK, 2);
  im.put(18, (uint64_t)im.nodeK, 2);
  im.put(24, 0, 8);      // base address
  im.put(32, UNDEF, 8);  // no free-space information
  im.put(48, UNDEF, 8);  // no driver information
  uint64_t btree = 0, heap = 0;
  const uint64_t root = new_group(im, &btree, &heap);
  im.put(56, 0, 8);  // root entry: name offset, header, cache type 1 with B-tree and heap
  im.put(64, root, 8);
  im.put(72, 1, 4);
  im.put(80, btree, 8);
  im.put(88, heap, 8);
  im.put(40, im.b.size(), 8);  // end of file
  spill(path, im.b);
}

void write(const std::string &path, const std::map<std::string, Data> &sets) {
  Image im;
  im.b = slurp(path);
  parse_superblock(im);
  if (im.version > 1) fail("files with a version 2 or 3 superblock are not written by this writer");
  for (const auto &kv : sets) write_one(im, kv.first, kv.second);
  im.put(im.eof_field, im.b.size(), 8);  // the end-of-file address is absolute
  spill(path, im.b);
}

}  // namespace h5lite
