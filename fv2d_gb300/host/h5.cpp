// h5.cpp -- see h5.hpp.  Layout references are to the HDF5 File Format
// Specification (superblock, object header, message and B-tree sections).
#include "h5.hpp"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <memory>

namespace fv2d {
namespace h5 {

namespace {

constexpr uint64_t UNDEF = ~0ull;
constexpr uint8_t SIGNATURE[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
// Group B-tree / symbol-table node sizes used by this writer: leaf K = 256
// (512 links per group, a single symbol-table node), internal K = 16.
constexpr int LEAF_K = 256;
constexpr int INTERNAL_K = 16;
constexpr uint64_t SNOD_SIZE = 8 + 2 * LEAF_K * 40;
constexpr uint64_t BTREE_SIZE = 24 + 2 * INTERNAL_K * 8 + (2 * INTERNAL_K + 1) * 8;
constexpr uint64_t ROOT_HEAP_CAP = 16 * (2 * LEAF_K + 2);
constexpr uint64_t HEAP_FREE_NULL = 1;  // "no free block" marker of local heaps

// ------------------------------------------------------------------ byte buffers
struct Buf {
  std::vector<uint8_t> b;
  void u8(uint64_t v) { b.push_back((uint8_t)v); }
  void u16(uint64_t v) { for (int k = 0; k < 2; ++k) b.push_back((uint8_t)(v >> (8 * k))); }
  void u32(uint64_t v) { for (int k = 0; k < 4; ++k) b.push_back((uint8_t)(v >> (8 * k))); }
  void u64(uint64_t v) { for (int k = 0; k < 8; ++k) b.push_back((uint8_t)(v >> (8 * k))); }
  void bytes(const void *p, size_t n) { b.insert(b.end(), (const uint8_t *)p, (const uint8_t *)p + n); }
  void pad8() { while (b.size() % 8) b.push_back(0); }
  void zeros(size_t n) { b.insert(b.end(), n, 0); }
  size_t size() const { return b.size(); }
};

uint64_t rd(const uint8_t *p, int n) {
  uint64_t v = 0;
  for (int k = 0; k < n; ++k) v |= (uint64_t)p[k] << (8 * k);
  return v;
}

uint64_t align8(uint64_t n) { return (n + 7) & ~7ull; }

// ------------------------------------------------------------------ messages (writer)
Buf dataspace_msg(const std::vector<uint64_t> &dims) {  // version 1; rank 0 = scalar
  Buf m;
  m.u8(1);
  m.u8(dims.size());
  m.u8(0);
  m.u8(0);
  m.u32(0);
  for (uint64_t d : dims) m.u64(d);
  return m;
}
Buf dtype_f64() {
  Buf m;
  m.u8(0x11);  // version 1, floating point
  m.u8(0x20);  // little-endian, implied leading mantissa bit
  m.u8(63);    // sign bit position
  m.u8(0);
  m.u32(8);
  m.u16(0);    // bit offset
  m.u16(64);   // precision
  m.u8(52);    // exponent location
  m.u8(11);    // exponent size
  m.u8(0);     // mantissa location
  m.u8(52);    // mantissa size
  m.u32(1023); // exponent bias
  return m;
}
Buf dtype_i32() {
  Buf m;
  m.u8(0x10);  // version 1, fixed point
  m.u8(0x08);  // little-endian, signed
  m.u8(0);
  m.u8(0);
  m.u32(4);
  m.u16(0);
  m.u16(32);
  return m;
}
Buf dtype_str(size_t n) {
  Buf m;
  m.u8(0x13);  // version 1, string
  m.u8(0x00);  // null-terminated, ASCII
  m.u8(0);
  m.u8(0);
  m.u32((uint32_t)n);
  return m;
}
Buf attr_msg(const std::string &name, const Buf &dt, const Buf &ds, const void *data, size_t nbytes) {
  Buf m;
  m.u8(1);
  m.u8(0);
  m.u16(name.size() + 1);
  m.u16(dt.size());
  m.u16(ds.size());
  m.bytes(name.c_str(), name.size() + 1);
  m.pad8();
  m.bytes(dt.b.data(), dt.size());
  m.pad8();
  m.bytes(ds.b.data(), ds.size());
  m.pad8();
  m.bytes(data, nbytes);
  m.pad8();
  return m;
}
Buf attr_int(const std::string &name, int32_t v) { return attr_msg(name, dtype_i32(), dataspace_msg({}), &v, 4); }
Buf attr_double(const std::string &name, double v) { return attr_msg(name, dtype_f64(), dataspace_msg({}), &v, 8); }
Buf attr_string(const std::string &name, const std::string &s) {
  std::string z = s;
  z.push_back('\0');
  return attr_msg(name, dtype_str(z.size()), dataspace_msg({}), z.data(), z.size());
}

// Version-1 object header holding the given (type, message) pairs.
Buf object_header(const std::vector<std::pair<int, Buf>> &msgs) {
  uint64_t body = 0;
  for (auto &m : msgs) body += 8 + align8(m.second.size());
  Buf h;
  h.u8(1);
  h.u8(0);
  h.u16(msgs.size());
  h.u32(1);
  h.u32(body);
  h.u32(0);  // align the message area
  for (auto &m : msgs) {
    h.u16(m.first);
    h.u16(align8(m.second.size()));
    h.u8(0);
    h.zeros(3);
    h.bytes(m.second.b.data(), m.second.size());
    h.pad8();
  }
  return h;
}

// ------------------------------------------------------------------ file writer
struct Writer {
  FILE *f = nullptr;
  uint64_t eof = 0;

  uint64_t alloc(uint64_t n) {
    const uint64_t a = align8(eof);
    eof = a + n;
    return a;
  }
  bool put(uint64_t addr, const void *p, size_t n) {
    return fseeko(f, (off_t)addr, SEEK_SET) == 0 && fwrite(p, 1, n, f) == n;
  }
  bool put(uint64_t addr, const Buf &b) { return put(addr, b.b.data(), b.size()); }
  bool get(uint64_t addr, void *p, size_t n) {
    return fseeko(f, (off_t)addr, SEEK_SET) == 0 && fread(p, 1, n, f) == n;
  }

  // contiguous binary64 dataset; returns the object header address
  uint64_t dataset(const double *data, uint64_t n, bool *ok) {
    Buf fill;
    fill.u8(2);  // fill value message version 2
    fill.u8(1);  // space allocated early
    fill.u8(1);  // fill value never written
    fill.u8(0);  // no fill value defined
    const uint64_t data_addr = alloc(8 * n);
    *ok = *ok && put(data_addr, data, 8 * n);
    Buf layout;
    layout.u8(3);
    layout.u8(1);  // contiguous
    layout.u64(data_addr);
    layout.u64(8 * n);
    Buf oh = object_header({{0x0001, dataspace_msg({n})}, {0x0003, dtype_f64()}, {0x0005, fill}, {0x0008, layout}});
    const uint64_t a = alloc(oh.size());
    *ok = *ok && put(a, oh);
    return a;
  }

  struct Entry {
    std::string name;
    uint64_t oh;
    bool group;
    uint64_t btree, heap;
  };

  // Symbol-table structures of a group: local heap with the names, one
  // B-tree node, one symbol-table node.  Returns (btree, heap); heap_cap
  // reserves room for later names.
  std::pair<uint64_t, uint64_t> symbol_table(std::vector<Entry> entries, uint64_t heap_cap, bool *ok) {
    std::sort(entries.begin(), entries.end(), [](const Entry &a, const Entry &b) { return a.name < b.name; });
    Buf names;
    names.zeros(8);  // offset 0: the empty name
    std::vector<uint64_t> off;
    for (auto &e : entries) {
      off.push_back(names.size());
      names.bytes(e.name.c_str(), e.name.size() + 1);
      names.pad8();
    }
    const uint64_t cap = std::max<uint64_t>(heap_cap, names.size());
    const uint64_t heap = alloc(32 + cap);
    Buf h;
    h.bytes("HEAP", 4);
    h.u8(0);
    h.zeros(3);
    h.u64(names.size());
    h.u64(HEAP_FREE_NULL);
    h.u64(heap + 32);
    *ok = *ok && put(heap, h) && put(heap + 32, names);
    const uint64_t btree = alloc(BTREE_SIZE);
    const uint64_t snod = alloc(SNOD_SIZE);
    *ok = *ok && write_btree(btree, snod, entries.empty() ? 0 : off.back());
    *ok = *ok && write_snod(snod, entries, off);
    return {btree, heap};
  }
  bool write_btree(uint64_t at, uint64_t snod, uint64_t last_name) {
    Buf t;
    t.bytes("TREE", 4);
    t.u8(0);   // group node
    t.u8(0);   // leaf level
    t.u16(1);  // one child
    t.u64(UNDEF);
    t.u64(UNDEF);
    t.u64(0);  // key 0: the empty name
    t.u64(snod);
    t.u64(last_name);  // key 1: the largest name in the child
    t.zeros(BTREE_SIZE - t.size());
    return put(at, t);
  }
  bool write_snod(uint64_t at, const std::vector<Entry> &entries, const std::vector<uint64_t> &off) {
    Buf s;
    s.bytes("SNOD", 4);
    s.u8(1);
    s.u8(0);
    s.u16(entries.size());
    for (size_t k = 0; k < entries.size(); ++k) {
      s.u64(off[k]);
      s.u64(entries[k].oh);
      s.u32(entries[k].group ? 1 : 0);
      s.u32(0);
      s.u64(entries[k].group ? entries[k].btree : 0);
      s.u64(entries[k].group ? entries[k].heap : 0);
    }
    s.zeros(SNOD_SIZE - s.size());
    return put(at, s);
  }
};

std::vector<double> plane(const double *q, size_t n, int f) {
  std::vector<double> v(n);
  for (size_t c = 0; c < n; ++c) v[c] = q[4 * c + f];
  return v;
}

void vertices(const RootInfo &r, std::vector<double> *x, std::vector<double> *y) {
  for (int j = r.jbeg; j <= r.jend; ++j)
    for (int i = r.ibeg; i <= r.iend; ++i) {
      x->push_back((i - r.ibeg) * r.dx + r.xmin);
      y->push_back((j - r.jbeg) * r.dy + r.ymin);
    }
}

std::vector<std::pair<int, Buf>> root_attrs(const RootInfo &r) {
  return {{0x000C, attr_int("Ntx", r.Ntx)},   {0x000C, attr_int("Nty", r.Nty)},  {0x000C, attr_int("Nx", r.Nx)},
          {0x000C, attr_int("Ny", r.Ny)},     {0x000C, attr_int("ibeg", r.ibeg)}, {0x000C, attr_int("iend", r.iend)},
          {0x000C, attr_int("jbeg", r.jbeg)}, {0x000C, attr_int("jend", r.jend)},
          {0x000C, attr_string("problem", r.problem)}};
}

Buf superblock(uint64_t eof, uint64_t root_oh, uint64_t root_btree, uint64_t root_heap) {
  Buf s;
  s.bytes(SIGNATURE, 8);
  s.u8(0);  // superblock version
  s.u8(0);  // free-space version
  s.u8(0);  // root group symbol table entry version
  s.u8(0);
  s.u8(0);  // shared header message format version
  s.u8(8);  // size of offsets
  s.u8(8);  // size of lengths
  s.u8(0);
  s.u16(LEAF_K);
  s.u16(INTERNAL_K);
  s.u32(0);  // consistency flags
  s.u64(0);  // base address
  s.u64(UNDEF);
  s.u64(eof);
  s.u64(UNDEF);
  // root group symbol table entry
  s.u64(0);
  s.u64(root_oh);
  s.u32(1);
  s.u32(0);
  s.u64(root_btree);
  s.u64(root_heap);
  return s;
}

// Group "ite_%04d" (or the root of a multiple-output file) payload.
bool write_fields(Writer &w, const double *q, size_t n, std::vector<Writer::Entry> *entries) {
  bool ok = true;
  static const char *names[4] = {"rho", "u", "v", "prs"};
  for (int f = 0; f < 4; ++f) {
    const std::vector<double> p = plane(q, n, f);
    entries->push_back({names[f], w.dataset(p.data(), n, &ok), false, 0, 0});
  }
  return ok;
}

std::string iteration_name(int it) {
  char buf[32];
  std::snprintf(buf, sizeof buf, "ite_%04d", it);
  return buf;
}

}  // namespace

bool write_unique(const std::string &path, bool truncate, const RootInfo &root, int iteration, double t,
                  const double *q, std::string *err) {
  const size_t n = (size_t)root.Nx * root.Ny;
  Writer w;
  const std::string gname = iteration_name(iteration);
  if (truncate) {
    w.f = std::fopen(path.c_str(), "w+b");
    if (!w.f) {
      if (err) *err = "cannot create " + path;
      return false;
    }
    bool ok = true;
    w.eof = 96;
    // root structures first, at fixed places: object header, heap, B-tree, SNOD
    std::vector<std::pair<int, Buf>> rmsgs = root_attrs(root);
    Buf st;
    st.u64(0);
    st.u64(0);
    rmsgs.insert(rmsgs.begin(), {0x0011, st});
    Buf roh = object_header(rmsgs);
    const uint64_t root_oh = w.alloc(roh.size());
    std::vector<Writer::Entry> entries;
    std::vector<double> x, y;
    vertices(root, &x, &y);
    // the root symbol table right after its object header, then the data
    std::vector<Writer::Entry> none;
    auto bt = w.symbol_table(none, ROOT_HEAP_CAP, &ok);
    entries.push_back({"x", w.dataset(x.data(), x.size(), &ok), false, 0, 0});
    entries.push_back({"y", w.dataset(y.data(), y.size(), &ok), false, 0, 0});
    // the snapshot group
    std::vector<Writer::Entry> g;
    ok = ok && write_fields(w, q, n, &g);
    auto gbt = w.symbol_table(g, 0, &ok);
    Buf gst;
    gst.u64(gbt.first);
    gst.u64(gbt.second);
    Buf goh = object_header({{0x0011, gst}, {0x000C, attr_double("time", t)}, {0x000C, attr_int("iteration", iteration)}});
    const uint64_t goh_at = w.alloc(goh.size());
    ok = ok && w.put(goh_at, goh);
    entries.push_back({gname, goh_at, true, gbt.first, gbt.second});
    // rewrite the root symbol table in place with its entries
    {
      std::sort(entries.begin(), entries.end(),
                [](const Writer::Entry &a, const Writer::Entry &b) { return a.name < b.name; });
      Buf names;
      names.zeros(8);
      std::vector<uint64_t> off;
      for (auto &e : entries) {
        off.push_back(names.size());
        names.bytes(e.name.c_str(), e.name.size() + 1);
        names.pad8();
      }
      Buf h;
      h.bytes("HEAP", 4);
      h.u8(0);
      h.zeros(3);
      h.u64(names.size());
      h.u64(HEAP_FREE_NULL);
      h.u64(bt.second + 32);
      ok = ok && w.put(bt.second, h) && w.put(bt.second + 32, names);
      uint64_t snod = 0;
      uint8_t tb[BTREE_SIZE];
      ok = ok && w.get(bt.first, tb, BTREE_SIZE);
      snod = rd(tb + 32, 8);
      ok = ok && w.write_btree(bt.first, snod, off.back()) && w.write_snod(snod, entries, off);
    }
    st.b.clear();
    st.u64(bt.first);
    st.u64(bt.second);
    rmsgs[0].second = st;
    roh = object_header(rmsgs);
    ok = ok && w.put(root_oh, roh);
    ok = ok && w.put(0, superblock(w.eof, root_oh, bt.first, bt.second));
    std::fclose(w.f);
    if (!ok && err) *err = "write failed: " + path;
    return ok;
  }

  // append a group to a file written by write_unique
  w.f = std::fopen(path.c_str(), "r+b");
  if (!w.f) {
    if (err) *err = "cannot open " + path;
    return false;
  }
  auto fail = [&](const std::string &m) {
    std::fclose(w.f);
    if (err) *err = m;
    return false;
  };
  uint8_t sb[96];
  if (!w.get(0, sb, 96) || std::memcmp(sb, SIGNATURE, 8) != 0 || sb[8] != 0 || rd(sb + 16, 2) != LEAF_K ||
      rd(sb + 18, 2) != INTERNAL_K)
    return fail("appending is supported for files written by this library only: " + path);
  w.eof = rd(sb + 40, 8);
  const uint64_t root_btree = rd(sb + 80, 8), root_heap = rd(sb + 88, 8);
  uint8_t tb[BTREE_SIZE];
  uint8_t hh[32];
  if (!w.get(root_btree, tb, BTREE_SIZE) || std::memcmp(tb, "TREE", 4) != 0 || rd(tb + 6, 2) != 1 ||
      !w.get(root_heap, hh, 32) || std::memcmp(hh, "HEAP", 4) != 0)
    return fail("unexpected root group structure in " + path);
  const uint64_t snod = rd(tb + 32, 8);
  const uint64_t heap_size = rd(hh + 8, 8), heap_data = rd(hh + 24, 8);
  if (heap_size > ROOT_HEAP_CAP) return fail("unexpected root group structure in " + path);
  std::vector<uint8_t> heap(heap_size), sn(SNOD_SIZE);
  if (!w.get(heap_data, heap.data(), heap_size) || !w.get(snod, sn.data(), SNOD_SIZE) ||
      std::memcmp(sn.data(), "SNOD", 4) != 0)
    return fail("unexpected root group structure in " + path);
  const int nsym = (int)rd(sn.data() + 6, 2);
  if (nsym + 1 > 2 * LEAF_K || heap_size + 16 + gname.size() > ROOT_HEAP_CAP)
    return fail("too many snapshots in one file (limit " + std::to_string(2 * LEAF_K - 2) + "): " + path);
  std::vector<Writer::Entry> entries;
  for (int k = 0; k < nsym; ++k) {
    const uint8_t *e = sn.data() + 8 + 40 * k;
    Writer::Entry en;
    const uint64_t noff = rd(e, 8);
    const void *z = noff < heap_size ? std::memchr(heap.data() + noff, 0, heap_size - noff) : nullptr;
    if (!z) return fail("unexpected root group structure in " + path);
    en.name = std::string((const char *)heap.data() + noff, (const char *)z - (const char *)heap.data() - noff);
    en.oh = rd(e + 8, 8);
    en.group = rd(e + 16, 4) == 1;
    en.btree = rd(e + 24, 8);
    en.heap = rd(e + 32, 8);
    if (en.name == gname) return fail("group " + gname + " already exists in " + path);
    entries.push_back(en);
  }
  bool ok = true;
  std::vector<Writer::Entry> g;
  ok = ok && write_fields(w, q, n, &g);
  auto gbt = w.symbol_table(g, 0, &ok);
  Buf gst;
  gst.u64(gbt.first);
  gst.u64(gbt.second);
  Buf goh = object_header({{0x0011, gst}, {0x000C, attr_double("time", t)}, {0x000C, attr_int("iteration", iteration)}});
  const uint64_t goh_at = w.alloc(goh.size());
  ok = ok && w.put(goh_at, goh);
  // new name at the end of the root heap, entry in sorted position
  std::vector<uint64_t> off;
  for (int k = 0; k < nsym; ++k) off.push_back(rd(sn.data() + 8 + 40 * k, 8));
  Buf nm;
  nm.bytes(gname.c_str(), gname.size() + 1);
  nm.pad8();
  const uint64_t new_off = heap_size;
  ok = ok && w.put(heap_data + heap_size, nm);
  Buf hdr;
  hdr.bytes("HEAP", 4);
  hdr.u8(0);
  hdr.zeros(3);
  hdr.u64(heap_size + nm.size());
  hdr.u64(HEAP_FREE_NULL);
  hdr.u64(heap_data);
  ok = ok && w.put(root_heap, hdr);
  size_t pos = 0;
  while (pos < entries.size() && entries[pos].name < gname) ++pos;
  entries.insert(entries.begin() + pos, Writer::Entry{gname, goh_at, true, gbt.first, gbt.second});
  off.insert(off.begin() + pos, new_off);
  ok = ok && w.write_snod(snod, entries, off) && w.write_btree(root_btree, snod, off.back());
  Buf eofb;
  eofb.u64(w.eof);
  ok = ok && w.put(40, eofb);
  std::fclose(w.f);
  if (!ok && err) *err = "write failed: " + path;
  return ok;
}

bool write_multiple(const std::string &path, const RootInfo &root, int iteration, double t, const double *q,
                    std::string *err) {
  const size_t n = (size_t)root.Nx * root.Ny;
  Writer w;
  w.f = std::fopen(path.c_str(), "w+b");
  if (!w.f) {
    if (err) *err = "cannot create " + path;
    return false;
  }
  bool ok = true;
  w.eof = 96;
  std::vector<Writer::Entry> entries;
  std::vector<double> x, y;
  vertices(root, &x, &y);
  entries.push_back({"x", w.dataset(x.data(), x.size(), &ok), false, 0, 0});
  entries.push_back({"y", w.dataset(y.data(), y.size(), &ok), false, 0, 0});
  ok = ok && write_fields(w, q, n, &entries);
  auto bt = w.symbol_table(entries, 0, &ok);
  std::vector<std::pair<int, Buf>> rmsgs = root_attrs(root);
  Buf st;
  st.u64(bt.first);
  st.u64(bt.second);
  rmsgs.insert(rmsgs.begin(), {0x0011, st});
  rmsgs.push_back({0x000C, attr_double("time", t)});
  rmsgs.push_back({0x000C, attr_int("iteration", iteration)});
  Buf roh = object_header(rmsgs);
  const uint64_t root_oh = w.alloc(roh.size());
  ok = ok && w.put(root_oh, roh) && w.put(0, superblock(w.eof, root_oh, bt.first, bt.second));
  std::fclose(w.f);
  if (!ok && err) *err = "write failed: " + path;
  return ok;
}

// ==================================================================== XDMF
namespace {
// Text of the XDMF sidecar (IOManager.h:22-73): a temporal collection whose
// grids point at the HDF5 datasets.
std::string xdmf_header(const std::string &h5name, const RootInfo &r) {
  char buf[1024];
  std::snprintf(buf, sizeof buf,
                "<?xml version=\"1.0\" ?>\n<!DOCTYPE Xdmf SYSTEM \"Xdmf.dtd\" [\n<!ENTITY file \"%s:\">\n"
                "<!ENTITY fdim \"%d %d\">\n<!ENTITY gdim \"%d %d\">\n<!ENTITY GridEntity '\n"
                "<Topology TopologyType=\"2DSMesh\" Dimensions=\"&gdim;\"/>\n<Geometry GeometryType=\"X_Y\">\n"
                "  <DataItem Dimensions=\"&gdim;\" NumberType=\"Float\" Precision=\"8\" Format=\"HDF\">&file;/x</DataItem>\n"
                "  <DataItem Dimensions=\"&gdim;\" NumberType=\"Float\" Precision=\"8\" Format=\"HDF\">&file;/y</DataItem>\n"
                "</Geometry>'>\n]>\n<Xdmf Version=\"3.0\">\n<Domain>\n"
                "  <Grid Name=\"TimeSeries\" GridType=\"Collection\" CollectionType=\"Temporal\">\n    ",
                h5name.c_str(), r.Ny, r.Nx, r.Ny + 1, r.Nx + 1);
  return buf;
}
const char *XDMF_FOOTER = "\n  </Grid>\n</Domain>\n</Xdmf>";
std::string xdmf_grid(const std::string &name, double t, const std::string &group) {
  auto scalar = [&](const char *f) {
    return std::string("\n      <Attribute Name=\"") + f +
           "\" AttributeType=\"Scalar\" Center=\"Cell\">\n        <DataItem Dimensions=\"&fdim;\" "
           "NumberType=\"Float\" Precision=\"8\" Format=\"HDF\">&file;/" +
           group + f + "</DataItem>\n      </Attribute>";
  };
  char tb[64];
  std::snprintf(tb, sizeof tb, "%lf", t);
  std::string g = "\n    <Grid Name=\"" + name + "\" GridType=\"Uniform\">\n      <Time Value=\"" + tb +
                  "\" />\n      &GridEntity;";
  g += scalar("rho");
  g += "\n      <Attribute Name=\"velocity\" AttributeType=\"Vector\" Center=\"Cell\">\n        <DataItem "
       "Dimensions=\"&fdim; 2\" ItemType=\"Function\" Function=\"JOIN($0, $1)\">\n          <DataItem "
       "Dimensions=\"&fdim;\" NumberType=\"Float\" Precision=\"8\" Format=\"HDF\">&file;/" +
       group + "u</DataItem>\n          <DataItem Dimensions=\"&fdim;\" NumberType=\"Float\" Precision=\"8\" "
       "Format=\"HDF\">&file;/" + group + "v</DataItem>\n        </DataItem>\n      </Attribute>";
  g += scalar("prs");
  g += "\n    </Grid>\n    ";
  return g;
}
}  // namespace

bool write_xdmf(const std::string &xmf_path, const std::string &h5name, const RootInfo &root, bool truncate,
                bool unique, const std::string &grid_name, double t, const std::string &group, std::string *err) {
  std::string text;
  if (!truncate) {
    std::ifstream in(xmf_path, std::ios::binary);
    if (!in) {
      if (err) *err = "Failed to open XDMF file '" + xmf_path + "' with mode 'r+'.";
      return false;
    }
    text.assign(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>());
  } else {
    text = xdmf_header(h5name, root);
    if (unique) text += XDMF_FOOTER;  // the reference writes the empty series first
  }
  if (unique || !truncate) {
    // rewind over the footer: sizeof includes its terminating zero, so one
    // more character goes (fseek(-sizeof(str_xdmf_footer), SEEK_END))
    const size_t back = std::strlen(XDMF_FOOTER) + (unique ? 1 : 0);
    text.resize(text.size() >= back ? text.size() - back : 0);
  }
  text += xdmf_grid(grid_name, t, group);
  text += XDMF_FOOTER;
  std::ofstream out(xmf_path, std::ios::binary | std::ios::trunc);
  if (!out) {
    if (err) *err = "Failed to open XDMF file for writing: " + xmf_path;
    return false;
  }
  out << text;
  return (bool)out;
}

// ==================================================================== reader
struct Msg {
  int type;
  std::vector<uint8_t> data;
};

// Bounds-checked little-endian field of a message payload.
bool field(const std::vector<uint8_t> &v, size_t off, int n, uint64_t *out) {
  if (n < 0 || n > 8 || off > v.size() || (size_t)n > v.size() - off) return false;
  *out = rd(v.data() + off, n);
  return true;
}

// The reader treats every size, offset and count in the file as untrusted:
// reads stay inside the file, payload fields inside their message, and the
// walks over header continuations and group B-trees are bounded.
constexpr size_t kMaxHeaderChunks = 1024;
constexpr int kMaxTreeDepth = 32;
constexpr size_t kMaxTreeNodes = 1 << 16;

struct File::Impl {
  std::ifstream in;
  uint64_t base = 0, file_size = 0;
  int so = 8, sl = 8;
  uint64_t root_oh = UNDEF;

  bool inside(uint64_t addr, uint64_t n) const {
    return addr <= file_size && base <= file_size - addr && n <= file_size - addr - base;
  }
  bool read(uint64_t addr, void *p, size_t n) {
    if (!inside(addr, n)) return false;
    in.clear();
    in.seekg((std::streamoff)(base + addr));
    in.read((char *)p, (std::streamsize)n);
    return (size_t)in.gcount() == n;
  }
  std::vector<uint8_t> read(uint64_t addr, uint64_t n) {
    std::vector<uint8_t> v;
    if (!inside(addr, n)) return v;  // never allocate more than the file holds
    v.resize((size_t)n);
    if (!read(addr, v.data(), (size_t)n)) v.clear();
    return v;
  }

  bool header(uint64_t addr, std::vector<Msg> *out) {
    uint8_t pre[16];
    if (!read(addr, pre, 16)) return false;
    if (pre[0] == 1) {  // version 1
      const int nmsgs = (int)rd(pre + 2, 2);
      std::vector<std::pair<uint64_t, uint64_t>> chunks{{addr + 16, rd(pre + 8, 4)}};
      int seen = 0;
      for (size_t c = 0; c < chunks.size() && seen < nmsgs; ++c) {
        if (c >= kMaxHeaderChunks) return false;
        std::vector<uint8_t> b = read(chunks[c].first, chunks[c].second);
        if (b.size() != chunks[c].second) return false;
        size_t p = 0;
        while (p + 8 <= b.size() && seen < nmsgs) {
          const int type = (int)rd(&b[p], 2);
          const size_t sz = rd(&b[p + 2], 2);
          if (sz > b.size() - p - 8) return false;
          std::vector<uint8_t> d(b.begin() + p + 8, b.begin() + p + 8 + sz);
          if (type == 0x0010) {
            uint64_t at, len;
            if (!field(d, 0, so, &at) || !field(d, so, sl, &len)) return false;
            chunks.push_back({at, len});
          } else {
            out->push_back({type, std::move(d)});
          }
          p += 8 + sz;
          ++seen;
        }
      }
      return true;
    }
    if (std::memcmp(pre, "OHDR", 4) == 0) {  // version 2
      const int flags = pre[5];
      size_t p = 6;
      if (flags & 0x20) p += 16;
      if (flags & 0x10) p += 4;
      uint8_t tmp[32];
      if (!read(addr, tmp, 32)) return false;
      const int szlen = 1 << (flags & 3);
      const uint64_t chunk0 = rd(tmp + p, szlen);
      p += szlen;
      std::vector<std::pair<uint64_t, uint64_t>> chunks{{addr + p, chunk0}};
      for (size_t c = 0; c < chunks.size(); ++c) {
        if (c >= kMaxHeaderChunks) return false;
        std::vector<uint8_t> b = read(chunks[c].first, chunks[c].second);
        if (b.size() != chunks[c].second) return false;
        if (c > 0 && b.size() < 4) return false;
        size_t q = (c == 0) ? 0 : 4;  // continuation chunks start with "OCHK"
        const size_t end = b.size() - (c == 0 ? 0 : 4);
        const size_t hdr = 4 + ((flags & 0x04) ? 2 : 0);
        while (q + hdr <= end) {
          const int type = b[q];
          const size_t sz = rd(&b[q + 1], 2);
          if (sz > end - q - hdr) break;
          std::vector<uint8_t> d(b.begin() + q + hdr, b.begin() + q + hdr + sz);
          if (type == 0x10) {
            uint64_t at, len;
            if (!field(d, 0, so, &at) || !field(d, so, sl, &len)) return false;
            chunks.push_back({at, len});
          } else if (type != 0) {
            out->push_back({type, std::move(d)});
          }
          q += hdr + sz;
        }
      }
      return true;
    }
    return false;
  }

  // links of the group whose object header is at `oh`
  bool links(uint64_t oh, std::map<std::string, uint64_t> *out) {
    std::vector<Msg> ms;
    if (!header(oh, &ms)) return false;
    bool found = false;
    for (auto &m : ms) {
      if (m.type == 0x0011) {  // symbol table
        found = true;
        uint64_t btree, heap;
        if (!field(m.data, 0, so, &btree) || !field(m.data, so, so, &heap)) return false;
        uint8_t hh[64];
        if (!read(heap, hh, 8 + 2 * sl + so) || std::memcmp(hh, "HEAP", 4) != 0) return false;
        const uint64_t hsize = rd(hh + 8, sl), hdata = rd(hh + 8 + 2 * sl, so);
        std::vector<uint8_t> names = read(hdata, hsize);
        if (names.size() != hsize) return false;
        size_t visited = 0;
        std::function<bool(uint64_t, int)> walk = [&](uint64_t node, int depth) -> bool {
          if (depth > kMaxTreeDepth || ++visited > kMaxTreeNodes) return false;
          uint8_t th[8];
          if (!read(node, th, 8) || std::memcmp(th, "TREE", 4) != 0) return false;
          const int level = th[5], used = (int)rd(th + 6, 2);
          const std::vector<uint8_t> body = read(node + 8 + 2 * so, (uint64_t)used * (so + sl) + sl);
          if (body.empty()) return false;
          for (int k = 0; k < used; ++k) {
            const uint64_t child = rd(body.data() + sl + (size_t)k * (so + sl), so);
            if (level > 0) {
              if (!walk(child, depth + 1)) return false;
              continue;
            }
            uint8_t sh[8];
            if (!read(child, sh, 8) || std::memcmp(sh, "SNOD", 4) != 0) return false;
            const int ns = (int)rd(sh + 6, 2);
            const size_t esz = 2 * so + 4 + 4 + 16;
            const std::vector<uint8_t> es = read(child + 8, (uint64_t)ns * esz);
            if (es.size() != (size_t)ns * esz) return false;
            for (int e = 0; e < ns; ++e) {
              const uint64_t noff = rd(es.data() + e * esz, so);
              if (noff >= names.size()) return false;
              const char *nm = (const char *)names.data() + noff;
              const void *z = std::memchr(nm, 0, names.size() - noff);
              if (!z) return false;  // a name must end inside the heap
              (*out)[std::string(nm, (const char *)z - nm)] = rd(es.data() + e * esz + so, so);
            }
          }
          return true;
        };
        if (!walk(btree, 0)) return false;
      } else if (m.type == 0x0006) {  // link message (compact new-style groups)
        const std::vector<uint8_t> &d = m.data;
        uint64_t fl, ltype = 0, nlen, addr;
        if (!field(d, 1, 1, &fl)) return false;
        size_t p = 2;
        if (fl & 0x08) {
          if (!field(d, p, 1, &ltype)) return false;
          ++p;
        }
        if (fl & 0x04) p += 8;
        if (fl & 0x10) p += 1;
        const int lsz = 1 << (fl & 3);
        if (!field(d, p, lsz, &nlen)) return false;
        p += lsz;
        if (p > d.size() || nlen > d.size() - p) return false;
        const std::string name((const char *)d.data() + p, (size_t)nlen);
        p += (size_t)nlen;
        if (ltype == 0) {
          if (!field(d, p, so, &addr)) return false;
          (*out)[name] = addr;
        }
        found = true;
      } else if (m.type == 0x0002) {
        found = true;  // link info: dense storage is not read here
      }
    }
    return found;
  }

  bool resolve(const std::string &path, uint64_t *oh) {
    uint64_t cur = root_oh;
    size_t p = 0;
    while (p < path.size()) {
      while (p < path.size() && path[p] == '/') ++p;
      if (p >= path.size()) break;
      size_t e = path.find('/', p);
      if (e == std::string::npos) e = path.size();
      std::map<std::string, uint64_t> l;
      if (!links(cur, &l)) return false;
      auto it = l.find(path.substr(p, e - p));
      if (it == l.end()) return false;
      cur = it->second;
      p = e;
    }
    *oh = cur;
    return true;
  }

  struct Attr {
    int dclass = -1, dsize = 0;
    bool is_signed = false;
    uint64_t nelem = 1;
    std::vector<uint8_t> data;
  };

  bool attribute(uint64_t oh, const std::string &name, Attr *a) {
    std::vector<Msg> ms;
    if (!header(oh, &ms)) return false;
    for (auto &m : ms) {
      if (m.type != 0x000C) continue;
      const std::vector<uint8_t> &v = m.data;
      uint64_t ver, nsz, dtsz, dssz;
      if (!field(v, 0, 1, &ver) || !field(v, 2, 2, &nsz) || !field(v, 4, 2, &dtsz) || !field(v, 6, 2, &dssz))
        return false;
      size_t p = 8 + (ver == 3 ? 1 : 0);
      auto adv = [&](uint64_t n) { return ver == 1 ? align8(n) : n; };
      if (p > v.size() || nsz > v.size() - p) return false;
      const std::string an((const char *)v.data() + p, nsz ? (size_t)nsz - 1 : 0);
      p += adv(nsz);
      const size_t dt = p;
      p += adv(dtsz);
      const size_t ds = p;
      p += adv(dssz);
      if (an != name) continue;
      uint64_t c0, c1, dsize, dver, rank, dstype = 0;
      if (!field(v, dt, 1, &c0) || !field(v, dt + 1, 1, &c1) || !field(v, dt + 4, 4, &dsize)) return false;
      if (!field(v, ds, 1, &dver) || !field(v, ds + 1, 1, &rank)) return false;
      if (dver == 2 && !field(v, ds + 3, 1, &dstype)) return false;
      if (dsize == 0 || dsize > 1024) return false;
      a->dclass = (int)(c0 & 0x0f);
      a->dsize = (int)dsize;
      a->is_signed = (c1 & 0x08) != 0;
      const size_t dp = (dver == 1) ? 8 : 4;
      a->nelem = 1;
      for (uint64_t k = 0; k < rank; ++k) {
        uint64_t e;
        if (!field(v, ds + dp + 8 * k, 8, &e)) return false;
        if (e != 0 && a->nelem > (v.size() / e)) return false;  // more elements than the message holds
        a->nelem *= e;
      }
      if (dver == 2 && dstype == 2) a->nelem = 0;  // null dataspace
      if (a->nelem > v.size() / (uint64_t)a->dsize) return false;
      const size_t nb = (size_t)a->nelem * a->dsize;
      if (p > v.size() || nb > v.size() - p) return false;
      a->data.assign(v.data() + p, v.data() + p + nb);
      return true;
    }
    return false;
  }
};

bool File::open(const std::string &path, std::string *err) {
  impl_ = std::make_shared<Impl>();
  Impl &I = *impl_;
  I.in.open(path, std::ios::binary);
  if (!I.in) {
    if (err) *err = "cannot open " + path;
    return false;
  }
  I.in.seekg(0, std::ios::end);
  const std::streamoff fsz = I.in.tellg();
  I.file_size = fsz > 0 ? (uint64_t)fsz : 0;
  // the superblock sits at 0 or after a user block of 512, 1024, 2048, ... bytes
  uint64_t at = 0;
  uint8_t sb[128];
  for (;;) {
    I.base = 0;
    if (!I.read(at, sb, 8)) {
      if (err) *err = "no HDF5 superblock in " + path;
      return false;
    }
    if (std::memcmp(sb, SIGNATURE, 8) == 0) break;
    at = at ? at * 2 : 512;
  }
  std::memset(sb, 0, sizeof sb);
  if (!I.read(at, sb, std::min<uint64_t>(sizeof sb, I.file_size - at))) {
    if (err) *err = "short superblock in " + path;
    return false;
  }
  const int ver = sb[8];
  uint64_t base;
  if (ver <= 1) {
    I.so = sb[13];
    I.sl = sb[14];
  } else {
    I.so = sb[9];
    I.sl = sb[10];
  }
  if ((I.so != 2 && I.so != 4 && I.so != 8) || (I.sl != 2 && I.sl != 4 && I.sl != 8)) {
    if (err) *err = "unsupported offset or length size in " + path;
    return false;
  }
  if (ver <= 1) {
    size_t p = 24 + (ver == 1 ? 4 : 0);
    base = rd(sb + p, I.so);
    p += 4 * I.so;  // base, free-space, end-of-file, driver info
    p += I.so;      // root entry: link name offset
    I.root_oh = rd(sb + p, I.so);
  } else {
    size_t p = 12;
    base = rd(sb + p, I.so);
    p += 3 * I.so;  // base, superblock extension, end of file
    I.root_oh = rd(sb + p, I.so);
  }
  I.base = base;
  if (I.base == 0 && at != 0) I.base = at;  // base address relative to the user block
  if (I.base > I.file_size) {
    if (err) *err = "base address past the end of " + path;
    return false;
  }
  return true;
}

bool File::list(const std::string &group, std::vector<std::string> *names, std::string *err) {
  uint64_t oh;
  std::map<std::string, uint64_t> l;
  if (!impl_ || !impl_->resolve(group, &oh) || !impl_->links(oh, &l)) {
    if (err) *err = "cannot list group " + group;
    return false;
  }
  names->clear();
  for (auto &e : l) names->push_back(e.first);
  return true;
}

bool File::read_doubles(const std::string &dataset, std::vector<double> *out, std::vector<uint64_t> *dims,
                        std::string *err) {
  auto fail = [&](const std::string &m) {
    if (err) *err = m + ": " + dataset;
    return false;
  };
  uint64_t oh;
  if (!impl_ || !impl_->resolve(dataset, &oh)) return fail("no such dataset");
  std::vector<Msg> ms;
  if (!impl_->header(oh, &ms)) return fail("bad object header");
  const int so = impl_->so, sl = impl_->sl;
  std::vector<uint64_t> d;
  int dclass = -1, dsize = 0;
  bool big_endian = false;
  int layout = -1;
  uint64_t addr = UNDEF, size = 0;
  std::vector<uint8_t> compact;
  for (auto &m : ms) {
    const std::vector<uint8_t> &v = m.data;
    uint64_t x0, x1, x2;
    if (m.type == 0x0001) {  // dataspace
      if (!field(v, 0, 1, &x0) || !field(v, 1, 1, &x1)) return fail("bad dataspace");
      const size_t o = x0 == 1 ? 8 : 4;
      d.clear();
      for (uint64_t k = 0; k < x1; ++k) {
        uint64_t e;
        if (!field(v, o + 8 * k, sl, &e)) return fail("bad dataspace");
        d.push_back(e);
      }
    } else if (m.type == 0x0003) {  // datatype
      if (!field(v, 0, 1, &x0) || !field(v, 1, 1, &x1) || !field(v, 4, 4, &x2)) return fail("bad datatype");
      dclass = (int)(x0 & 0x0f);
      big_endian = (x1 & 1) != 0;
      dsize = (int)std::min<uint64_t>(x2, 1u << 20);
    } else if (m.type == 0x0008) {  // data layout
      if (!field(v, 0, 1, &x0)) return fail("bad layout");
      if (x0 >= 3) {
        if (!field(v, 1, 1, &x1)) return fail("bad layout");
        layout = (int)x1;
        if (layout == 1) {
          if (!field(v, 2, so, &addr) || !field(v, 2 + so, sl, &size)) return fail("bad layout");
        } else if (layout == 0) {
          if (!field(v, 2, 2, &x2) || x2 > v.size() - 4) return fail("bad layout");
          compact.assign(v.begin() + 4, v.begin() + 4 + (size_t)x2);
        }
      } else {  // versions 1 and 2
        if (!field(v, 1, 1, &x1) || !field(v, 2, 1, &x2)) return fail("bad layout");
        const uint64_t rank = x1;
        layout = (int)x2;
        size_t q = 8;
        if (layout != 0) {
          if (!field(v, q, so, &addr)) return fail("bad layout");
          q += so;
        }
        q += 4 * rank;
        if (layout == 0) {
          uint64_t cn;
          if (!field(v, q, 4, &cn) || cn > v.size() - q - 4) return fail("bad layout");
          compact.assign(v.begin() + q + 4, v.begin() + q + 4 + (size_t)cn);
        }
      }
    }
  }
  if (dclass != 1 || (dsize != 8 && dsize != 4) || big_endian) return fail("not a little-endian float dataset");
  uint64_t n = 1;
  for (uint64_t x : d) {
    if (x != 0 && n > impl_->file_size / x) return fail("dataset larger than the file");
    n *= x;
  }
  std::vector<uint8_t> raw;
  if (layout == 1) {
    if (addr == UNDEF) {
      if (n > (1ull << 40) / (uint64_t)dsize) return fail("dataset too large");
      raw.assign(n * dsize, 0);
    } else {
      if (n > impl_->file_size / (uint64_t)dsize) return fail("dataset larger than the file");
      raw = impl_->read(addr, n * dsize);
      if (raw.size() != n * dsize) return fail("short read");
    }
  } else if (layout == 0) {
    raw = compact;
    if (n > raw.size() / (uint64_t)dsize) return fail("short compact data");
  } else {
    return fail("chunked datasets are not read here");
  }
  (void)size;
  out->resize(n);
  for (uint64_t k = 0; k < n; ++k) {
    if (dsize == 8) {
      std::memcpy(&(*out)[k], raw.data() + 8 * k, 8);
    } else {
      float f;
      std::memcpy(&f, raw.data() + 4 * k, 4);
      (*out)[k] = f;
    }
  }
  if (dims) *dims = d;
  return true;
}

bool File::has_attr(const std::string &object, const std::string &name) {
  uint64_t oh;
  Impl::Attr a;
  return impl_ && impl_->resolve(object, &oh) && impl_->attribute(oh, name, &a);
}

bool File::attr_double(const std::string &object, const std::string &name, double *v, std::string *err) {
  uint64_t oh;
  Impl::Attr a;
  if (!impl_ || !impl_->resolve(object, &oh) || !impl_->attribute(oh, name, &a) || a.nelem < 1) {
    if (err) *err = "no attribute " + name + " on " + object;
    return false;
  }
  if (a.dclass == 1 && a.dsize == 8) {
    std::memcpy(v, a.data.data(), 8);
  } else if (a.dclass == 1 && a.dsize == 4) {
    float f;
    std::memcpy(&f, a.data.data(), 4);
    *v = f;
  } else if (a.dclass == 0 && a.dsize >= 1 && a.dsize <= 8) {
    long long i = (long long)rd(a.data.data(), a.dsize);
    if (a.is_signed && a.dsize < 8 && (i >> (8 * a.dsize - 1)) & 1) i -= 1LL << (8 * a.dsize);
    *v = (double)i;
  } else {
    if (err) *err = "attribute " + name + " is not numeric";
    return false;
  }
  return true;
}

bool File::attr_int(const std::string &object, const std::string &name, long long *v, std::string *err) {
  uint64_t oh;
  Impl::Attr a;
  if (!impl_ || !impl_->resolve(object, &oh) || !impl_->attribute(oh, name, &a) || a.nelem < 1 || a.dclass != 0 ||
      a.dsize < 1 || a.dsize > 8) {
    if (err) *err = "no integer attribute " + name + " on " + object;
    return false;
  }
  long long i = (long long)rd(a.data.data(), a.dsize);
  if (a.is_signed && a.dsize < 8 && ((i >> (8 * a.dsize - 1)) & 1)) i -= 1LL << (8 * a.dsize);
  *v = i;
  return true;
}

bool File::attr_string(const std::string &object, const std::string &name, std::string *v, std::string *err) {
  uint64_t oh;
  Impl::Attr a;
  if (!impl_ || !impl_->resolve(object, &oh) || !impl_->attribute(oh, name, &a) || a.dclass != 3) {
    if (err) *err = "no fixed-length string attribute " + name + " on " + object;
    return false;
  }
  v->assign((const char *)a.data.data(), a.data.size());
  const size_t z = v->find('\0');
  if (z != std::string::npos) v->resize(z);
  return true;
}

bool read_snapshot(const std::string &path, const std::string &group_in, int nx, int ny, std::vector<double> *q,
                   double *time, int *iteration, std::string *err) {
  File f;
  if (!f.open(path, err)) return false;
  std::string group = group_in;
  long long it = 0;
  if (f.has_attr("/", "time")) {  // one file per snapshot (IOManager.h:321-327)
    if (!f.attr_double("/", "time", time, err) || !f.attr_int("/", "iteration", &it, err)) return false;
    group = "";
  } else {
    if (group.empty()) {  // the object before x and y (IOManager.h:330-334)
      std::vector<std::string> names;
      if (!f.list("/", &names, err)) return false;
      if (names.size() < 3) {
        if (err) *err = "no snapshot group in " + path;
        return false;
      }
      group = names[names.size() - 3];
    }
    if (!f.attr_double(group, "time", time, err) || !f.attr_int(group, "iteration", &it, err)) return false;
  }
  *iteration = (int)it;
  static const char *fields[4] = {"rho", "u", "v", "prs"};
  const size_t n = (size_t)nx * ny;
  q->assign(4 * n, 0.0);
  for (int k = 0; k < 4; ++k) {
    std::vector<double> v;
    std::vector<uint64_t> dims;
    if (!f.read_doubles(group + "/" + fields[k], &v, &dims, err)) return false;
    if (v.size() != n) {  // IOManager.h:345-351
      if (err)
        *err = "Attempting to restart with a different resolution ! Ncells (restart) = " + std::to_string(v.size()) +
               "; Run resolution = " + std::to_string(nx) + "x" + std::to_string(ny) + "=" + std::to_string(n);
      return false;
    }
    for (size_t c = 0; c < n; ++c) (*q)[4 * c + k] = v[c];
  }
  return true;
}

}  // namespace h5
}  // namespace fv2d
