// tag_h5_write: a self-contained writer of HDF5 files in the layout Trixi's
// SaveSolutionCallback produces and Trixi2Vtk reads (root attributes, one
// 1-D float64 dataset per variable with a "name" string attribute).  No
// HDF5 library is linked; the file is encoded here from the HDF5 File Format
// Specification (The HDF Group, format version 0 structures):
//   superblock version 0, version-1 object headers, a root group held in a
//   symbol table (one version-1 B-tree node of group type, symbol-table nodes,
//   one local heap), contiguous dataset storage, version-1 attribute messages.
// Every HDF5 library since 1.0 reads these structures.  The encodings of the
// pieces that the specification leaves to the implementation follow what the
// HDF5 library itself writes (a MATLAB 7.3 file written by it serves as the
// check in the tests): an empty local-heap free list is stored as offset 1,
// the first B-tree key names the empty string, key i + 1 the last name of
// child i, scalar dataspaces have rank 0, fixed-length strings carry no
// terminator when they fill their size exactly.
//
// Reference: Trixi.save_solution_file as TrixiAtmo.jl overrides it,
// src/callbacks_step/save_solution_2d_manifold_in_3d_cartesian.jl:44-118
// (attributes :73-84, variables :86-95, element / node variables :97-115).
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>

#include "trixiatmo_gpu.h"

namespace tag {
void set_last_error(const std::string& msg);
}

namespace {

constexpr uint64_t kUndef = ~0ull;
constexpr int kLeafK = 4;        // group leaf node K: 2K entries per symbol-table node
constexpr int kInternalK = 16;   // group internal node K: 2K children per B-tree node
constexpr size_t kSuperblock = 96;
constexpr size_t kEntry = 40;    // symbol-table entry with 8-byte offsets and lengths
constexpr size_t kSnodBytes = 8 + 2 * kLeafK * kEntry;
constexpr size_t kTreeBytes = 24 + (2 * kInternalK) * 8 + (2 * kInternalK + 1) * 8;

int h5fail(int code, const std::string& msg) {
  tag::set_last_error("tag_h5_write: " + msg);
  return code;
}

size_t pad8(size_t n) { return (n + 7) & ~size_t(7); }

struct Bytes {
  std::vector<uint8_t> b;
  void u8(unsigned v) { b.push_back(uint8_t(v)); }
  void u16(unsigned v) { for (int k = 0; k < 2; ++k) b.push_back(uint8_t(v >> (8 * k))); }
  void u32(uint32_t v) { for (int k = 0; k < 4; ++k) b.push_back(uint8_t(v >> (8 * k))); }
  void u64(uint64_t v) { for (int k = 0; k < 8; ++k) b.push_back(uint8_t(v >> (8 * k))); }
  void raw(const void* p, size_t n) {
    const uint8_t* c = static_cast<const uint8_t*>(p);
    b.insert(b.end(), c, c + n);
  }
  void zeros(size_t n) { b.insert(b.end(), n, 0); }
  void align8() { b.resize(pad8(b.size()), 0); }
  size_t size() const { return b.size(); }
};

// ---- datatype and dataspace messages (the message bodies) -------------------

// IEEE binary64, little endian: class 1, version 1
std::vector<uint8_t> dtype_f64() {
  Bytes m;
  m.u8(0x11);                 // version 1, class floating point
  m.u8(0x20); m.u8(63); m.u8(0);  // little endian, implied msb mantissa; sign at bit 63
  m.u32(8);
  m.u16(0); m.u16(64);        // bit offset, precision
  m.u8(52); m.u8(11);         // exponent location, size
  m.u8(0); m.u8(52);          // mantissa location, size
  m.u32(1023);                // exponent bias
  return m.b;
}

// 64-bit two's complement, little endian: class 0, version 1
std::vector<uint8_t> dtype_i64() {
  Bytes m;
  m.u8(0x10);
  m.u8(0x08); m.u8(0); m.u8(0);  // signed
  m.u32(8);
  m.u16(0); m.u16(64);
  return m.b;
}

// fixed-length string of `len` bytes, null-terminated padding, UTF-8: class 3
std::vector<uint8_t> dtype_string(uint32_t len) {
  Bytes m;
  m.u8(0x13);
  m.u8(0x10); m.u8(0); m.u8(0);
  m.u32(len);
  return m.b;
}

// version-1 dataspace: rank 0 (scalar) or rank 1 of `n` elements
std::vector<uint8_t> dspace(int rank, uint64_t n) {
  Bytes m;
  m.u8(1); m.u8(uint8_t(rank)); m.u8(0); m.u8(0);
  m.u32(0);
  if (rank == 1) m.u64(n);
  return m.b;
}

// version-1 attribute message body
std::vector<uint8_t> attribute_msg(const char* name, const std::vector<uint8_t>& dt,
                                   const std::vector<uint8_t>& ds, const void* data, size_t bytes) {
  const size_t nlen = std::strlen(name) + 1;
  Bytes m;
  m.u8(1); m.u8(0);
  m.u16(unsigned(nlen)); m.u16(unsigned(dt.size())); m.u16(unsigned(ds.size()));
  m.raw(name, nlen); m.align8();
  m.raw(dt.data(), dt.size()); m.align8();
  m.raw(ds.data(), ds.size()); m.align8();
  m.raw(data, bytes);
  return m.b;
}

struct Msg {
  uint16_t type;
  uint8_t flags;
  std::vector<uint8_t> body;
};

enum : uint16_t { kMsgDataspace = 1, kMsgDatatype = 3, kMsgFill = 5, kMsgLayout = 8,
                  kMsgAttribute = 12, kMsgSymbolTable = 17 };

// version-1 object header: 16-byte prefix, messages padded to 8 bytes
size_t object_header_bytes(const std::vector<Msg>& msgs) {
  size_t s = 16;
  for (const Msg& m : msgs) s += 8 + pad8(m.body.size());
  return s;
}

void object_header(Bytes& out, const std::vector<Msg>& msgs) {
  const size_t body = object_header_bytes(msgs) - 16;
  out.u8(1); out.u8(0);
  out.u16(unsigned(msgs.size()));
  out.u32(1);                 // reference count
  out.u32(uint32_t(body));
  out.u32(0);                 // alignment of the first message
  for (const Msg& m : msgs) {
    out.u16(m.type);
    out.u16(unsigned(pad8(m.body.size())));
    out.u8(m.flags); out.u8(0); out.u8(0); out.u8(0);
    out.raw(m.body.data(), m.body.size());
    out.align8();
  }
}

Msg attribute(const tag_h5_attribute& a) {
  if (a.type == TAG_H5_INT64) {
    const int64_t v = a.i;
    return {kMsgAttribute, 0, attribute_msg(a.name, dtype_i64(), dspace(0, 0), &v, 8)};
  }
  if (a.type == TAG_H5_FLOAT64) {
    const double v = a.d;
    return {kMsgAttribute, 0, attribute_msg(a.name, dtype_f64(), dspace(0, 0), &v, 8)};
  }
  const char* s = a.s ? a.s : "";
  const size_t len = std::strlen(s);
  const char zero = 0;
  return {kMsgAttribute, 0,
          attribute_msg(a.name, dtype_string(uint32_t(std::max<size_t>(len, 1))), dspace(0, 0),
                        len ? static_cast<const void*>(s) : &zero, std::max<size_t>(len, 1))};
}

std::vector<Msg> dataset_messages(const tag_h5_dataset& d, uint64_t data_addr) {
  std::vector<Msg> msgs;
  // fill value, version 1: allocation late, write if set, defined, no value
  Bytes fill;
  fill.u8(1); fill.u8(2); fill.u8(2); fill.u8(1); fill.u32(0);
  msgs.push_back({kMsgFill, 1, fill.b});
  msgs.push_back({kMsgDatatype, 1, dtype_f64()});
  msgs.push_back({kMsgDataspace, 0, dspace(1, uint64_t(d.count))});
  // layout version 3, contiguous
  Bytes lay;
  lay.u8(3); lay.u8(1);
  lay.u64(d.count > 0 ? data_addr : kUndef);
  lay.u64(uint64_t(d.count) * 8);
  msgs.push_back({kMsgLayout, 1, lay.b});
  if (d.var_name) {
    tag_h5_attribute a{"name", TAG_H5_STRING, 0, 0.0, d.var_name};
    msgs.push_back(attribute(a));
  }
  return msgs;
}

// a link name: not empty, not ".", no '/', at most 1024 bytes
bool valid_name(const char* s) {
  if (!s || !*s || std::strcmp(s, ".") == 0 || std::strlen(s) > 1024) return false;
  return std::strchr(s, '/') == nullptr;
}

}  // namespace

extern "C" int tag_h5_write(const char* path, const tag_h5_attribute* attrs, int32_t nattrs,
                            const tag_h5_dataset* sets, int32_t nsets) {
  if (!path || nattrs < 0 || nsets < 0 || (nattrs && !attrs) || (nsets && !sets))
    return h5fail(TAG_E_INVALID, "bad argument");
  // numbers are stored in the host's byte order, declared little endian
  const uint16_t probe = 1;
  if (*reinterpret_cast<const uint8_t*>(&probe) != 1)
    return h5fail(TAG_E_INVALID, "big-endian hosts are not supported");
  if (nsets > 2 * kLeafK * 2 * kInternalK)
    return h5fail(TAG_E_INVALID, "at most 256 datasets per file");
  for (int32_t k = 0; k < nattrs; ++k) {
    const tag_h5_attribute& a = attrs[k];
    if (!a.name || !*a.name || std::strlen(a.name) > 1024)
      return h5fail(TAG_E_INVALID, "attribute name empty or longer than 1024 bytes");
    if (a.type < TAG_H5_INT64 || a.type > TAG_H5_STRING)
      return h5fail(TAG_E_INVALID, "attribute type must be TAG_H5_INT64, _FLOAT64 or _STRING");
    if (a.type == TAG_H5_STRING && a.s && std::strlen(a.s) > 60000)
      return h5fail(TAG_E_INVALID, "string attribute longer than 60000 bytes");
    for (int32_t l = 0; l < k; ++l)
      if (std::strcmp(attrs[l].name, a.name) == 0)
        return h5fail(TAG_E_INVALID, std::string("duplicate attribute ") + a.name);
  }
  // the group's entries in name order (strcmp), as the B-tree requires
  std::vector<int> order(nsets);
  for (int32_t k = 0; k < nsets; ++k) {
    const tag_h5_dataset& d = sets[k];
    if (!valid_name(d.name)) return h5fail(TAG_E_INVALID, "dataset name empty or with '/'");
    if (d.count < 0 || d.count > (int64_t(1) << 56) || (d.count > 0 && !d.data))
      return h5fail(TAG_E_INVALID, std::string("dataset ") + d.name + ": bad data or count");
    if (d.var_name && std::strlen(d.var_name) > 60000)
      return h5fail(TAG_E_INVALID, "variable name longer than 60000 bytes");
    order[k] = k;
  }
  std::sort(order.begin(), order.end(),
            [&](int a, int b) { return std::strcmp(sets[a].name, sets[b].name) < 0; });
  for (int32_t k = 1; k < nsets; ++k)
    if (std::strcmp(sets[order[k - 1]].name, sets[order[k]].name) == 0)
      return h5fail(TAG_E_INVALID, std::string("duplicate dataset ") + sets[order[k]].name);

  // local heap data segment: the empty name at 0, then each dataset name
  Bytes heap_data;
  heap_data.zeros(8);
  std::vector<uint64_t> name_off(nsets);
  for (int32_t r = 0; r < nsets; ++r) {
    const char* nm = sets[order[r]].name;
    name_off[r] = heap_data.size();
    heap_data.raw(nm, std::strlen(nm) + 1);
    heap_data.align8();
  }
  const int nsnod = (nsets + 2 * kLeafK - 1) / (2 * kLeafK);

  // root group messages: the symbol table (addresses filled in below) and attributes
  std::vector<Msg> root;
  root.push_back({kMsgSymbolTable, 1, std::vector<uint8_t>(16, 0)});
  for (int32_t k = 0; k < nattrs; ++k) root.push_back(attribute(attrs[k]));

  // addresses: superblock, root header, heap, B-tree, symbol-table nodes,
  // dataset headers, raw data
  const uint64_t a_root = kSuperblock;
  const uint64_t a_heap = a_root + object_header_bytes(root);
  const uint64_t a_heap_data = a_heap + 32;
  const uint64_t a_tree = a_heap_data + heap_data.size();
  const uint64_t a_snod = a_tree + kTreeBytes;
  uint64_t a = a_snod + (uint64_t)nsnod * kSnodBytes;
  std::vector<uint64_t> a_oh(nsets), a_raw(nsets);
  std::vector<std::vector<Msg>> oh(nsets);
  for (int32_t r = 0; r < nsets; ++r) {
    oh[r] = dataset_messages(sets[order[r]], 0);
    a_oh[r] = a;
    a += object_header_bytes(oh[r]);
  }
  for (int32_t r = 0; r < nsets; ++r) {
    a_raw[r] = a;
    a += (uint64_t)sets[order[r]].count * 8;
    oh[r] = dataset_messages(sets[order[r]], a_raw[r]);
  }
  const uint64_t eof = a;
  {
    Bytes st;
    st.u64(a_tree);
    st.u64(a_heap);
    root[0].body = st.b;
  }

  Bytes meta;
  // superblock version 0
  const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
  meta.raw(sig, 8);
  meta.u8(0); meta.u8(0); meta.u8(0); meta.u8(0);  // superblock, free space, root entry, reserved
  meta.u8(0); meta.u8(8); meta.u8(8); meta.u8(0);  // shared header version, offsets, lengths
  meta.u16(kLeafK); meta.u16(kInternalK);
  meta.u32(0);                                     // consistency flags
  meta.u64(0);                                     // base address
  meta.u64(kUndef);                                // free-space info
  meta.u64(eof);
  meta.u64(kUndef);                                // driver information block
  // root group symbol-table entry: cached B-tree and heap addresses
  meta.u64(0); meta.u64(a_root); meta.u32(1); meta.u32(0); meta.u64(a_tree); meta.u64(a_heap);
  object_header(meta, root);
  // local heap
  meta.raw("HEAP", 4); meta.u8(0); meta.zeros(3);
  meta.u64(heap_data.size());
  meta.u64(1);                                     // no free block
  meta.u64(a_heap_data);
  meta.raw(heap_data.b.data(), heap_data.size());
  // B-tree node (group type, leaf level): key 0 the empty name, key s + 1 the
  // last name of symbol-table node s
  const size_t tree0 = meta.size();
  meta.raw("TREE", 4); meta.u8(0); meta.u8(0); meta.u16(unsigned(nsnod));
  meta.u64(kUndef); meta.u64(kUndef);
  meta.u64(0);
  for (int s = 0; s < nsnod; ++s) {
    meta.u64(a_snod + (uint64_t)s * kSnodBytes);
    const int last = std::min<int>(nsets, (s + 1) * 2 * kLeafK) - 1;
    meta.u64(name_off[last]);
  }
  meta.zeros(tree0 + kTreeBytes - meta.size());
  // symbol-table nodes
  for (int s = 0; s < nsnod; ++s) {
    const size_t n0 = meta.size();
    const int r0 = s * 2 * kLeafK, r1 = std::min<int>(nsets, r0 + 2 * kLeafK);
    meta.raw("SNOD", 4); meta.u8(1); meta.u8(0); meta.u16(unsigned(r1 - r0));
    for (int r = r0; r < r1; ++r) {
      meta.u64(name_off[r]); meta.u64(a_oh[r]); meta.u32(0); meta.u32(0); meta.zeros(16);
    }
    meta.zeros(n0 + kSnodBytes - meta.size());
  }
  for (int32_t r = 0; r < nsets; ++r) object_header(meta, oh[r]);
  if (nsets ? meta.size() != a_raw[0] : meta.size() != eof)
    return h5fail(TAG_E_INVALID, "internal layout error");

  FILE* f = std::fopen(path, "wb");
  if (!f) return h5fail(TAG_E_IO, std::string("cannot open ") + path + " for writing");
  bool ok = std::fwrite(meta.b.data(), 1, meta.size(), f) == meta.size();
  for (int32_t r = 0; ok && r < nsets; ++r) {
    const tag_h5_dataset& d = sets[order[r]];
    const size_t bytes = (size_t)d.count * 8;
    if (bytes) ok = std::fwrite(d.data, 1, bytes, f) == bytes;
  }
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return h5fail(TAG_E_IO, std::string("write to ") + path + " failed");
  return TAG_OK;
}
