// hdf5_io.cpp -- the reference's HDF5 files without libhdf5.
//
// The reference reads its measurement from the dataset "messung" of an HDF5
// file (H5Reader.hpp:16, :39-70: any shape, read as float) and writes images
// as the 3-D float dataset "density" [nx][ny][nz] with scalar attributes
// xmin, ymin, zmin (float, the grid origin), xmax, ymax, zmax (float, origin +
// n * pitch) and xnbin, ynbin, znbin (int) (H5DensityWriter.hpp:140-199).
// libhdf5 is not part of this build, so this file reads and writes those
// files itself, following the published HDF5 file format specification:
//
//  * reading: a superblock of version 0-3 (after a user block of 0, 512,
//    1024, ... bytes), object headers of version 1 and 2 (with continuation
//    blocks), groups held as symbol tables (version-1 B-tree, symbol table
//    nodes, local heap) or as compact link messages, datasets with
//    contiguous or compact storage, IEEE float and integer element types of
//    either byte order (converted to float), scalar attributes;
//  * writing: what libhdf5 writes by default for these files -- superblock
//    version 0, version-1 object headers, the root group as a symbol table,
//    contiguous little-endian float data -- so libhdf5 (and the reference's
//    readers) open them.
// Host code only: paths and host buffers.
#include <stdint.h>

#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/epet_gb300.h"

namespace epet {
epet_status set_error(epet_status st, const char* fmt, ...);  // runtime.cu

namespace h5 {

#define H5_CHECK(call)            \
  do {                            \
    epet_status s_ = (call);      \
    if (s_ != EPET_OK) return s_; \
  } while (0)

constexpr uint64_t kUndef = ~uint64_t(0);
const unsigned char kSig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};

// ------------------------------------------------------------------ reading

struct Reader {
  std::vector<unsigned char> d;
  uint64_t base = 0;       // file offset of the superblock (addresses are relative to it)
  int so = 8, sl = 8;      // sizes of offsets and lengths
  std::string err;

  bool ok(uint64_t off, uint64_t n) const { return off <= d.size() && n <= d.size() - off; }
  uint64_t uint(uint64_t off, int n) const {  // little-endian
    uint64_t v = 0;
    for (int i = n - 1; i >= 0; i--) v = (v << 8) | d[off + i];
    return v;
  }
  uint64_t addr(uint64_t a) const { return a == kUndef ? kUndef : a + base; }
};

struct DatasetInfo {
  std::vector<uint64_t> dims;
  int cls = -1;        // 0 fixed point, 1 floating point
  int size = 0;        // element bytes
  bool big = false, sgn = false;
  int layout = -1;     // 0 compact, 1 contiguous, 2 chunked
  uint64_t data = kUndef, data_size = 0;
  struct Attr {
    std::string name;
    int cls, size;
    bool big, sgn;
    std::vector<unsigned char> raw;
  };
  std::vector<Attr> attrs;
};

struct Msg {
  int type;
  uint64_t off, size;  // file offsets of the message data
};

static bool header_messages(Reader& R, uint64_t oh, std::vector<Msg>* out) {
  if (!R.ok(oh, 16)) return false;
  if (R.d[oh] == 1) {  // version 1: 16-byte prefix, 8-byte-aligned messages
    uint64_t nmsg = R.uint(oh + 2, 2);
    std::vector<std::pair<uint64_t, uint64_t>> blocks = {{oh + 16, R.uint(oh + 8, 4)}};
    for (size_t b = 0; b < blocks.size() && out->size() <= nmsg + 64; b++) {
      uint64_t p = blocks[b].first, end = p + blocks[b].second;
      if (!R.ok(p, end - p)) return false;
      while (p + 8 <= end) {
        const int type = (int)R.uint(p, 2);
        const uint64_t sz = R.uint(p + 2, 2);
        if (p + 8 + sz > end) return false;
        out->push_back({type, p + 8, sz});
        if (type == 0x10 && sz >= (uint64_t)(R.so + R.sl))
          blocks.push_back({R.addr(R.uint(p + 8, R.so)), R.uint(p + 8 + R.so, R.sl)});
        p += 8 + ((sz + 7) & ~uint64_t(7));
      }
    }
    return true;
  }
  if (memcmp(&R.d[oh], "OHDR", 4) != 0 || R.d[oh + 4] != 2) return false;
  const int flags = R.d[oh + 5];
  uint64_t p = oh + 6;
  if (flags & 0x20) p += 16;  // times
  if (flags & 0x10) p += 4;   // attribute phase change values
  const int csz = 1 << (flags & 3);
  const uint64_t chunk = R.uint(p, csz);
  p += csz;
  std::vector<std::pair<uint64_t, uint64_t>> blocks = {{p, chunk}};
  for (size_t b = 0; b < blocks.size() && b < 4096; b++) {
    uint64_t q = blocks[b].first, end = q + blocks[b].second;
    if (b > 0) q += 4;  // "OCHK"
    if (!R.ok(q, end - q)) return false;
    while (q + 4 <= end) {
      const int type = R.d[q];
      const uint64_t sz = R.uint(q + 1, 2);
      const int mflags = R.d[q + 3];
      q += 4 + ((flags & 0x04) ? 2 : 0);
      if (q + sz > end) break;
      (void)mflags;
      out->push_back({type, q, sz});
      if (type == 0x10 && sz >= (uint64_t)(R.so + R.sl))
        blocks.push_back({R.addr(R.uint(q, R.so)), R.uint(q + R.so, R.sl) - 4});
      q += sz;
    }
  }
  return true;
}

// Datatype message at off: class, size, byte order, sign.
static bool parse_type(const Reader& R, uint64_t off, int* cls, int* size, bool* big, bool* sgn) {
  if (!R.ok(off, 8)) return false;
  *cls = R.d[off] & 0x0f;
  const int bf0 = R.d[off + 1];
  *size = (int)R.uint(off + 4, 4);
  *big = (bf0 & 1) != 0;
  *sgn = *cls == 0 ? (bf0 & 0x08) != 0 : true;
  return true;
}

static bool parse_space(const Reader& R, uint64_t off, std::vector<uint64_t>* dims) {
  if (!R.ok(off, 8)) return false;
  const int ver = R.d[off], nd = R.d[off + 1];
  uint64_t p = off + (ver == 1 ? 8 : 4);
  dims->clear();
  for (int i = 0; i < nd; i++) {
    if (!R.ok(p, R.sl)) return false;
    dims->push_back(R.uint(p, R.sl));
    p += R.sl;
  }
  return true;
}

static bool parse_dataset(Reader& R, uint64_t oh, DatasetInfo* di) {
  std::vector<Msg> ms;
  if (!header_messages(R, oh, &ms)) return false;
  bool have_space = false, have_type = false;
  for (const Msg& m : ms) {
    if (m.type == 0x01) have_space = parse_space(R, m.off, &di->dims);
    if (m.type == 0x03) have_type = parse_type(R, m.off, &di->cls, &di->size, &di->big, &di->sgn);
    if (m.type == 0x08 && R.ok(m.off, 2)) {
      const int ver = R.d[m.off];
      if (ver == 3 || ver == 4) {
        di->layout = R.d[m.off + 1];
        if (di->layout == 1) {
          di->data = R.addr(R.uint(m.off + 2, R.so));
          di->data_size = R.uint(m.off + 2 + R.so, R.sl);
        } else if (di->layout == 0) {
          di->data_size = R.uint(m.off + 2, 2);
          di->data = m.off + 4;
        }
      } else if (ver == 1 || ver == 2) {  // old layout message
        const int nd = R.d[m.off + 1];
        di->layout = R.d[m.off + 2];
        if (di->layout == 1) di->data = R.addr(R.uint(m.off + 8, R.so));
        (void)nd;
      }
    }
    if (m.type == 0x0C && R.ok(m.off, 8)) {
      const int ver = R.d[m.off];
      const uint64_t nsz = R.uint(m.off + 2, 2), tsz = R.uint(m.off + 4, 2), ssz = R.uint(m.off + 6, 2);
      uint64_t p = m.off + 8 + (ver == 3 ? 1 : 0);
      auto pad = [&](uint64_t n) { return ver == 1 ? (n + 7) & ~uint64_t(7) : n; };
      DatasetInfo::Attr a;
      if (!R.ok(p, pad(nsz) + pad(tsz) + pad(ssz))) continue;
      a.name.assign(reinterpret_cast<const char*>(&R.d[p]), strnlen(reinterpret_cast<const char*>(&R.d[p]), nsz));
      p += pad(nsz);
      if (!parse_type(R, p, &a.cls, &a.size, &a.big, &a.sgn)) continue;
      p += pad(tsz) + pad(ssz);
      const uint64_t end = m.off + m.size;
      if (p > end) continue;
      a.raw.assign(R.d.begin() + p, R.d.begin() + std::min<uint64_t>(end, p + (uint64_t)a.size));
      di->attrs.push_back(a);
    }
  }
  return have_space && have_type;
}

// Element i of a numeric array as double.
static double element(const unsigned char* p, int cls, int size, bool big, bool sgn) {
  unsigned char b[8] = {0};
  for (int k = 0; k < size && k < 8; k++) b[k] = big ? p[size - 1 - k] : p[k];
  if (cls == 1) {
    if (size == 4) {
      float f;
      memcpy(&f, b, 4);
      return f;
    }
    double v;
    memcpy(&v, b, 8);
    return v;
  }
  uint64_t u = 0;
  for (int k = size - 1; k >= 0; k--) u = (u << 8) | b[k];
  if (sgn && size < 8 && (u >> (8 * size - 1)) & 1) u |= ~uint64_t(0) << (8 * size);
  return sgn ? (double)(int64_t)u : (double)u;
}

// The object header of a child `name` of the group at header oh.
static uint64_t find_child(Reader& R, uint64_t oh, const std::string& name, int depth = 0) {
  std::vector<Msg> ms;
  if (depth > 8 || !header_messages(R, oh, &ms)) return kUndef;
  for (const Msg& m : ms) {
    if (m.type == 0x11) {  // symbol table: v1 B-tree of symbol table nodes, local heap
      const uint64_t bt = R.addr(R.uint(m.off, R.so)), hp = R.addr(R.uint(m.off + R.so, R.so));
      if (!R.ok(hp, 8 + 2 * R.sl + R.so) || memcmp(&R.d[hp], "HEAP", 4) != 0) return kUndef;
      const uint64_t seg = R.addr(R.uint(hp + 8 + 2 * R.sl, R.so));
      std::vector<uint64_t> nodes = {bt};
      for (size_t i = 0; i < nodes.size() && i < 100000; i++) {
        const uint64_t n = nodes[i];
        if (!R.ok(n, 8)) return kUndef;
        if (memcmp(&R.d[n], "TREE", 4) == 0) {
          const int level = R.d[n + 5];
          const uint64_t used = R.uint(n + 6, 2);
          uint64_t p = n + 8 + 2 * R.so + R.sl;  // past the header and key 0
          for (uint64_t c = 0; c < used; c++) {
            if (!R.ok(p, R.so + R.sl)) return kUndef;
            nodes.push_back(R.addr(R.uint(p, R.so)));
            p += R.so + R.sl;
          }
          (void)level;
        } else if (memcmp(&R.d[n], "SNOD", 4) == 0) {
          const uint64_t cnt = R.uint(n + 6, 2);
          uint64_t p = n + 8;
          for (uint64_t c = 0; c < cnt; c++) {
            if (!R.ok(p, 2 * R.so + 24)) return kUndef;
            const uint64_t no = R.uint(p, R.so), ohc = R.addr(R.uint(p + R.so, R.so));
            if (R.ok(seg + no, 1)) {
              const char* s = reinterpret_cast<const char*>(&R.d[seg + no]);
              if (name == std::string(s, strnlen(s, R.d.size() - (seg + no)))) return ohc;
            }
            p += 2 * R.so + 24;
          }
        }
      }
    }
    if (m.type == 0x06 && R.ok(m.off, 4)) {  // link message (compact groups)
      const int flags = R.d[m.off + 1];
      uint64_t p = m.off + 2;
      int ltype = 0;
      if (flags & 0x08) ltype = R.d[p++];
      if (flags & 0x04) p += 8;
      if (flags & 0x10) p++;
      const int lsz = 1 << (flags & 3);
      const uint64_t nlen = R.uint(p, lsz);
      p += lsz;
      if (!R.ok(p, nlen + R.so)) continue;
      if (ltype == 0 && name == std::string(reinterpret_cast<const char*>(&R.d[p]), nlen))
        return R.addr(R.uint(p + nlen, R.so));
    }
  }
  return kUndef;
}

static epet_status open_file(const char* path, Reader* R, uint64_t* root) {
  if (!path) return set_error(EPET_ERR_INVALID, "path is NULL");
  FILE* f = fopen(path, "rb");
  if (!f) return set_error(EPET_ERR_INVALID, "cannot open %s", path);
  fseek(f, 0, SEEK_END);
  const long n = ftell(f);
  fseek(f, 0, SEEK_SET);
  R->d.resize(n > 0 ? (size_t)n : 0);
  const size_t got = n > 0 ? fread(R->d.data(), 1, (size_t)n, f) : 0;
  fclose(f);
  if ((long)got != n) return set_error(EPET_ERR_INVALID, "cannot read %s", path);
  for (uint64_t off = 0; off + 8 <= R->d.size(); off = off ? off * 2 : 512) {
    if (memcmp(&R->d[off], kSig, 8) != 0) continue;
    R->base = off;
    const int ver = R->d[off + 8];
    if (ver <= 1) {
      R->so = R->d[off + 13];
      R->sl = R->d[off + 14];
      uint64_t p = off + 24 + (ver == 1 ? 4 : 0) + 4 * R->so;  // root symbol table entry
      if (!R->ok(p, 2 * R->so)) break;
      *root = R->addr(R->uint(p + R->so, R->so));
    } else {
      R->so = R->d[off + 9];
      R->sl = R->d[off + 10];
      *root = R->addr(R->uint(off + 12 + 3 * R->so, R->so));
    }
    if ((R->so != 4 && R->so != 8) || (R->sl != 4 && R->sl != 8))
      return set_error(EPET_ERR_UNSUPPORTED, "%s: offset/length sizes %d/%d", path, R->so, R->sl);
    return EPET_OK;
  }
  return set_error(EPET_ERR_INVALID, "%s is not an HDF5 file", path);
}

static epet_status open_dataset(const char* path, const char* name, Reader* R, DatasetInfo* di) {
  uint64_t root = kUndef;
  H5_CHECK(open_file(path, R, &root));
  if (!name) return set_error(EPET_ERR_INVALID, "dataset name is NULL");
  uint64_t oh = root;
  std::string s(name);
  size_t pos = 0;
  while (pos <= s.size()) {  // path components separated by '/'
    size_t q = s.find('/', pos);
    if (q == std::string::npos) q = s.size();
    const std::string part = s.substr(pos, q - pos);
    if (!part.empty()) {
      oh = find_child(*R, oh, part);
      if (oh == kUndef) return set_error(EPET_ERR_INVALID, "%s: no object \"%s\"", path, name);
    }
    pos = q + 1;
  }
  if (!parse_dataset(*R, oh, di))
    return set_error(EPET_ERR_UNSUPPORTED, "%s: \"%s\" is not a dataset this reader handles", path,
                     name);
  if (di->cls != 0 && di->cls != 1)
    return set_error(EPET_ERR_UNSUPPORTED, "%s: \"%s\": element class %d (numbers only)", path,
                     name, di->cls);
  if (di->cls == 0 && (di->size < 1 || di->size > 8))
    return set_error(EPET_ERR_UNSUPPORTED, "%s: \"%s\": %d-byte integers", path, name, di->size);
  if (di->cls == 1 && di->size != 4 && di->size != 8)
    return set_error(EPET_ERR_UNSUPPORTED, "%s: \"%s\": %d-byte floats", path, name, di->size);
  if (di->layout != 0 && di->layout != 1)
    return set_error(EPET_ERR_UNSUPPORTED,
                     "%s: \"%s\": storage layout %d (contiguous or compact only)", path, name,
                     di->layout);
  return EPET_OK;
}

static uint64_t count(const DatasetInfo& di) {
  uint64_t n = 1;
  for (uint64_t v : di.dims) n *= v;
  return n;
}

// ------------------------------------------------------------------ writing

struct Writer {
  std::vector<unsigned char> d;
  void put(uint64_t off, uint64_t v, int n) {
    if (d.size() < off + n) d.resize(off + n, 0);
    for (int i = 0; i < n; i++) d[off + i] = (unsigned char)(v >> (8 * i));
  }
  uint64_t alloc(uint64_t n) {  // 8-byte aligned
    const uint64_t off = (d.size() + 7) & ~uint64_t(7);
    d.resize(off + n, 0);
    return off;
  }
};

struct AttrOut {
  std::string name;
  bool is_float;
  uint32_t bits;
};

// A version-1 header message: type, size, flags, data (padded to 8).
static void message(std::vector<unsigned char>* m, int type, const std::vector<unsigned char>& data) {
  const size_t sz = (data.size() + 7) & ~size_t(7);
  const size_t o = m->size();
  m->resize(o + 8 + sz, 0);
  (*m)[o] = (unsigned char)type;
  (*m)[o + 1] = (unsigned char)(type >> 8);
  (*m)[o + 2] = (unsigned char)sz;
  (*m)[o + 3] = (unsigned char)(sz >> 8);
  (*m)[o + 4] = type == 0x03 ? 1 : 0;  // the datatype message is constant
  memcpy(m->data() + o + 8, data.data(), data.size());
}

static void le(std::vector<unsigned char>* v, uint64_t x, int n) {
  for (int i = 0; i < n; i++) v->push_back((unsigned char)(x >> (8 * i)));
}

// Datatype: IEEE little-endian float32, or little-endian signed int32.
static std::vector<unsigned char> type_msg(bool is_float) {
  std::vector<unsigned char> t;
  if (is_float) {
    t = {0x11, 0x20, 0x1f, 0x00};  // version 1, class 1; LE, IEEE normalization, sign at bit 31
    le(&t, 4, 4);
    le(&t, 0, 2);   // bit offset
    le(&t, 32, 2);  // precision
    t.push_back(23);  // exponent location
    t.push_back(8);   // exponent size
    t.push_back(0);   // mantissa location
    t.push_back(23);  // mantissa size
    le(&t, 127, 4);   // exponent bias
  } else {
    t = {0x10, 0x08, 0x00, 0x00};  // version 1, class 0; LE, signed
    le(&t, 4, 4);
    le(&t, 0, 2);
    le(&t, 32, 2);
  }
  return t;
}

// Dataspace version 1: simple (or scalar with no dims).
static std::vector<unsigned char> space_msg(const std::vector<uint64_t>& dims) {
  std::vector<unsigned char> s = {1, (unsigned char)dims.size(), 0, 0, 0, 0, 0, 0};
  for (uint64_t v : dims) le(&s, v, 8);
  return s;
}

// A file whose root group holds one float32 dataset `name` of shape dims,
// with the given scalar attributes.
static epet_status write_file(const char* path, const char* name, const float* data,
                              const std::vector<uint64_t>& dims, const std::vector<AttrOut>& attrs) {
  if (!path || !name || strlen(name) == 0 || strchr(name, '/'))
    return set_error(EPET_ERR_INVALID, "bad path or dataset name");
  uint64_t n = 1;
  for (uint64_t v : dims) n *= v;
  if (n > 0 && !data) return set_error(EPET_ERR_INVALID, "data is NULL");
  Writer W;
  W.d.resize(96, 0);  // superblock version 0
  memcpy(W.d.data(), kSig, 8);
  W.put(13, 8, 1);  // size of offsets
  W.put(14, 8, 1);  // size of lengths
  W.put(16, 4, 2);  // group leaf node K
  W.put(18, 16, 2); // group internal node K
  W.put(24, 0, 8);  // base address
  W.put(32, kUndef, 8);  // free-space info
  W.put(48, kUndef, 8);  // driver information block
  // local heap of the root group: "" at 0, the dataset's name at 8, then one
  // free block (next-free offset 1 = end of the list, as libhdf5 writes it;
  // libhdf5 rejects the undefined address there)
  const size_t nlen = strlen(name) + 1;
  const uint64_t used = 8 + ((nlen + 7) & ~size_t(7));
  const uint64_t seg_size = used + 16;
  const uint64_t heap = W.alloc(32);
  const uint64_t seg = W.alloc(seg_size);
  memcpy(&W.d[seg + 8], name, nlen - 1);
  W.put(seg + used, 1, 8);
  W.put(seg + used + 8, seg_size - used, 8);
  memcpy(&W.d[heap], "HEAP", 4);
  W.put(heap + 8, seg_size, 8);
  W.put(heap + 16, used, 8);  // the free block
  W.put(heap + 24, seg, 8);
  // symbol table node (2 * leaf K = 8 entries) with the one entry
  const uint64_t snod = W.alloc(8 + 8 * 40);
  memcpy(&W.d[snod], "SNOD", 4);
  W.put(snod + 4, 1, 1);
  W.put(snod + 6, 1, 2);
  // group B-tree node (2 * internal K keys + children), one child
  const uint64_t tree = W.alloc(24 + 33 * 8 + 32 * 8);
  memcpy(&W.d[tree], "TREE", 4);
  W.put(tree + 4, 0, 1);  // group node
  W.put(tree + 5, 0, 1);  // leaf level
  W.put(tree + 6, 1, 2);
  W.put(tree + 8, kUndef, 8);
  W.put(tree + 16, kUndef, 8);
  W.put(tree + 24, 0, 8);     // key 0: ""
  W.put(tree + 32, snod, 8);  // child 0
  W.put(tree + 40, 8, 8);     // key 1: the name
  // root group object header: the symbol table message
  std::vector<unsigned char> rm;
  {
    std::vector<unsigned char> st;
    le(&st, tree, 8);
    le(&st, heap, 8);
    message(&rm, 0x11, st);
  }
  const uint64_t root = W.alloc(16 + rm.size());
  W.put(root, 1, 1);
  W.put(root + 2, 1, 2);  // messages
  W.put(root + 4, 1, 4);  // reference count
  W.put(root + 8, rm.size(), 4);
  memcpy(&W.d[root + 16], rm.data(), rm.size());
  // the dataset's object header and data
  std::vector<unsigned char> dm;
  message(&dm, 0x01, space_msg(dims));
  message(&dm, 0x03, type_msg(true));
  message(&dm, 0x05, {2, 2, 2, 0});  // fill value v2: late allocation, write if set, undefined
  const uint64_t data_off_slot_msg = dm.size();
  {
    std::vector<unsigned char> lay = {3, 1};  // version 3, contiguous
    le(&lay, 0, 8);
    le(&lay, n * 4, 8);
    message(&dm, 0x08, lay);
  }
  for (const AttrOut& a : attrs) {
    std::vector<unsigned char> at = {1, 0};
    const std::vector<unsigned char> t = type_msg(a.is_float), sp = space_msg({});
    le(&at, a.name.size() + 1, 2);
    le(&at, t.size(), 2);
    le(&at, sp.size(), 2);
    std::vector<unsigned char> nm(a.name.begin(), a.name.end());
    nm.resize((a.name.size() + 1 + 7) & ~size_t(7), 0);
    at.insert(at.end(), nm.begin(), nm.end());
    std::vector<unsigned char> tp = t;
    tp.resize((t.size() + 7) & ~size_t(7), 0);
    at.insert(at.end(), tp.begin(), tp.end());
    at.insert(at.end(), sp.begin(), sp.end());  // 8 bytes: already padded
    le(&at, a.bits, 4);
    message(&dm, 0x0C, at);
  }
  const uint64_t oh = W.alloc(16 + dm.size());
  W.put(oh, 1, 1);
  W.put(oh + 2, 4 + attrs.size(), 2);
  W.put(oh + 4, 1, 4);
  W.put(oh + 8, dm.size(), 4);
  memcpy(&W.d[oh + 16], dm.data(), dm.size());
  const uint64_t raw = W.alloc(n * 4);
  if (n > 0) memcpy(&W.d[raw], data, n * 4);  // float32 little-endian hosts (x86_64, aarch64)
  W.put(oh + 16 + data_off_slot_msg + 8 + 2, raw, 8);  // the layout message's address
  // the dataset's symbol table entry; the root's entry in the superblock
  W.put(snod + 8, 8, 8);
  W.put(snod + 16, oh, 8);
  W.put(56 + 0, 0, 8);  // (superblock) root entry: link name offset ""
  W.put(64, root, 8);
  W.put(72, 1, 4);      // cache type 1: the symbol table's addresses in the scratch pad
  W.put(80, tree, 8);
  W.put(88, heap, 8);
  W.put(40, W.d.size(), 8);  // end-of-file address
  FILE* f = fopen(path, "wb");
  if (!f) return set_error(EPET_ERR_INVALID, "cannot create %s", path);
  const size_t wrote = fwrite(W.d.data(), 1, W.d.size(), f);
  const int cl = fclose(f);
  if (wrote != W.d.size() || cl != 0) return set_error(EPET_ERR_INVALID, "cannot write %s", path);
  return EPET_OK;
}

static uint32_t fbits(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}

}  // namespace h5
}  // namespace epet

using namespace epet;
using namespace epet::h5;

extern "C" {

epet_status epet_h5_dataset_shape(const char* path, const char* name, int32_t* ndims_h,
                                  int64_t* dims_h) {
  Reader R;
  DatasetInfo di;
  H5_CHECK(open_dataset(path, name, &R, &di));
  if (di.dims.size() > 8) return set_error(EPET_ERR_UNSUPPORTED, "more than 8 dimensions");
  if (ndims_h) *ndims_h = (int32_t)di.dims.size();
  if (dims_h)
    for (size_t i = 0; i < di.dims.size(); i++) dims_h[i] = (int64_t)di.dims[i];
  return EPET_OK;
}

epet_status epet_h5_read_f32(const char* path, const char* name, float* out_h, int64_t n) {
  Reader R;
  DatasetInfo di;
  H5_CHECK(open_dataset(path, name, &R, &di));
  const uint64_t cnt = count(di);
  if (n < 0 || (uint64_t)n != cnt)
    return set_error(EPET_ERR_CAPACITY, "%s: \"%s\" holds %llu elements, %lld given", path, name,
                     (unsigned long long)cnt, (long long)n);
  if (cnt > 0 && !out_h) return set_error(EPET_ERR_INVALID, "out is NULL");
  if (cnt > 0 && (di.data == kUndef || !R.ok(di.data, cnt * (uint64_t)di.size)))
    return set_error(EPET_ERR_INVALID, "%s: \"%s\": data outside the file", path, name);
  for (uint64_t i = 0; i < cnt; i++)
    out_h[i] = (float)element(&R.d[di.data + i * di.size], di.cls, di.size, di.big, di.sgn);
  return EPET_OK;
}

epet_status epet_h5_read_measurement(const char* path, int32_t* rows_h, float* y_h,
                                     int64_t capacity, int64_t* m_h, int64_t* nchannels_h) {
  Reader R;
  DatasetInfo di;
  H5_CHECK(open_dataset(path, "messung", &R, &di));
  const uint64_t cnt = count(di);
  if (cnt > (uint64_t)INT32_MAX)
    return set_error(EPET_ERR_UNSUPPORTED, "%s: %llu channels (int32 row ids)", path,
                     (unsigned long long)cnt);
  if (cnt > 0 && (di.data == kUndef || !R.ok(di.data, cnt * (uint64_t)di.size)))
    return set_error(EPET_ERR_INVALID, "%s: \"messung\": data outside the file", path);
  int64_t m = 0;
  for (uint64_t i = 0; i < cnt; i++) {
    const float v = (float)element(&R.d[di.data + i * di.size], di.cls, di.size, di.big, di.sgn);
    if (v == 0.f) continue;
    if (rows_h && y_h && m < capacity) {
      rows_h[m] = (int32_t)i;
      y_h[m] = v;
    }
    m++;
  }
  if (m_h) *m_h = m;
  if (nchannels_h) *nchannels_h = (int64_t)cnt;
  if (rows_h && y_h && m > capacity)
    return set_error(EPET_ERR_CAPACITY, "%s: %lld measured channels, capacity %lld", path,
                     (long long)m, (long long)capacity);
  return EPET_OK;
}

epet_status epet_h5_write_measurement(const char* path, const float* y_h, int64_t n) {
  if (n < 0) return set_error(EPET_ERR_INVALID, "n < 0");
  return write_file(path, "messung", y_h, {(uint64_t)n}, {});
}

static epet_status write_density(const char* path, const float* x_h, const epet_grid* g,
                                 int64_t iteration) {
  if (!g) return set_error(EPET_ERR_INVALID, "grid is NULL");
  if (iteration > INT32_MAX) return set_error(EPET_ERR_INVALID, "iteration over 2^31");
  std::vector<AttrOut> at;
  const char* ax[3] = {"x", "y", "z"};
  float mx[3];
  for (int d = 0; d < 3; d++) {
    if (g->n[d] < 1) return set_error(EPET_ERR_INVALID, "grid counts must be >= 1");
    mx[d] = g->o[d] + (float)g->n[d] * g->d[d];  // as H5DensityWriter.hpp:131-132
  }
  for (int d = 0; d < 3; d++) at.push_back({std::string(ax[d]) + "min", true, fbits(g->o[d])});
  for (int d = 0; d < 3; d++) at.push_back({std::string(ax[d]) + "max", true, fbits(mx[d])});
  for (int d = 0; d < 3; d++) at.push_back({std::string(ax[d]) + "nbin", false, (uint32_t)g->n[d]});
  if (iteration >= 0) at.push_back({"iteration", false, (uint32_t)iteration});
  return write_file(path, "density", x_h,
                    {(uint64_t)g->n[0], (uint64_t)g->n[1], (uint64_t)g->n[2]}, at);
}

epet_status epet_h5_write_density(const char* path, const float* x_h, const epet_grid* g) {
  return write_density(path, x_h, g, -1);
}

epet_status epet_h5_write_checkpoint(const char* path, const float* x_h, const epet_grid* g,
                                     int64_t iteration) {
  if (iteration < 0) return set_error(EPET_ERR_INVALID, "iteration < 0");
  return write_density(path, x_h, g, iteration);
}

epet_status epet_h5_read_attribute(const char* path, const char* name, const char* attr,
                                   double* value_h) {
  Reader R;
  DatasetInfo di;
  H5_CHECK(open_dataset(path, name, &R, &di));
  if (!attr) return set_error(EPET_ERR_INVALID, "attribute name is NULL");
  for (const DatasetInfo::Attr& a : di.attrs)
    if (a.name == attr && (int)a.raw.size() >= a.size && (a.cls == 0 || a.cls == 1)) {
      if (value_h) *value_h = element(a.raw.data(), a.cls, a.size, a.big, a.sgn);
      return EPET_OK;
    }
  return set_error(EPET_ERR_INVALID, "%s: \"%s\" has no numeric attribute %s", path, name, attr);
}

epet_status epet_h5_read_density(const char* path, float* x_h, int64_t n, epet_grid* g_h) {
  Reader R;
  DatasetInfo di;
  H5_CHECK(open_dataset(path, "density", &R, &di));
  if (di.dims.size() != 3)
    return set_error(EPET_ERR_INVALID, "%s: \"density\" has %zu dimensions", path, di.dims.size());
  if (g_h) {
    double v[9];
    const char* names[9] = {"xmin", "ymin", "zmin", "xmax", "ymax", "zmax",
                            "xnbin", "ynbin", "znbin"};
    for (int k = 0; k < 9; k++) {
      bool found = false;
      for (const DatasetInfo::Attr& a : di.attrs)
        if (a.name == names[k] && (int)a.raw.size() >= a.size) {
          v[k] = element(a.raw.data(), a.cls, a.size, a.big, a.sgn);
          found = true;
        }
      if (!found) return set_error(EPET_ERR_INVALID, "%s: attribute %s missing", path, names[k]);
    }
    for (int d = 0; d < 3; d++) {
      g_h->n[d] = (int32_t)v[6 + d];
      g_h->o[d] = (float)v[d];
      g_h->d[d] = g_h->n[d] > 0 ? (float)((v[3 + d] - v[d]) / v[6 + d]) : 0.f;
      if ((uint64_t)g_h->n[d] != di.dims[d])
        return set_error(EPET_ERR_INVALID, "%s: %cnbin %d != dimension %llu", path, "xyz"[d],
                         g_h->n[d], (unsigned long long)di.dims[d]);
    }
  }
  return x_h ? epet_h5_read_f32(path, "density", x_h, n) : EPET_OK;
}

}  // extern "C"
