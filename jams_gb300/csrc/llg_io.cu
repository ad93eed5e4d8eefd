// Array files in the two formats the reference reads spins and per-spin
// parameters from (src/jams/helpers/load.h:14-60, used by init_h5,
// src/jams/initializer/init_h5.cc:10-34) and writes them in (the HDF5
// monitor, src/jams/monitors/hdf5.cc:94-150, 292-307):
//
//  * ".h5": HDF5.  The writer emits the file the HDF5 library writes for
//    `createDataSet<double>(name, {rows, cols})` without chunking or
//    compression: version-0 superblock, root group as a symbol table
//    (v1 B-tree + local heap), one version-1 object header per dataset with
//    dataspace, IEEE float64 little-endian datatype, fill-value and
//    contiguous layout messages, then the raw rows.  The reader follows the
//    HDF5 File Format Specification (superblock versions 0-3, symbol-table
//    and compact link-message groups, object header versions 1 and 2 with
//    continuation blocks, contiguous, compact or chunked float32/float64
//    datasets).  Chunked datasets are read through their version-1 B-tree,
//    with the deflate and shuffle filters of the monitor's "compressed"
//    option undone by this file's own zlib decoder.  Version-4 chunk
//    indexes, other filters and dense link storage are rejected with an
//    error.
//  * anything else: whitespace-separated text, '#' or '//' comment lines,
//    every number read in file order.
//
// Host code only; no device work.
#include <algorithm>
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <exception>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "llg_io.h"

namespace llgio {
namespace {

constexpr uint64_t kUndef = ~0ull;

std::string extension(const std::string& path) {
  const size_t dot = path.find_last_of('.');
  return dot == std::string::npos ? std::string() : path.substr(dot + 1);
}

std::string strip_slash(const char* name) {
  std::string s = name ? name : "";
  while (!s.empty() && s[0] == '/') s.erase(0, 1);
  return s;
}

// ------------------------------------------------------------------ text --

// A line is a comment when its first non-blank character is '#', its first
// two are "//", or it holds fewer than two non-blank characters
// (src/jams/helpers/utils.h:115-126).
bool line_is_comment(const std::string& line) {
  std::istringstream ss(line);
  char c0 = 0, c1 = 0;
  ss >> c0;
  ss >> c1;
  return !ss || c0 == '#' || (c0 == '/' && c1 == '/');
}

int read_text(const std::string& path, std::vector<double>& out, std::string& err) {
  std::ifstream f(path);
  if (!f.is_open()) {
    err = "failed to open file: " + path;
    return 1;
  }
  out.clear();
  for (std::string line; std::getline(f, line);) {
    if (line.empty() || line_is_comment(line)) continue;
    // one value per extraction attempt while the stream is good, as the
    // reference counts them (a failed extraction counts and reads as 0)
    std::istringstream is(line);
    while (is.good()) {
      double v = 0.0;
      is >> v;
      out.push_back(v);
    }
  }
  return 0;
}

int write_text(const std::string& path, const double* data, int64_t rows, int64_t cols, std::string& err) {
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) {
    err = "failed to open file for writing: " + path + ": " + std::strerror(errno);
    return 1;
  }
  for (int64_t r = 0; r < rows; ++r) {
    for (int64_t c = 0; c < cols; ++c) std::fprintf(f, c ? " %.17g" : "%.17g", data[r * cols + c]);
    std::fputc('\n', f);
  }
  const bool ok = std::fflush(f) == 0 && !std::ferror(f);
  std::fclose(f);
  if (!ok) {
    err = "failed writing " + path;
    return 1;
  }
  return 0;
}

// ------------------------------------------------------------ HDF5 write --

struct Out {
  std::vector<uint8_t> b;
  void u8(uint64_t v) { b.push_back((uint8_t)v); }
  void u16(uint64_t v) { for (int i = 0; i < 2; ++i) u8(v >> (8 * i)); }
  void u32(uint64_t v) { for (int i = 0; i < 4; ++i) u8(v >> (8 * i)); }
  void u64(uint64_t v) { for (int i = 0; i < 8; ++i) u8(v >> (8 * i)); }
  void zeros(size_t n) { b.insert(b.end(), n, 0); }
  void bytes(const void* p, size_t n) { b.insert(b.end(), (const uint8_t*)p, (const uint8_t*)p + n); }
  void pad8() { while (b.size() % 8) u8(0); }
  void put64(size_t at, uint64_t v) { for (int i = 0; i < 8; ++i) b[at + i] = (uint8_t)(v >> (8 * i)); }
};

constexpr int kLeafK = 4;       // group leaf node K: a symbol node holds 2K entries
constexpr int kInternalK = 16;  // group internal node K: a B-tree node holds 2K children

// version-1 object header message: type, size (padded to 8), flags
void message(Out& o, int type, const Out& body, int flags) {
  o.u16(type);
  o.u16((body.b.size() + 7) / 8 * 8);
  o.u8(flags);
  o.zeros(3);
  o.bytes(body.b.data(), body.b.size());
  o.pad8();
}

int write_h5(const std::string& path, const std::vector<Dataset>& sets, std::string& err) {
  if (sets.empty() || (int)sets.size() > 2 * kLeafK) {
    err = "HDF5 writer: 1 to 8 datasets per file";
    return 1;
  }
  // names in strcmp order (the order of a group's symbol node)
  std::vector<int> order(sets.size());
  for (size_t i = 0; i < sets.size(); ++i) order[i] = (int)i;
  for (size_t i = 1; i < order.size(); ++i)
    for (size_t j = i; j > 0 && sets[order[j]].name < sets[order[j - 1]].name; --j) std::swap(order[j], order[j - 1]);
  for (size_t i = 0; i < sets.size(); ++i) {
    if (sets[i].name.empty() || sets[i].name.find('/') != std::string::npos) {
      err = "HDF5 writer: dataset names are plain names in the root group";
      return 1;
    }
    if (i && sets[order[i]].name == sets[order[i - 1]].name) {
      err = "HDF5 writer: duplicate dataset name " + sets[order[i]].name;
      return 1;
    }
  }
  // local heap data: "" at 0, then each name, 8-byte padded
  Out heap;
  heap.zeros(8);
  std::vector<uint64_t> name_off(sets.size());
  for (int k : order) {
    name_off[k] = heap.b.size();
    heap.bytes(sets[k].name.c_str(), sets[k].name.size() + 1);
    heap.pad8();
  }

  const uint64_t a_root = 96;                              // root object header (16 + 24)
  const uint64_t a_heap = a_root + 40;                     // local heap header (32) + data
  const uint64_t a_tree = a_heap + 32 + heap.b.size();     // B-tree node
  const uint64_t tree_size = 24 + (2 * kInternalK + 1) * 8 + 2 * kInternalK * 8;
  const uint64_t a_snod = a_tree + tree_size;              // symbol node
  const uint64_t snod_size = 8 + 2 * kLeafK * 40;
  uint64_t a = a_snod + snod_size;
  std::vector<uint64_t> a_head(sets.size()), a_data(sets.size());
  constexpr uint64_t kHeadSize = 16 + 4 * 8 + 24 + 24 + 8 + 24;
  for (size_t i = 0; i < sets.size(); ++i) {
    a_head[i] = a;
    a += kHeadSize;
  }
  for (size_t i = 0; i < sets.size(); ++i) {
    a_data[i] = a;
    a += (uint64_t)sets[i].rows * sets[i].cols * 8;
  }
  const uint64_t eof = a;

  Out o;
  // superblock, version 0
  const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
  o.bytes(sig, 8);
  o.u8(0);  // superblock version
  o.u8(0);  // free-space storage version
  o.u8(0);  // root group symbol table entry version
  o.u8(0);
  o.u8(0);  // shared header message format version
  o.u8(8);  // size of offsets
  o.u8(8);  // size of lengths
  o.u8(0);
  o.u16(kLeafK);
  o.u16(kInternalK);
  o.u32(0);       // file consistency flags
  o.u64(0);       // base address
  o.u64(kUndef);  // free-space info
  o.u64(eof);     // end of file address
  o.u64(kUndef);  // driver information block
  // root group symbol table entry: name offset, header, cache type 1 with
  // the B-tree and heap addresses in the scratch pad
  o.u64(0);
  o.u64(a_root);
  o.u32(1);
  o.u32(0);
  o.u64(a_tree);
  o.u64(a_heap);
  // root object header, version 1: one symbol table message
  {
    Out m;
    m.u64(a_tree);
    m.u64(a_heap);
    o.u8(1);
    o.u8(0);
    o.u16(1);   // messages
    o.u32(1);   // reference count
    o.u32(24);  // header data size
    o.zeros(4);
    message(o, 0x11, m, 0);
  }
  // local heap
  o.bytes("HEAP", 4);
  o.u8(0);
  o.zeros(3);
  o.u64(heap.b.size());
  o.u64(kUndef);  // no free block
  o.u64(a_heap + 32);
  o.bytes(heap.b.data(), heap.b.size());
  // B-tree node (group, leaf level): one child, the symbol node
  {
    const size_t start = o.b.size();
    o.bytes("TREE", 4);
    o.u8(0);  // node type: group
    o.u8(0);  // level
    o.u16(1);
    o.u64(kUndef);
    o.u64(kUndef);
    o.u64(0);                              // key 0: the empty name
    o.u64(a_snod);                         // child 0
    o.u64(name_off[order.back()]);         // key 1: the last name in the child
    o.zeros(tree_size - (o.b.size() - start));
  }
  // symbol node
  {
    const size_t start = o.b.size();
    o.bytes("SNOD", 4);
    o.u8(1);
    o.u8(0);
    o.u16(sets.size());
    for (int k : order) {
      o.u64(name_off[k]);
      o.u64(a_head[k]);
      o.u32(0);  // cache type: none
      o.u32(0);
      o.zeros(16);
    }
    o.zeros(snod_size - (o.b.size() - start));
  }
  // dataset object headers, version 1
  for (size_t i = 0; i < sets.size(); ++i) {
    const size_t start = o.b.size();
    o.u8(1);
    o.u8(0);
    o.u16(4);
    o.u32(1);
    o.u32(kHeadSize - 16);
    o.zeros(4);
    Out ds;  // dataspace, version 1, rank 2, no maximum dimensions
    ds.u8(1);
    ds.u8(2);
    ds.u8(0);
    ds.u8(0);
    ds.u32(0);
    ds.u64(sets[i].rows);
    ds.u64(sets[i].cols);
    message(o, 0x01, ds, 0);
    Out dt;  // IEEE float64 little-endian
    dt.u8(0x11);   // version 1, class 1 (floating point)
    dt.u8(0x20);   // little-endian, mantissa normalisation: implied msb
    dt.u8(63);     // sign bit location
    dt.u8(0);
    dt.u32(8);     // size
    dt.u16(0);     // bit offset
    dt.u16(64);    // bit precision
    dt.u8(52);     // exponent location
    dt.u8(11);     // exponent size
    dt.u8(0);      // mantissa location
    dt.u8(52);     // mantissa size
    dt.u32(1023);  // exponent bias
    message(o, 0x03, dt, 1);
    Out fv;  // fill value, version 2: late allocation, write if set, undefined
    fv.u8(2);
    fv.u8(2);
    fv.u8(2);
    fv.u8(0);
    message(o, 0x05, fv, 1);
    Out ly;  // layout, version 3, contiguous
    ly.u8(3);
    ly.u8(1);
    ly.u64(a_data[i]);
    ly.u64((uint64_t)sets[i].rows * sets[i].cols * 8);
    message(o, 0x08, ly, 0);
    if (o.b.size() - start != kHeadSize) {
      err = "HDF5 writer: internal header size mismatch";
      return 1;
    }
  }
  if (o.b.size() != a_data[0]) {
    err = "HDF5 writer: internal layout mismatch";
    return 1;
  }
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) {
    err = "failed to open file for writing: " + path + ": " + std::strerror(errno);
    return 1;
  }
  bool ok = std::fwrite(o.b.data(), 1, o.b.size(), f) == o.b.size();
  for (size_t i = 0; i < sets.size() && ok; ++i) {
    // raw data: little-endian doubles, row-major
    const int64_t n = sets[i].rows * sets[i].cols;
    std::vector<uint8_t> buf((size_t)std::min<int64_t>(n, 1 << 16) * 8);
    for (int64_t j0 = 0; j0 < n && ok; j0 += 1 << 16) {
      const int64_t m = std::min<int64_t>(n - j0, 1 << 16);
      for (int64_t j = 0; j < m; ++j) {
        uint64_t u;
        std::memcpy(&u, &sets[i].data[j0 + j], 8);
        for (int b = 0; b < 8; ++b) buf[j * 8 + b] = (uint8_t)(u >> (8 * b));
      }
      ok = std::fwrite(buf.data(), 8, (size_t)m, f) == (size_t)m;
    }
  }
  ok = ok && std::fflush(f) == 0;
  std::fclose(f);
  if (!ok) {
    err = "failed writing " + path;
    return 1;
  }
  return 0;
}

// ------------------------------------------------------------- HDF5 read --

struct File {
  std::vector<uint8_t> d;
  int so = 8, sl = 8;  // size of offsets / lengths
  uint64_t base = 0;
  std::string err;
  // a field read outside the file (a corrupt offset or length): the read
  // gives 0 and the parse fails once the flag is seen
  mutable bool oob = false;

  bool in(uint64_t at, uint64_t n) const { return at <= d.size() && n <= d.size() - at; }
  uint8_t u8(uint64_t at) const {
    if (at >= d.size()) {
      oob = true;
      return 0;
    }
    return d[at];
  }
  uint64_t uint(uint64_t at, int n) const {
    if (!in(at, (uint64_t)n)) {
      oob = true;
      return 0;
    }
    uint64_t v = 0;
    for (int i = 0; i < n; ++i) v |= (uint64_t)d[at + i] << (8 * i);
    return v;
  }
  uint64_t addr(uint64_t at) const {
    const uint64_t v = uint(at, so);
    return (so < 8 && v == ((1ull << (8 * so)) - 1)) ? kUndef : v;
  }
  bool fail(const std::string& m) {
    if (err.empty()) err = m;
    return false;
  }
};

struct Message {
  int type;
  uint64_t at, size;
};

// messages of an object header (versions 1 and 2) and its continuation blocks
bool header_messages(File& F, uint64_t at, std::vector<Message>& msgs) {
  at += F.base;
  if (!F.in(at, 16)) return F.fail("object header outside the file");
  std::vector<std::pair<uint64_t, uint64_t>> blocks;  // (start, end) of message data
  int version = 0, flags = 0;
  if (std::memcmp(&F.d[at], "OHDR", 4) == 0) {
    version = 2;
    flags = F.d[at + 5];
    uint64_t p = at + 6;
    if (flags & 0x20) p += 16;  // times
    if (flags & 0x10) p += 4;   // attribute phase change values
    const int csz = 1 << (flags & 3);
    if (!F.in(p, csz)) return F.fail("truncated object header");
    const uint64_t size0 = F.uint(p, csz);
    p += csz;
    blocks.push_back({p, p + size0});
  } else if (F.d[at] == 1) {
    version = 1;
    const uint64_t size0 = F.uint(at + 8, 4);
    blocks.push_back({at + 16, at + 16 + size0});
  } else {
    return F.fail("unsupported object header version");
  }
  for (size_t bi = 0; bi < blocks.size(); ++bi) {
    uint64_t p = blocks[bi].first;
    const uint64_t end = blocks[bi].second;
    if (!F.in(p, end - p)) return F.fail("object header block outside the file");
    if (blocks.size() > 64) return F.fail("too many object header continuation blocks");
    while (true) {
      const uint64_t hsz = version == 1 ? 8 : ((flags & 0x04) ? 6 : 4);
      if (p + hsz > end) break;
      int type;
      uint64_t size;
      if (version == 1) {
        type = (int)F.uint(p, 2);
        size = F.uint(p + 2, 2);
      } else {
        type = F.d[p];
        size = F.uint(p + 1, 2);
      }
      const uint64_t data = p + hsz;
      if (data + size > end) return F.fail("object header message overruns its block");
      if (type == 0x10) {  // continuation: address, length
        const uint64_t ca = F.addr(data) + F.base, cl = F.uint(data + F.so, F.sl);
        if (version == 1) {
          blocks.push_back({ca, ca + cl});
        } else {
          if (!F.in(ca, 4) || std::memcmp(&F.d[ca], "OCHK", 4) != 0) return F.fail("bad continuation block");
          blocks.push_back({ca + 4, ca + cl - 4});  // minus the checksum
        }
      } else if (type != 0) {
        msgs.push_back({type, data, size});
      }
      p = data + size;
    }
  }
  if (F.oob) return F.fail("object header field outside the file");
  return true;
}

bool find_in_symbol_table(File& F, uint64_t btree, uint64_t heap, const std::string& name, uint64_t& header,
                          int depth) {
  if (depth > 32) return F.fail("group B-tree too deep");
  heap += F.base;
  btree += F.base;
  if (!F.in(heap, 8 + 2 * F.sl + F.so) || std::memcmp(&F.d[heap], "HEAP", 4) != 0) return F.fail("bad local heap");
  const uint64_t heap_data = F.addr(heap + 8 + 2 * F.sl) + F.base;
  const uint64_t heap_size = F.uint(heap + 8, F.sl);
  if (!F.in(btree, 8 + 2 * F.so) || std::memcmp(&F.d[btree], "TREE", 4) != 0) return F.fail("bad group B-tree");
  const int level = F.d[btree + 5];
  const int used = (int)F.uint(btree + 6, 2);
  uint64_t p = btree + 8 + 2 * F.so;  // key 0
  for (int c = 0; c < used; ++c) {
    const uint64_t child = F.addr(p + F.sl);
    p += F.sl + F.so;
    if (F.oob) return F.fail("group B-tree entry outside the file");
    if (level > 0) {
      if (find_in_symbol_table(F, child, heap - F.base, name, header, depth + 1)) return true;
      if (!F.err.empty()) return false;
      continue;
    }
    const uint64_t sn = child + F.base;
    if (!F.in(sn, 8) || std::memcmp(&F.d[sn], "SNOD", 4) != 0) return F.fail("bad symbol table node");
    const int nsym = (int)F.uint(sn + 6, 2);
    const uint64_t esz = 2 * F.so + 4 + 4 + 16;
    if (!F.in(sn + 8, esz * nsym)) return F.fail("symbol table node outside the file");
    for (int e = 0; e < nsym; ++e) {
      const uint64_t ep = sn + 8 + e * esz;
      const uint64_t noff = F.uint(ep, F.so);
      if (noff >= heap_size || !F.in(heap_data + noff, 1)) return F.fail("bad link name offset");
      const char* nm = (const char*)&F.d[heap_data + noff];
      // the name ends within the heap and within the file
      const size_t maxlen = (size_t)std::min<uint64_t>(heap_size - noff, F.d.size() - (heap_data + noff));
      if (strnlen(nm, maxlen) == name.size() && std::memcmp(nm, name.data(), name.size()) == 0) {
        header = F.addr(ep + F.so);
        return true;
      }
    }
  }
  return false;
}

bool find_link(File& F, uint64_t group_header, const std::string& name, uint64_t& header) {
  std::vector<Message> msgs;
  if (!header_messages(F, group_header, msgs)) return false;
  for (const Message& m : msgs) {
    if (m.type == 0x11) {  // symbol table: B-tree, heap
      return find_in_symbol_table(F, F.addr(m.at), F.addr(m.at + F.so), name, header, 0);
    }
    if (m.type == 0x02) return F.fail("groups with dense link storage are not supported");
    if (m.type == 0x06) {  // link message
      uint64_t p = m.at;
      const int flags = F.u8(p + 1);
      p += 2;
      int ltype = 0;
      if (flags & 0x08) ltype = F.u8(p++);
      if (flags & 0x04) p += 8;  // creation order
      if (flags & 0x10) p += 1;  // character set
      const int lsz = 1 << (flags & 3);
      const uint64_t nlen = F.uint(p, lsz);
      p += lsz;
      if (F.oob || p + nlen > m.at + m.size) return F.fail("bad link message");
      if (ltype == 0 && nlen == name.size() && std::memcmp(&F.d[p], name.data(), nlen) == 0) {
        header = F.addr(p + nlen);
        if (F.oob) return F.fail("bad link message");
        return true;
      }
    }
  }
  return false;
}

// --------------------------------------------------------------- inflate --
//
// Decoder of the zlib format (RFC 1950) around a DEFLATE stream (RFC 1951),
// the encoding of the HDF5 deflate filter (filter 1).  Stored, fixed- and
// dynamic-Huffman blocks; the Adler-32 trailer is checked.  Huffman codes
// decode through one lookup table per code, indexed by the next (longest
// code length) input bits: the codes are canonical, so each is written into
// every slot whose low bits are its bit-reversed value.

struct BitReader {
  const uint8_t* p;
  size_t n, pos = 0;
  uint64_t buf = 0;
  int cnt = 0;
  size_t pad = 0;  // zero bytes supplied past the end of the input

  BitReader(const uint8_t* p_, size_t n_) : p(p_), n(n_) {}
  void fill(int k) {
    while (cnt < k) {
      uint64_t b = 0;
      if (pos < n) b = p[pos++];
      else ++pad;
      buf |= b << cnt;
      cnt += 8;
    }
  }
  uint32_t peek(int k) {
    fill(k);
    return (uint32_t)(buf & ((1ull << k) - 1));
  }
  void drop(int k) {
    buf >>= k;
    cnt -= k;
  }
  uint32_t bits(int k) {
    const uint32_t v = peek(k);
    drop(k);
    return v;
  }
  void align() { drop(cnt & 7); }
  // true once a bit past the end of the input has been consumed
  bool overrun() const { return pad * 8 > (size_t)cnt; }
};

struct HuffTable {
  int maxlen = 0;
  std::vector<uint16_t> slot;  // (symbol << 4) | code length; 0 = no code
};

// canonical code from the code lengths; false for an over-subscribed set
bool huff_build(const uint8_t* len, int n, HuffTable& t) {
  int count[16] = {0};
  for (int i = 0; i < n; ++i) count[len[i]]++;
  count[0] = 0;
  int left = 1;
  t.maxlen = 0;
  for (int l = 1; l < 16; ++l) {
    left = 2 * left - count[l];
    if (left < 0) return false;
    if (count[l]) t.maxlen = l;
  }
  if (t.maxlen == 0) t.maxlen = 1;  // no codes: every lookup fails
  t.slot.assign((size_t)1 << t.maxlen, 0);
  int next[16] = {0};
  for (int l = 1, code = 0; l < 16; ++l) {
    code = (code + count[l - 1]) << 1;
    next[l] = code;
  }
  for (int sym = 0; sym < n; ++sym) {
    const int l = len[sym];
    if (!l) continue;
    const int code = next[l]++;
    int rev = 0;
    for (int b = 0; b < l; ++b) rev |= ((code >> b) & 1) << (l - 1 - b);
    for (int k = rev; k < (1 << t.maxlen); k += 1 << l) t.slot[k] = (uint16_t)((sym << 4) | l);
  }
  return true;
}

int huff_decode(BitReader& br, const HuffTable& t) {
  const uint16_t e = t.slot[br.peek(t.maxlen)];
  if (!e) return -1;
  br.drop(e & 15);
  return e >> 4;
}

bool zlib_inflate(const uint8_t* in, size_t n, std::vector<uint8_t>& out, size_t limit, std::string& err) {
  out.clear();
  if (n < 6) return err = "deflate chunk shorter than a zlib stream", false;
  const int cmf = in[0], flg = in[1];
  if ((cmf & 15) != 8 || (cmf >> 4) > 7 || ((cmf << 8) | flg) % 31 != 0)
    return err = "deflate chunk: bad zlib header", false;
  if (flg & 0x20) return err = "deflate chunk: preset dictionaries are not supported", false;
  // length and distance codes: base value and extra bits
  int lbase[29], lext[29], dbase[30], dext[30];
  for (int i = 0, b = 3; i < 28; ++i) {
    lext[i] = i < 8 ? 0 : (i - 4) / 4;
    lbase[i] = b;
    b += 1 << lext[i];
  }
  lbase[28] = 258;
  lext[28] = 0;
  for (int i = 0, b = 1; i < 30; ++i) {
    dext[i] = i < 2 ? 0 : (i - 2) / 2;
    dbase[i] = b;
    b += 1 << dext[i];
  }
  static const int kLenOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
  BitReader br(in + 2, n - 2);
  out.reserve(std::min<size_t>(limit, (size_t)1 << 26));
  HuffTable lit, dist;
  bool last = false;
  while (!last) {
    last = br.bits(1) != 0;
    const int type = (int)br.bits(2);
    if (type == 0) {
      br.align();
      const uint32_t len = br.bits(16), nlen = br.bits(16);
      if (len != (~nlen & 0xffffu)) return err = "deflate chunk: bad stored block length", false;
      if (out.size() + len > limit) return err = "deflate chunk inflates past its chunk size", false;
      for (uint32_t i = 0; i < len; ++i) out.push_back((uint8_t)br.bits(8));
    } else if (type == 1 || type == 2) {
      uint8_t lens[320] = {0};
      int nlit = 288, ndist = 30;
      if (type == 1) {
        for (int i = 0; i < 288; ++i) lens[i] = i < 144 ? 8 : (i < 256 ? 9 : (i < 280 ? 7 : 8));
        for (int i = 0; i < 30; ++i) lens[288 + i] = 5;
      } else {
        nlit = (int)br.bits(5) + 257;
        ndist = (int)br.bits(5) + 1;
        const int ncl = (int)br.bits(4) + 4;
        if (nlit > 286 || ndist > 30) return err = "deflate chunk: bad code counts", false;
        uint8_t cl[19] = {0};
        for (int i = 0; i < ncl; ++i) cl[kLenOrder[i]] = (uint8_t)br.bits(3);
        HuffTable clt;
        if (!huff_build(cl, 19, clt)) return err = "deflate chunk: bad code-length code", false;
        for (int i = 0; i < nlit + ndist;) {
          const int sym = huff_decode(br, clt);
          if (sym < 0) return err = "deflate chunk: bad code length", false;
          if (sym < 16) {
            lens[i++] = (uint8_t)sym;
            continue;
          }
          int rep = 0;
          uint8_t v = 0;
          if (sym == 16) {
            if (i == 0) return err = "deflate chunk: repeat with no previous length", false;
            v = lens[i - 1];
            rep = 3 + (int)br.bits(2);
          } else if (sym == 17) {
            rep = 3 + (int)br.bits(3);
          } else {
            rep = 11 + (int)br.bits(7);
          }
          if (i + rep > nlit + ndist) return err = "deflate chunk: code lengths overrun", false;
          while (rep--) lens[i++] = v;
        }
        if (lens[256] == 0) return err = "deflate chunk: no end-of-block code", false;
        // the distance lengths follow the literal/length lengths
        std::memmove(lens + 288, lens + nlit, (size_t)ndist);
        std::memset(lens + nlit, 0, (size_t)(288 - nlit));
      }
      if (!huff_build(lens, 288, lit) || !huff_build(lens + 288, 30, dist))
        return err = "deflate chunk: bad Huffman code", false;
      while (true) {
        const int sym = huff_decode(br, lit);
        if (sym < 0 || br.overrun()) return err = "deflate chunk: bad or truncated literal/length code", false;
        if (sym < 256) {
          if (out.size() >= limit) return err = "deflate chunk inflates past its chunk size", false;
          out.push_back((uint8_t)sym);
          continue;
        }
        if (sym == 256) break;
        if (sym > 285) return err = "deflate chunk: bad length code", false;
        const size_t len = (size_t)lbase[sym - 257] + br.bits(lext[sym - 257]);
        const int ds = huff_decode(br, dist);
        if (ds < 0 || ds > 29) return err = "deflate chunk: bad distance code", false;
        const size_t d = (size_t)dbase[ds] + br.bits(dext[ds]);
        if (d > out.size()) return err = "deflate chunk: distance before the start of the output", false;
        if (out.size() + len > limit) return err = "deflate chunk inflates past its chunk size", false;
        const size_t from = out.size() - d;
        if (d >= len) {
          out.resize(out.size() + len);
          std::memcpy(&out[out.size() - len], &out[from], len);
        } else {
          for (size_t k = 0; k < len; ++k) out.push_back(out[from + k]);  // overlapping: a run
        }
      }
    } else {
      return err = "deflate chunk: reserved block type", false;
    }
    if (br.overrun()) return err = "deflate chunk: truncated stream", false;
  }
  br.align();
  uint32_t want = 0;
  for (int i = 0; i < 4; ++i) want = (want << 8) | br.bits(8);
  if (br.overrun()) return err = "deflate chunk: missing Adler-32 trailer", false;
  // Adler-32, reduced modulo 65521 once per 2^20 bytes: the 64-bit sums
  // stay below 2^49 in between
  uint64_t a = 1, b = 0;
  for (size_t i0 = 0; i0 < out.size(); i0 += (size_t)1 << 20) {
    const size_t i1 = std::min(out.size(), i0 + ((size_t)1 << 20));
    for (size_t i = i0; i < i1; ++i) {
      a += out[i];
      b += a;
    }
    a %= 65521u;
    b %= 65521u;
  }
  if ((uint32_t)((b << 16) | a) != want) return err = "deflate chunk: Adler-32 mismatch", false;
  return true;
}

// ------------------------------------------------------- chunked datasets --

struct Filter {
  int id = 0, flags = 0;
  std::vector<uint32_t> cd;  // client data
};

// filter pipeline message (versions 1 and 2)
bool parse_filters(File& F, const Message& m, std::vector<Filter>& fl) {
  const int v = F.u8(m.at), nf = F.u8(m.at + 1);
  if (v != 1 && v != 2) return F.fail("unsupported filter pipeline message version");
  uint64_t p = m.at + (v == 1 ? 8 : 2);
  const uint64_t end = m.at + m.size;
  for (int i = 0; i < nf; ++i) {
    Filter f;
    f.id = (int)F.uint(p, 2);
    p += 2;
    uint64_t nlen = 0;
    if (v == 1 || f.id >= 256) {
      nlen = F.uint(p, 2);
      p += 2;
    }
    f.flags = (int)F.uint(p, 2);
    const uint64_t ncd = F.uint(p + 2, 2);
    p += 4;
    p += v == 1 ? (nlen + 7) / 8 * 8 : nlen;  // name
    if (ncd > 64 || p + 4 * ncd > end) return F.fail("bad filter pipeline message");
    for (uint64_t c = 0; c < ncd; ++c) f.cd.push_back((uint32_t)F.uint(p + 4 * c, 4));
    p += 4 * ncd;
    if (v == 1 && (ncd & 1)) p += 4;
    if (F.oob || p > end) return F.fail("bad filter pipeline message");
    fl.push_back(f);
  }
  return true;
}

struct Chunk {
  uint64_t size = 0, at = 0;
  uint32_t mask = 0;
  uint64_t off[2] = {0, 0};
};

// the chunks of a version-1 B-tree of raw data chunks (node type 1); keys
// hold the chunk's stored size, filter mask and element offsets.  At most
// 2^16 nodes are visited, so a node that lists itself cannot blow up.
bool chunk_btree(File& F, uint64_t at, int ndims, std::vector<Chunk>& out, int depth, int& nodes) {
  if (depth > 32) return F.fail("chunk B-tree too deep");
  if (++nodes > (1 << 16)) return F.fail("chunk B-tree has too many nodes");
  at += F.base;
  if (!F.in(at, 8 + 2 * (uint64_t)F.so) || std::memcmp(&F.d[at], "TREE", 4) != 0 || F.d[at + 4] != 1)
    return F.fail("bad chunk B-tree node");
  const int level = F.d[at + 5];
  const int used = (int)F.uint(at + 6, 2);
  const uint64_t ksz = 8 + 8 * (uint64_t)ndims;
  uint64_t p = at + 8 + 2 * F.so;
  if (!F.in(p, (uint64_t)used * (ksz + F.so) + ksz)) return F.fail("chunk B-tree node outside the file");
  for (int c = 0; c < used; ++c) {
    Chunk ch;
    ch.size = F.uint(p, 4);
    ch.mask = (uint32_t)F.uint(p + 4, 4);
    for (int d = 0; d < ndims - 1 && d < 2; ++d) ch.off[d] = F.uint(p + 8 + 8 * d, 8);
    ch.at = F.addr(p + ksz);
    p += ksz + F.so;
    if (F.oob || ch.at == kUndef) return F.fail("bad chunk B-tree entry");
    if (level > 0) {
      if (!chunk_btree(F, ch.at, ndims, out, depth + 1, nodes)) return false;
    } else {
      if (out.size() >= (1u << 24)) return F.fail("too many chunks");
      out.push_back(ch);
    }
  }
  return true;
}

// Reads a chunked dataset of rank 1 or 2 (layout message version 3, class
// 2): each chunk is un-filtered (deflate, byte shuffle, in the reverse of
// the pipeline's order, skipping the filters its mask excludes) and copied
// into the rows x cols array; chunks never written read as 0.  This is the
// layout of the HDF5 monitor's "compressed" option
// (src/jams/monitors/hdf5.cc:292-323: chunks of min(4095, rows) x 1
// values, shuffle, deflate level 6).
bool read_chunked(File& F, uint64_t btree, const std::vector<uint64_t>& cdims, const std::vector<Filter>& filters,
                  int tsize, uint64_t d0, uint64_t d1, int rank, std::vector<double>& out) {
  const int ndims = rank + 1;
  if ((int)cdims.size() != ndims || cdims[rank] != (uint64_t)tsize) return F.fail("chunk dimensions do not match the dataset");
  uint64_t c0 = cdims[0], c1 = rank == 2 ? cdims[1] : 1;
  if (c0 == 0 || c1 == 0 || c0 > (1ull << 31) || c1 > (1ull << 31) || c0 * c1 > (1ull << 28))
    return F.fail("chunk dimensions out of range");
  for (const Filter& f : filters)
    if (f.id != 1 && f.id != 2 && !(f.flags & 1))
      return F.fail("filter " + std::to_string(f.id) + " is not supported (deflate and shuffle are)");
  std::vector<Chunk> chunks;
  int nodes = 0;
  if (btree != kUndef && !chunk_btree(F, btree, ndims, chunks, 0, nodes)) return false;
  // the array is allocated only as large as its chunks can fill (plus up
  // to 2^24 values of unwritten fill), so corrupt extents cannot ask for
  // more memory than the file describes
  if (d0 * d1 > (1ull << 24) + (uint64_t)chunks.size() * c0 * c1)
    return F.fail("extents larger than the chunks written");
  out.assign(d0 * d1, 0.0);
  const size_t cbytes = (size_t)(c0 * c1) * tsize;
  std::vector<uint8_t> a, b;
  std::string ferr;
  for (const Chunk& ch : chunks) {
    const uint64_t o0 = ch.off[0], o1 = rank == 2 ? ch.off[1] : 0;
    if (o0 >= d0 || o1 >= d1 || o0 % c0 || o1 % c1) return F.fail("chunk offset outside the dataset");
    const uint64_t at = ch.at + F.base;
    if (!F.in(at, ch.size)) return F.fail("chunk data outside the file");
    // zlib expands by at most 1032:1; an unfiltered chunk is stored whole
    bool inflates = false;
    for (size_t i = 0; i < filters.size(); ++i)
      if (filters[i].id == 1 && !(i < 32 && (ch.mask >> i) & 1)) inflates = true;
    if (inflates ? cbytes > 1032 * ch.size + 64 : ch.size < cbytes)
      return F.fail("chunk stored size does not match its extents");
    a.assign(F.d.begin() + at, F.d.begin() + at + ch.size);
    for (int i = (int)filters.size() - 1; i >= 0; --i) {
      if (i < 32 && (ch.mask >> i) & 1) continue;  // skipped when written
      const Filter& f = filters[i];
      if (f.id == 1) {
        if (!zlib_inflate(a.data(), a.size(), b, cbytes, ferr)) return F.fail(ferr);
        a.swap(b);
      } else if (f.id == 2) {
        const size_t es = f.cd.empty() ? (size_t)tsize : f.cd[0];
        if (es > 1 && a.size() >= es) {
          const size_t ne = a.size() / es;
          b.resize(a.size());
          for (size_t j = 0; j < es; ++j)
            for (size_t e = 0; e < ne; ++e) b[e * es + j] = a[j * ne + e];
          std::copy(a.begin() + ne * es, a.end(), b.begin() + ne * es);
          a.swap(b);
        }
      } else {
        return F.fail("optional filter " + std::to_string(f.id) + " was applied to a chunk: not supported");
      }
    }
    if (a.size() != cbytes) return F.fail("chunk decodes to " + std::to_string(a.size()) + " bytes, not " + std::to_string(cbytes));
    for (uint64_t i = 0; i < c0 && o0 + i < d0; ++i)
      for (uint64_t j = 0; j < c1 && o1 + j < d1; ++j) {
        const uint8_t* q = &a[(size_t)(i * c1 + j) * tsize];
        double v;
        if (tsize == 8) {
          uint64_t u = 0;
          for (int k = 0; k < 8; ++k) u |= (uint64_t)q[k] << (8 * k);
          std::memcpy(&v, &u, 8);
        } else {
          uint32_t u = 0;
          for (int k = 0; k < 4; ++k) u |= (uint32_t)q[k] << (8 * k);
          float f;
          std::memcpy(&f, &u, 4);
          v = f;
        }
        out[(o0 + i) * d1 + (o1 + j)] = v;
      }
  }
  return true;
}

int read_h5(const std::string& path, const std::string& dataset, std::vector<double>& out, int64_t& rows,
            int64_t& cols, std::string& err) {
  File F;
  {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) {
      err = "failed to open file: " + path;
      return 1;
    }
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    F.d.resize(n > 0 ? (size_t)n : 0);
    const bool ok = n > 0 && std::fread(F.d.data(), 1, F.d.size(), f) == F.d.size();
    std::fclose(f);
    if (!ok) {
      err = "failed reading " + path;
      return 1;
    }
  }
  const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
  uint64_t sb = kUndef;
  for (uint64_t at = 0; at + 8 <= F.d.size(); at = at ? at * 2 : 512)
    if (std::memcmp(&F.d[at], sig, 8) == 0) {
      sb = at;
      break;
    }
  if (sb == kUndef) {
    err = path + " is not an HDF5 file";
    return 1;
  }
  if (!F.in(sb, 64)) {
    err = "truncated HDF5 superblock";
    return 1;
  }
  const int sbv = F.d[sb + 8];
  uint64_t root = kUndef;
  if (sbv == 0 || sbv == 1) {
    F.so = F.d[sb + 13];
    F.sl = F.d[sb + 14];
    uint64_t p = sb + 24 + (sbv == 1 ? 4 : 0);
    if ((F.so != 2 && F.so != 4 && F.so != 8) || (F.sl != 2 && F.sl != 4 && F.sl != 8) ||
        !F.in(p, 4 * F.so + 2 * F.so + 24)) {
      err = "unsupported HDF5 superblock";
      return 1;
    }
    F.base = F.addr(p);
    p += 4 * F.so;            // base, free space, end of file, driver block
    root = F.addr(p + F.so);  // root entry: name offset, object header
  } else if (sbv == 2 || sbv == 3) {
    F.so = F.d[sb + 9];
    F.sl = F.d[sb + 10];
    if ((F.so != 2 && F.so != 4 && F.so != 8) || !F.in(sb + 12, 4 * F.so)) {
      err = "unsupported HDF5 superblock";
      return 1;
    }
    F.base = F.addr(sb + 12);
    root = F.addr(sb + 12 + 3 * F.so);  // base, extension, end of file, root header
  } else {
    err = "unsupported HDF5 superblock version " + std::to_string(sbv);
    return 1;
  }
  uint64_t head = kUndef;
  if (!find_link(F, root, dataset, head)) {
    err = F.err.empty() ? "dataset /" + dataset + " not found in " + path : F.err;
    return 1;
  }
  std::vector<Message> msgs;
  if (!header_messages(F, head, msgs)) {
    err = F.err;
    return 1;
  }
  std::vector<uint64_t> dims;
  int tsize = 0;
  bool tfloat = false, tle = true;
  int layout = -1;
  uint64_t data_at = kUndef, data_size = 0;
  std::vector<uint64_t> cdims;  // chunked: chunk extents, the element size last
  std::vector<Filter> filters;
  for (const Message& m : msgs) {
    const uint64_t p = m.at;
    if (m.type == 0x01) {  // dataspace
      const int v = F.u8(p), rank = F.u8(p + 1);
      const uint64_t q = p + (v == 1 ? 8 : 4);
      for (int r = 0; r < rank; ++r) dims.push_back(F.uint(q + (uint64_t)r * F.sl, F.sl));
    } else if (m.type == 0x03) {  // datatype
      tfloat = (F.u8(p) & 0x0f) == 1;
      tle = (F.u8(p + 1) & 0x41) == 0;
      tsize = (int)F.uint(p + 4, 4);
    } else if (m.type == 0x08) {  // layout
      const int v = F.u8(p);
      if (v == 3 || v == 4) {
        layout = F.u8(p + 1);
        if (layout == 1) {
          data_at = F.addr(p + 2);
          data_size = F.uint(p + 2 + F.so, F.sl);
        } else if (layout == 0) {
          data_size = F.uint(p + 2, 2);
          data_at = p + 4 - F.base;
        } else if (layout == 2 && v == 3) {  // dimensionality, B-tree address, extents
          const int nd = F.u8(p + 2);
          data_at = F.addr(p + 3);
          for (int r = 0; r < nd && r < 4; ++r) cdims.push_back(F.uint(p + 3 + F.so + 4 * (uint64_t)r, 4));
        } else if (layout == 2) {
          err = "dataset /" + dataset + " uses a version-4 chunk index: only version-3 (B-tree) chunked layouts are supported";
          return 1;
        }
      } else if (v == 1 || v == 2) {
        const int rank = F.u8(p + 1);
        layout = F.u8(p + 2);
        if (layout == 1) {
          data_at = F.addr(p + 8);
          uint64_t n = 1;
          for (int r = 0; r < rank; ++r) n *= F.uint(p + 8 + F.so + 4 * (uint64_t)r, 4);
          data_size = n;  // elements x element size; fixed below
        }
      }
    } else if (m.type == 0x0B) {
      if (!parse_filters(F, m, filters)) {
        err = "dataset /" + dataset + ": " + F.err;
        return 1;
      }
    }
  }
  if (F.oob) {
    err = "dataset /" + dataset + ": a header field lies outside the file";
    return 1;
  }
  if (layout != 0 && layout != 1 && layout != 2) {
    err = "dataset /" + dataset + " is virtual: only contiguous, compact and chunked datasets are supported";
    return 1;
  }
  if (layout != 2 && !filters.empty()) {
    err = "dataset /" + dataset + " has a filter pipeline but is not chunked";
    return 1;
  }
  if (!tfloat || !tle || (tsize != 8 && tsize != 4)) {
    err = "dataset /" + dataset + " is not a little-endian float32/float64 array";
    return 1;
  }
  if (dims.empty() || dims.size() > 2) {
    err = "dataset /" + dataset + " is not one- or two-dimensional";
    return 1;
  }
  // extents below 2^40 and at most 2^34 values, so that neither the value
  // count nor the byte count wraps; a dataset never written (no data
  // address) reads as zeros, up to 2^24 values
  const uint64_t d0 = dims[0], d1 = dims.size() == 2 ? dims[1] : 1;
  if (d0 >= (1ull << 40) || d1 >= (1ull << 40) || (d1 != 0 && d0 > (1ull << 34) / d1)) {
    err = "dataset /" + dataset + " has extents too large for this reader";
    return 1;
  }
  rows = (int64_t)d0;
  cols = (int64_t)d1;
  const uint64_t n = d0 * d1;
  if (layout == 2) {
    if (!read_chunked(F, data_at, cdims, filters, tsize, d0, d1, (int)dims.size(), out)) {
      err = "dataset /" + dataset + ": " + F.err;
      out.clear();
      return 1;
    }
    return 0;
  }
  if (data_at == kUndef) {  // never written: fill value 0
    if (n > (1ull << 24)) {
      err = "dataset /" + dataset + " was never written and is too large to read as zeros";
      return 1;
    }
    out.assign(n, 0.0);
    return 0;
  }
  data_at += F.base;
  if (!F.in(data_at, n * tsize) || (data_size && data_size < n * tsize && layout == 0)) {
    err = "dataset /" + dataset + " data lies outside the file";
    return 1;
  }
  out.resize(n);
  for (uint64_t i = 0; i < n; ++i) {
    if (tsize == 8) {
      const uint64_t u = F.uint(data_at + 8 * i, 8);
      std::memcpy(&out[i], &u, 8);
    } else {
      const uint32_t u = (uint32_t)F.uint(data_at + 4 * i, 4);
      float f;
      std::memcpy(&f, &u, 4);
      out[i] = f;
    }
  }
  return 0;
}

}  // namespace

int write_array(const std::string& path, const std::vector<Dataset>& sets, std::string& err) {
  if (extension(path) == "h5") return write_h5(path, sets, err);
  if (sets.size() != 1) {
    err = "a text array file holds one array";
    return 1;
  }
  return write_text(path, sets[0].data, sets[0].rows, sets[0].cols, err);
}

int read_array(const std::string& path, const char* dataset, std::vector<double>& out, int64_t& rows,
               int64_t& cols, std::string& err) {
  // the callers are C entry points: an allocation failure becomes an error
  try {
    if (extension(path) == "h5") return read_h5(path, strip_slash(dataset), out, rows, cols, err);
    const int rc = read_text(path, out, err);
    rows = (int64_t)out.size();
    cols = 1;
    return rc;
  } catch (const std::exception& e) {
    out.clear();
    err = std::string("reading ") + path + ": " + e.what();
    return 1;
  }
}

std::string dataset_name(const char* name) { return strip_slash(name); }

}  // namespace llgio
