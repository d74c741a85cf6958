/* The reference's ECAL data files read without ROOT, for C++ drivers
 * (header-only, C++17, no dependencies; nothing here touches the GPU).
 *
 *   mfgb::rootio::RootFile   a closed ROOT file in memory: directories, keys,
 *                            TTree branches (fixed-size leaves and
 *                            std::vector<T> entries), TGraph points.
 *   mfgb::Pulse              the pulse shape and noise correlation of a
 *                            pulse-shape file (multifit_cpu/interface/Pulse.h:
 *                            38-168): TGraph PulseShape/grPulseShape below
 *                            800 ns, the PulseShape/Tail exponential above,
 *                            NoiseInit's CRRC correlation.
 *   mfgb::driver_fullpulse   the driver's conditions (multifit_cpu/src/
 *   mfgb::driver_noisecor    multifit.cpp:45-81): template at fullpulse(7..18),
 *                            corr(|i-j|), BXs -5..4, pederr 1.0.
 *   mfgb::ecal_data_io       io/src/ecal_data_io.cpp:6-53: entries of the
 *                            Samples tree as (samples, pulse matrix),
 *                            round-robin.
 *
 * The on-disk layout read here (all numbers big-endian): the file header
 * ("root", version >= 1000000 for 64-bit seeks, fBEGIN, fEND, fSeekFree,
 * fNbytesFree, nfree, fNbytesName, ...); a key in front of every record
 * (Nbytes, version > 1000 for 64-bit seeks, ObjLen, Datime, KeyLen, Cycle,
 * SeekKey, SeekPdir, class name, name, title); directory records (version,
 * dates, NbytesKeys, NbytesName, SeekDir, SeekParent, SeekKeys) and keys
 * lists (a key, an int32 count, the key headers); compressed records as
 * blocks of a 9-byte header (algorithm "ZL", method, 3-byte little-endian
 * compressed and uncompressed sizes) and a zlib stream (RFC 1950/1951,
 * inflated by the decoder below); basket keys extended by version,
 * BufferSize, NevBufSize, NevBuf, Last and a flag, their buffers holding the
 * entries up to Last, then, for entries of varying size, an int32 count and
 * the entries' start offsets; streamed objects as a byte count (bit 30 set),
 * a version and their members, base classes skipped by their byte counts.
 * A branch's entries come from its basket keys in file order and must add up
 * to the tree's fEntries. Files written without TFile::Close, and LZMA, LZ4
 * or ZSTD blocks, raise mfgb::rootio::FormatError. */
#ifndef MULTIFIT_GB300_IO_HPP
#define MULTIFIT_GB300_IO_HPP

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace mfgb {
namespace rootio {

struct FormatError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

namespace detail {

// ---- inflate (RFC 1951 DEFLATE inside an RFC 1950 zlib stream) -------------

class BitReader {
 public:
  BitReader(const uint8_t* p, size_t n) : p_(p), n_(n) {}
  unsigned bit() {
    if (cnt_ == 0) {
      if (pos_ >= n_) throw FormatError("zlib: compressed data ends early");
      buf_ = p_[pos_++];
      cnt_ = 8;
    }
    const unsigned b = buf_ & 1u;
    buf_ >>= 1;
    --cnt_;
    return b;
  }
  uint32_t bits(int k) {  // k bits, least significant first
    uint32_t v = 0;
    for (int i = 0; i < k; ++i) v |= uint32_t(bit()) << i;
    return v;
  }
  void align() { cnt_ = 0; }
  uint8_t byte() {
    if (pos_ >= n_) throw FormatError("zlib: compressed data ends early");
    return p_[pos_++];
  }
  size_t pos() const { return pos_; }

 private:
  const uint8_t* p_;
  size_t n_;
  size_t pos_ = 0;
  unsigned buf_ = 0;
  int cnt_ = 0;
};

// Canonical Huffman code: how many codes have each length, and the symbols
// ordered by (length, symbol value). Codes of one length are consecutive
// integers following the last code of the previous length, shifted left.
struct Huffman {
  uint16_t count[16] = {};
  std::vector<uint16_t> symbol;

  void build(const uint8_t* lengths, int n) {
    std::fill(std::begin(count), std::end(count), uint16_t(0));
    for (int s = 0; s < n; ++s) ++count[lengths[s]];
    count[0] = 0;
    int left = 1;  // unused codes of the current length
    for (int len = 1; len < 16; ++len) {
      left = 2 * left - count[len];
      if (left < 0) throw FormatError("zlib: over-subscribed Huffman code");
    }
    int offs[16] = {};
    for (int len = 1; len < 15; ++len) offs[len + 1] = offs[len] + count[len];
    symbol.assign(size_t(n), 0);
    for (int s = 0; s < n; ++s)
      if (lengths[s]) symbol[size_t(offs[lengths[s]]++)] = uint16_t(s);
  }

  int decode(BitReader& br) const {
    int code = 0, first = 0, index = 0;
    for (int len = 1; len < 16; ++len) {
      code |= int(br.bit());
      const int c = count[len];
      if (code - first < c) return symbol[size_t(index + code - first)];
      index += c;
      first = (first + c) << 1;
      code <<= 1;
    }
    throw FormatError("zlib: invalid Huffman code");
  }
};

// RFC 1951 3.2.5: base lengths / distances of the length and distance codes
// and their extra bits.
constexpr uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                   31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
constexpr uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
constexpr uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                    193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
constexpr uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
// RFC 1951 3.2.7: order in which the code-length code lengths are sent
constexpr uint8_t kClOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

// Output beyond `limit` bytes (the block's declared inflated size) is an
// error at once, so a damaged stream cannot grow memory past what it declares.
inline void inflate_block(BitReader& br, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out,
                          size_t limit) {
  for (;;) {
    const int sym = lit.decode(br);
    if (sym < 256) {
      if (out.size() >= limit) throw FormatError("zlib: output exceeds the declared size");
      out.push_back(uint8_t(sym));
    } else if (sym == 256) {
      return;
    } else {
      const int li = sym - 257;
      if (li >= 29) throw FormatError("zlib: invalid length code");
      const size_t len = kLenBase[li] + br.bits(kLenExtra[li]);
      const int di = dist.decode(br);
      if (di >= 30) throw FormatError("zlib: invalid distance code");
      const size_t d = kDistBase[di] + br.bits(kDistExtra[di]);
      if (d > out.size()) throw FormatError("zlib: distance before the start of the data");
      if (len > limit - out.size()) throw FormatError("zlib: output exceeds the declared size");
      const size_t from = out.size() - d;
      for (size_t i = 0; i < len; ++i) {  // byte by byte: the copy may overlap its own output
        const uint8_t c = out[from + i];
        out.push_back(c);
      }
    }
  }
}

/* Inflates one zlib stream (2-byte header, DEFLATE blocks, Adler-32) whose
 * inflated size is at most `expected` bytes (FormatError beyond). */
inline std::vector<uint8_t> zlib_inflate(const uint8_t* p, size_t n, size_t expected) {
  if (n < 6) throw FormatError("zlib: stream too short");
  const unsigned cmf = p[0], flg = p[1];
  if ((cmf & 15u) != 8 || (cmf >> 4) > 7 || ((cmf << 8) | flg) % 31 != 0)
    throw FormatError("zlib: bad stream header");
  if (flg & 0x20u) throw FormatError("zlib: preset dictionaries are not supported");
  BitReader br(p + 2, n - 2);
  std::vector<uint8_t> out;
  out.reserve(expected);
  Huffman fixed_lit, fixed_dist;
  {
    uint8_t l[288];
    for (int s = 0; s < 288; ++s) l[s] = s < 144 ? 8 : s < 256 ? 9 : s < 280 ? 7 : 8;
    fixed_lit.build(l, 288);
    uint8_t d[30];
    std::fill(d, d + 30, uint8_t(5));
    fixed_dist.build(d, 30);
  }
  unsigned last = 0;
  while (!last) {
    last = br.bit();
    const uint32_t type = br.bits(2);
    if (type == 0) {  // stored
      br.align();
      const unsigned len = br.byte() | (unsigned(br.byte()) << 8);
      const unsigned nlen = br.byte() | (unsigned(br.byte()) << 8);
      if ((len ^ 0xffffu) != nlen) throw FormatError("zlib: stored block length check failed");
      if (len > expected - out.size()) throw FormatError("zlib: output exceeds the declared size");
      for (unsigned i = 0; i < len; ++i) out.push_back(br.byte());
    } else if (type == 1) {
      inflate_block(br, fixed_lit, fixed_dist, out, expected);
    } else if (type == 2) {
      const int hlit = int(br.bits(5)) + 257, hdist = int(br.bits(5)) + 1, hclen = int(br.bits(4)) + 4;
      if (hlit > 286 || hdist > 30) throw FormatError("zlib: bad dynamic block counts");
      uint8_t cl[19] = {};
      for (int i = 0; i < hclen; ++i) cl[kClOrder[i]] = uint8_t(br.bits(3));
      Huffman clh;
      clh.build(cl, 19);
      uint8_t lens[286 + 30] = {};
      int k = 0;
      while (k < hlit + hdist) {
        const int sym = clh.decode(br);
        if (sym < 16) {
          lens[k++] = uint8_t(sym);
          continue;
        }
        int rep = 0;
        uint8_t val = 0;
        if (sym == 16) {
          if (k == 0) throw FormatError("zlib: repeat with no previous length");
          val = lens[k - 1];
          rep = 3 + int(br.bits(2));
        } else if (sym == 17) {
          rep = 3 + int(br.bits(3));
        } else {
          rep = 11 + int(br.bits(7));
        }
        if (k + rep > hlit + hdist) throw FormatError("zlib: code lengths overrun");
        while (rep--) lens[k++] = val;
      }
      if (lens[256] == 0) throw FormatError("zlib: no end-of-block code");
      Huffman lit, dist;
      lit.build(lens, hlit);
      dist.build(lens + hlit, hdist);
      inflate_block(br, lit, dist, out, expected);
    } else {
      throw FormatError("zlib: reserved block type");
    }
  }
  br.align();
  uint32_t want = 0;
  for (int i = 0; i < 4; ++i) want = (want << 8) | br.byte();
  uint32_t a = 1, b = 0;  // Adler-32 (RFC 1950 2.2), modulus 65521
  for (uint8_t c : out) {
    a = (a + c) % 65521u;
    b = (b + a) % 65521u;
  }
  if (((b << 16) | a) != want) throw FormatError("zlib: Adler-32 check failed");
  return out;
}

// ---- big-endian reads -------------------------------------------------------

inline uint64_t be(const std::vector<uint8_t>& d, size_t p, int nbytes) {
  if (p + size_t(nbytes) > d.size()) throw FormatError("read past the end of a record");
  uint64_t v = 0;
  for (int i = 0; i < nbytes; ++i) v = (v << 8) | d[p + size_t(i)];
  return v;
}
inline int16_t i16(const std::vector<uint8_t>& d, size_t p) { return int16_t(uint16_t(be(d, p, 2))); }
inline int32_t i32(const std::vector<uint8_t>& d, size_t p) { return int32_t(uint32_t(be(d, p, 4))); }
inline uint32_t u32(const std::vector<uint8_t>& d, size_t p) { return uint32_t(be(d, p, 4)); }
inline int64_t i64(const std::vector<uint8_t>& d, size_t p) { return int64_t(be(d, p, 8)); }

template <typename T>
T value(const std::vector<uint8_t>& d, size_t p) {
  static_assert(sizeof(T) == 1 || sizeof(T) == 2 || sizeof(T) == 4 || sizeof(T) == 8, "plain value types only");
  const uint64_t bits = be(d, p, int(sizeof(T)));
  T v;
  if constexpr (sizeof(T) == 1) {
    const uint8_t b = uint8_t(bits);
    std::memcpy(&v, &b, 1);
  } else if constexpr (sizeof(T) == 2) {
    const uint16_t b = uint16_t(bits);
    std::memcpy(&v, &b, 2);
  } else if constexpr (sizeof(T) == 4) {
    const uint32_t b = uint32_t(bits);
    std::memcpy(&v, &b, 4);
  } else {
    std::memcpy(&v, &bits, 8);
  }
  return v;
}

constexpr uint32_t kByteCount = 0x40000000u;

inline size_t skip_streamed(const std::vector<uint8_t>& d, size_t p, const char* what) {
  const uint32_t bc = u32(d, p);
  if (!(bc & kByteCount)) throw FormatError(std::string(what) + ": no byte count");
  const size_t end = p + 4 + (bc & ~kByteCount);
  if (end > d.size()) throw FormatError(std::string(what) + ": byte count runs past the record");
  return end;
}

// After the class header, TNamed, TAttLine, TAttFill and TAttMarker of a
// TTree or TGraph record; *bits = TObject::fBits.
inline size_t skip_named_and_attributes(const std::vector<uint8_t>& d, uint32_t* bits, const char* what) {
  size_t p = 6;
  *bits = u32(d, p + 6 + 2 + 4);
  for (int i = 0; i < 4; ++i) p = skip_streamed(d, p, what);
  return p;
}

}  // namespace detail

constexpr uint32_t kIsSortedX = 1u << 14;  // TGraph::kIsSortedX in TObject::fBits

struct Key {
  int64_t pos = 0, nbytes = 0, objlen = 0, keylen = 0, seek_key = 0, seek_pdir = 0;
  int version = 0, cycle = 0;
  std::string class_name, name, title;
  size_t header_end = 0;
  bool compressed() const { return objlen > nbytes - keylen; }
};

struct Graph {
  std::vector<double> x, y;
  uint32_t bits = 0;
};

class Tree;

class RootFile {
 public:
  explicit RootFile(const std::string& path) : path_(path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw FormatError(path + ": cannot open");
    data_.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    init();
  }
  RootFile(std::vector<uint8_t> bytes, std::string label) : path_(std::move(label)), data_(std::move(bytes)) {
    init();
  }

  const std::vector<uint8_t>& data() const { return data_; }
  const std::string& path() const { return path_; }
  bool closed() const { return end_ == int64_t(data_.size()); }
  int64_t end() const { return end_; }

  Key read_key(size_t pos) const {
    using namespace detail;
    Key k;
    k.pos = int64_t(pos);
    k.nbytes = i32(data_, pos);
    k.version = i16(data_, pos + 4);
    k.objlen = i32(data_, pos + 6);
    k.keylen = i16(data_, pos + 14);
    k.cycle = i16(data_, pos + 16);
    size_t p = pos + 18;
    if (k.version > 1000) {
      k.seek_key = i64(data_, p);
      k.seek_pdir = i64(data_, p + 8);
      p += 16;
    } else {
      k.seek_key = i32(data_, p);
      k.seek_pdir = i32(data_, p + 4);
      p += 8;
    }
    k.class_name = tstring(p);
    k.name = tstring(p);
    k.title = tstring(p);
    k.header_end = p;
    return k;
  }

  std::vector<Key> keys(const std::string& directory = "") const {
    int64_t seek_keys = top_seek_keys_;
    size_t start = 0;
    while (start < directory.size()) {
      size_t slash = directory.find('/', start);
      if (slash == std::string::npos) slash = directory.size();
      const std::string part = directory.substr(start, slash - start);
      start = slash + 1;
      if (part.empty()) continue;
      const Key k = find(keys_list(seek_keys), part);
      if (k.class_name.rfind("TDirectory", 0) != 0)
        throw FormatError(path_ + ": " + part + " is a " + k.class_name + ", not a directory");
      seek_keys = dir_seek_keys(size_t(k.seek_key + k.keylen));
    }
    return keys_list(seek_keys);
  }

  Key get_key(const std::string& path) const {
    const size_t slash = path.rfind('/');
    const std::string dir = slash == std::string::npos ? "" : path.substr(0, slash);
    const std::string name = slash == std::string::npos ? path : path.substr(slash + 1);
    return find(keys(dir), name);
  }

  std::vector<uint8_t> payload(const Key& k) const {
    const size_t start = size_t(k.seek_key + k.keylen), stop = size_t(k.seek_key + k.nbytes);
    if (stop > data_.size() || start > stop) throw FormatError(path_ + ": record " + k.name + " runs past the file");
    if (!k.compressed()) return std::vector<uint8_t>(data_.begin() + long(start), data_.begin() + long(stop));
    std::vector<uint8_t> out;
    out.reserve(size_t(k.objlen));
    size_t p = start;
    while (int64_t(out.size()) < k.objlen) {
      if (p + 9 > stop) throw FormatError(path_ + ": " + k.name + ": truncated compressed block");
      const size_t csize = data_[p + 3] | size_t(data_[p + 4]) << 8 | size_t(data_[p + 5]) << 16;
      const size_t usize = data_[p + 6] | size_t(data_[p + 7]) << 8 | size_t(data_[p + 8]) << 16;
      if (data_[p] != 'Z' || data_[p + 1] != 'L')
        throw FormatError(path_ + ": " + k.name + ": compression '" + std::string(1, char(data_[p])) +
                          std::string(1, char(data_[p + 1])) + "' is not supported (zlib is)");
      if (p + 9 + csize > stop) throw FormatError(path_ + ": " + k.name + ": compressed block runs past the record");
      const std::vector<uint8_t> part = detail::zlib_inflate(&data_[p + 9], csize, usize);
      if (part.size() != usize) throw FormatError(path_ + ": " + k.name + ": block inflated to a wrong size");
      out.insert(out.end(), part.begin(), part.end());
      p += 9 + csize;
    }
    if (int64_t(out.size()) != k.objlen) throw FormatError(path_ + ": " + k.name + ": inflated size is not ObjLen");
    return out;
  }

  /* Every key from fBEGIN on, in file order (free gaps stepped over). */
  std::vector<Key> walk() const {
    std::vector<Key> out;
    size_t pos = size_t(begin_);
    while (pos + 4 <= data_.size()) {
      const int32_t n = detail::i32(data_, pos);
      if (n < 0) {
        pos += size_t(-int64_t(n));
        continue;
      }
      if (n == 0) break;
      out.push_back(read_key(pos));
      pos += size_t(n);
    }
    return out;
  }

  Graph graph(const std::string& path) const {
    const Key k = get_key(path);
    if (k.class_name != "TGraph") throw FormatError(path_ + ": " + path + " is not a TGraph");
    const std::vector<uint8_t> d = payload(k);
    Graph g;
    size_t p = detail::skip_named_and_attributes(d, &g.bits, "TGraph");
    const int32_t n = detail::i32(d, p);
    p += 4;
    for (std::vector<double>* arr : {&g.x, &g.y}) {
      if (p >= d.size()) throw FormatError(path_ + ": " + path + ": record ends before its arrays");
      const uint8_t present = d[p++];
      if (!present) continue;
      if (n < 0 || p + 8 * size_t(n) > d.size()) throw FormatError(path_ + ": " + path + ": array runs past the record");
      arr->resize(size_t(n));
      for (int32_t i = 0; i < n; ++i) (*arr)[size_t(i)] = detail::value<double>(d, p + 8 * size_t(i));
      p += 8 * size_t(n);
    }
    return g;
  }

  inline Tree tree(const std::string& path) const;

 private:
  void init() {
    using namespace detail;
    if (data_.size() < 64 || std::string(data_.begin(), data_.begin() + 4) != "root")
      throw FormatError(path_ + ": not a ROOT file");
    const int32_t version = i32(data_, 4);
    begin_ = i32(data_, 8);
    size_t p;
    if (version >= 1000000) {
      end_ = i64(data_, 12);
      p = 28;
    } else {
      end_ = i32(data_, 12);
      p = 20;
    }
    const int32_t nbytes_name = i32(data_, p + 8);
    if (begin_ <= 0 || size_t(begin_) >= data_.size())
      throw FormatError(path_ + ": header fBEGIN outside the file");
    top_seek_keys_ = dir_seek_keys(size_t(begin_ + nbytes_name));
  }

  int64_t dir_seek_keys(size_t pos) const {
    using namespace detail;
    const int16_t version = i16(data_, pos);
    const size_t p = pos + 18;
    return version > 1000 ? i64(data_, p + 16) : i32(data_, p + 8);
  }

  std::vector<Key> keys_list(int64_t seek_keys) const {
    if (seek_keys <= 0)
      throw FormatError(path_ + ": directory without a keys list (file not closed: header fEND " +
                        std::to_string(end_) + ", file size " + std::to_string(data_.size()) + ")");
    const Key head = read_key(size_t(seek_keys));
    size_t p = size_t(seek_keys + head.keylen);
    const int32_t n = detail::i32(data_, p);
    p += 4;
    std::vector<Key> out;
    for (int32_t i = 0; i < n; ++i) {
      out.push_back(read_key(p));
      p = out.back().header_end;
    }
    return out;
  }

  Key find(const std::vector<Key>& keys, const std::string& name) const {
    const Key* best = nullptr;
    for (const Key& k : keys)
      if (k.name == name && (!best || k.cycle > best->cycle)) best = &k;
    if (!best) throw FormatError(path_ + ": no object named '" + name + "'");
    return *best;
  }

  std::string tstring(size_t& p) const {
    if (p >= data_.size()) throw FormatError(path_ + ": string runs past the file");
    size_t n = data_[p++];
    if (n == 255) {
      n = size_t(detail::i32(data_, p));
      p += 4;
    }
    if (p + n > data_.size()) throw FormatError(path_ + ": string runs past the file");
    std::string s(data_.begin() + long(p), data_.begin() + long(p + n));
    p += n;
    return s;
  }

  std::string path_;
  std::vector<uint8_t> data_;
  int64_t begin_ = 0, end_ = 0, top_seek_keys_ = 0;
};

class Tree {
 public:
  Tree(const RootFile& f, const Key& key) : file_(&f), name_(key.name) {
    const std::vector<uint8_t> d = f.payload(key);
    uint32_t bits = 0;
    entries_ = detail::i64(d, detail::skip_named_and_attributes(d, &bits, "TTree"));
    for (const Key& k : f.walk()) {
      if (k.class_name != "TBasket" || k.title != name_) continue;
      Basket b;
      b.key = k;
      b.nev_buf_size = detail::i32(f.data(), k.header_end + 6);
      b.nev_buf = detail::i32(f.data(), k.header_end + 10);
      b.last = detail::i32(f.data(), k.header_end + 14);
      baskets_.push_back(b);
    }
  }

  int64_t entries() const { return entries_; }

  /* One fixed-size value per entry (a leaf such as x/D, x/F, x/I); T is the
   * value's C type, as SetBranchAddress takes it. */
  template <typename T>
  std::vector<T> array(const std::string& branch) const {
    std::vector<T> out;
    for (const Basket* b : branch_baskets(branch)) {
      const std::vector<uint8_t> d = file_->payload(b->key);
      const int64_t data_len = b->last - b->key.keylen;
      if (data_len != int64_t(d.size()))
        throw FormatError(file_->path() + ": branch " + branch + " has entries of varying size");
      if (data_len != int64_t(b->nev_buf) * int64_t(sizeof(T)))
        throw FormatError(file_->path() + ": branch " + branch + ": basket size does not match the value type");
      for (int32_t i = 0; i < b->nev_buf; ++i) out.push_back(detail::value<T>(d, sizeof(T) * size_t(i)));
    }
    return out;
  }

  /* A std::vector<T> branch: one vector per entry. */
  template <typename T>
  std::vector<std::vector<T>> vectors(const std::string& branch) const {
    std::vector<std::vector<T>> out;
    for (const Basket* b : branch_baskets(branch)) {
      const std::vector<uint8_t> d = file_->payload(b->key);
      const int64_t kl = b->key.keylen, data_len = b->last - kl;
      if (data_len < 0 || data_len >= int64_t(d.size()))
        throw FormatError(file_->path() + ": branch " + branch + " has no entry offsets");
      const int32_t cnt = detail::i32(d, size_t(data_len));
      if (cnt < b->nev_buf) throw FormatError(file_->path() + ": branch " + branch + ": too few entry offsets");
      for (int32_t i = 0; i < b->nev_buf; ++i) {
        const int64_t s = detail::i32(d, size_t(data_len + 4 + 4 * i)) - kl;
        const int64_t e = i + 1 < b->nev_buf ? detail::i32(d, size_t(data_len + 8 + 4 * i)) - kl : data_len;
        if (s < 0 || e > data_len || s + 10 > e)
          throw FormatError(file_->path() + ": branch " + branch + ": entry offsets out of range");
        const uint32_t bc = detail::u32(d, size_t(s));
        const int32_t n = detail::i32(d, size_t(s + 6));
        if (!(bc & detail::kByteCount) || s + 4 + int64_t(bc & ~detail::kByteCount) != e || n < 0 ||
            s + 10 + int64_t(n) * int64_t(sizeof(T)) != e)
          throw FormatError(file_->path() + ": branch " + branch + ": malformed vector entry");
        std::vector<T> v(static_cast<size_t>(n));
        for (int32_t j = 0; j < n; ++j) v[size_t(j)] = detail::value<T>(d, size_t(s + 10) + sizeof(T) * size_t(j));
        out.push_back(std::move(v));
      }
    }
    return out;
  }

 private:
  struct Basket {
    Key key;
    int32_t nev_buf_size = 0, nev_buf = 0, last = 0;
  };

  std::vector<const Basket*> branch_baskets(const std::string& branch) const {
    std::vector<const Basket*> out;
    int64_t total = 0;
    for (const Basket& b : baskets_)
      if (b.key.name == branch) {
        out.push_back(&b);
        total += b.nev_buf;
      }
    if (out.empty()) throw FormatError(file_->path() + ": tree " + name_ + " has no baskets of branch " + branch);
    if (total != entries_)
      throw FormatError(file_->path() + ": branch " + branch + " holds " + std::to_string(total) +
                        " entries in its basket keys, tree " + name_ + " has " + std::to_string(entries_));
    return out;
  }

  const RootFile* file_;
  std::string name_;
  int64_t entries_ = 0;
  std::vector<Basket> baskets_;
};

inline Tree RootFile::tree(const std::string& path) const {
  const Key k = get_key(path);
  if (k.class_name != "TTree") throw FormatError(path_ + ": " + path + " is a " + k.class_name + ", not a TTree");
  return Tree(*this, k);
}

/* TGraph::Eval's linear rule: the two neighbours of x (the two nearest
 * points on one side outside the abscissa range); an unsorted graph returns a
 * point's own y where x equals its abscissa. */
inline double graph_eval(const Graph& g, double x) {
  const std::vector<double>& X = g.x;
  const std::vector<double>& Y = g.y;
  const long n = long(X.size());
  if (n == 0) return 0.0;
  if (n == 1) return Y[0];
  long low = -1, up = -1;
  if (g.bits & kIsSortedX) {
    low = long(std::upper_bound(X.begin(), X.end(), x) - X.begin()) - 1;
    if (low == n - 1) {
      up = low;
      low = up - 1;
    } else if (low == -1) {
      low = 0;
      up = 1;
    } else {
      up = low + 1;
    }
  } else {
    long low2 = -1, up2 = -1;
    for (long i = 0; i < n; ++i) {
      if (X[size_t(i)] < x) {
        if (low == -1 || X[size_t(i)] > X[size_t(low)]) {
          low2 = low;
          low = i;
        } else if (low2 == -1) {
          low2 = i;
        }
      } else if (X[size_t(i)] > x) {
        if (up == -1 || X[size_t(i)] < X[size_t(up)]) {
          up2 = up;
          up = i;
        } else if (up2 == -1) {
          up2 = i;
        }
      } else {
        return Y[size_t(i)];
      }
    }
    if (up == -1) {
      up = low;
      low = low2;
    }
    if (low == -1) {
      low = up;
      up = up2;
    }
  }
  const size_t l = size_t(low), u = size_t(up);
  if (X[l] == X[u]) return Y[l];
  return Y[u] + (x - X[u]) * (Y[l] - Y[u]) / (X[l] - X[u]);
}

}  // namespace rootio

constexpr int kIoSamples = 10;
constexpr int kIoNfreq = 25;           // ns between samples
constexpr int kIoIdstart = 150 + 13;   // first sample in the waveform (ns)
constexpr double kIoTau = 43.0;        // CRRC shaping time for the noise correlation (ns)
constexpr double kIoTailStart = 800.0; // the shape switches to the exponential tail here (ns)
constexpr double kIoPedrms = 1.0;      // the driver's pederr

class Pulse {
 public:
  explicit Pulse(const std::string& shape_file) {
    const rootio::RootFile f(shape_file);
    graph_ = f.graph("PulseShape/grPulseShape");
    const rootio::Tree tail = f.tree("PulseShape/Tail");
    tmin_ = tail.array<float>("timeMin").at(0);
    par0_ = tail.array<float>("expAmplitude").at(0);
    par1_ = tail.array<float>("expTime").at(0);
    for (int i = 0; i < kIoSamples; ++i) {
      const double y = 1. - std::exp(-double(kIoNfreq * i) / (std::sqrt(2.) * kIoTau));
      mC_[size_t(i)] = 1. - y * y;
    }
  }
  double fShape(double x) const {
    if (x > 0.) {
      if (x < kIoTailStart) {
        const double y = rootio::graph_eval(graph_, x);
        return y <= 0 ? 0. : y;
      }
      return par0_ * std::exp(-x * par1_);
    }
    return 0.;
  }
  double corr(int i) const { return mC_.at(size_t(i)); }
  float tMin() const { return tmin_; }
  float fPar0() const { return par0_; }
  float fPar1() const { return par1_; }
  const rootio::Graph& graph() const { return graph_; }

 private:
  rootio::Graph graph_;
  float tmin_ = 0, par0_ = 0, par1_ = 0;
  std::array<double, kIoSamples> mC_{};
};

/* fullpulse(7 + i) = fShape(IDSTART + NFREQ*(i+3) + NFREQ - 250), i < 12. */
inline std::array<double, kIoSamples + 9> driver_fullpulse(const Pulse& p) {
  std::array<double, kIoSamples + 9> fp{};
  for (int i = 0; i < kIoSamples + 2; ++i)
    fp[size_t(i + 7)] = p.fShape(double(kIoIdstart + kIoNfreq * (i + 3) + kIoNfreq - 500 / 2));
  return fp;
}

/* noisecor(i, j) = corr(|i - j|), row-major (symmetric). */
inline std::array<double, kIoSamples * kIoSamples> driver_noisecor(const Pulse& p) {
  std::array<double, kIoSamples * kIoSamples> R{};
  for (int i = 0; i < kIoSamples; ++i)
    for (int j = 0; j < kIoSamples; ++j) R[size_t(i * kIoSamples + j)] = p.corr(std::abs(j - i));
  return R;
}

constexpr std::array<int, kIoSamples> kIoActiveBxs = {-5, -4, -3, -2, -1, 0, 1, 2, 3, 4};

class ecal_data_io {  // NOLINT(readability-identifier-naming): the reference's class name
 public:
  using input_vector_type = std::array<double, kIoSamples>;
  using pulse_matrix_type = std::array<double, kIoSamples * kIoSamples>;  // column-major, as Eigen's default
  using entry_type = std::pair<input_vector_type, pulse_matrix_type>;

  ecal_data_io(const std::string& file_name, const std::string& shape_file) : pulse_(shape_file) {
    const rootio::RootFile f(file_name);
    const rootio::Tree t = f.tree("Samples");
    truth_ = t.array<double>("amplitudeTruth");
    const std::vector<std::vector<double>> vecs = t.vectors<double>("samples");
    samples_.assign(vecs.size(), input_vector_type{});
    for (size_t e = 0; e < vecs.size(); ++e) {
      if (vecs[e].size() > size_t(kIoSamples)) throw rootio::FormatError(file_name + ": entry with over 10 samples");
      std::copy(vecs[e].begin(), vecs[e].end(), samples_[e].begin());
    }
    // io/src/ecal_data_io.cpp:26-41: column ip (bx) holds the extended pulse
    // from sample max(0, bx+3) on, at offset 7 - 3 - bx
    fullpulse_ = driver_fullpulse(pulse_);
    for (int ip = 0; ip < kIoSamples; ++ip) {
      const int bx = kIoActiveBxs[size_t(ip)];
      const int first = std::max(0, bx + 3), offset = 7 - 3 - bx;
      for (int i = first; i < kIoSamples; ++i)
        pulse_matrix_[size_t(ip * kIoSamples + i)] = fullpulse_[size_t(i + offset)];
    }
  }

  entry_type get_one_entry() {
    const size_t i = size_t(ientry_ % int64_t(samples_.size()));
    ++ientry_;
    return {samples_[i], pulse_matrix_};
  }
  std::vector<entry_type> get_n_entries(int n) {
    std::vector<entry_type> out;
    for (int i = 0; i < n; ++i) out.push_back(get_one_entry());
    return out;
  }

  int64_t entries() const { return int64_t(samples_.size()); }
  const std::vector<double>& truth() const { return truth_; }
  const std::vector<input_vector_type>& samples() const { return samples_; }
  const Pulse& pulse() const { return pulse_; }
  const std::array<double, kIoSamples + 9>& fullpulse() const { return fullpulse_; }
  const pulse_matrix_type& pulse_matrix() const { return pulse_matrix_; }

 private:
  Pulse pulse_;
  std::vector<double> truth_;
  std::vector<input_vector_type> samples_;
  std::array<double, kIoSamples + 9> fullpulse_{};
  pulse_matrix_type pulse_matrix_{};
  int64_t ientry_ = 0;
};

}  // namespace mfgb

#endif  // MULTIFIT_GB300_IO_HPP
