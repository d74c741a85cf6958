// Checks of the C++ ROOT-format reader (include/multifit_gb300_io.hpp), run
// by tests/test_rootio_cpp.py on the CPU.
//
//   rootio_check inflate <streams.bin>
//       streams.bin: records of [u64 raw length][u64 stream length][zlib
//       stream][raw bytes] (little-endian lengths); inflates every stream and
//       compares it with its raw bytes.
//   rootio_check dump <Samples file> <pulse-shape file> <out.bin>
//       reads the file as the reference driver does (ecal_data_io) and writes
//       entries (i64), samples [entries][10], truth [entries], fullpulse [19],
//       noisecor [10][10], pulse matrix [10][10] column-major, the Tail
//       parameters [3] (f64, native byte order), and the graph's point count
//       and sorted flag (i64 each).
//   rootio_check expect-error <file> <tree> <branch> <substring>
//       reading the branch must throw a FormatError whose message contains the
//       substring.
//   rootio_check branches <file> <out.bin>
//       the Samples tree's amplitudeTruth and samples branches: writes
//       i64 entries, entries f64 truth values, then per entry i64 length and
//       that many f64 samples; or exits 3 with the FormatError message.
//   rootio_check patch-compression <file> <branch>
//       the branch's first basket with its "ZL" block tag changed to "L4" must
//       be refused.
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "multifit_gb300_io.hpp"

namespace {

std::vector<uint8_t> read_all(const char* path) {
  std::ifstream f(path, std::ios::binary);
  return std::vector<uint8_t>(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
}

template <typename T>
void put(std::ofstream& f, const T& v) {
  f.write(reinterpret_cast<const char*>(&v), sizeof(T));
}

int inflate_check(const char* path) {
  const std::vector<uint8_t> d = read_all(path);
  size_t p = 0;
  int n = 0;
  while (p + 16 <= d.size()) {
    uint64_t raw = 0, comp = 0;
    std::memcpy(&raw, &d[p], 8);
    std::memcpy(&comp, &d[p + 8], 8);
    p += 16;
    const std::vector<uint8_t> got = mfgb::rootio::detail::zlib_inflate(d.data() + p, comp, raw);
    if (got.size() != raw || std::memcmp(got.data(), d.data() + p + comp, raw) != 0) {
      std::printf("mismatch in stream %d (raw %llu bytes, inflated %zu)\n", n, (unsigned long long)raw, got.size());
      return 1;
    }
    p += comp + raw;
    ++n;
  }
  std::printf("ok %d\n", n);
  return 0;
}

int dump(const char* samples_file, const char* shape_file, const char* out_path) {
  mfgb::ecal_data_io io(samples_file, shape_file);
  std::ofstream f(out_path, std::ios::binary);
  put(f, int64_t(io.entries()));
  for (const auto& s : io.samples())
    for (double v : s) put(f, v);
  for (double v : io.truth()) put(f, v);
  for (double v : io.fullpulse()) put(f, v);
  for (double v : mfgb::driver_noisecor(io.pulse())) put(f, v);
  for (double v : io.pulse_matrix()) put(f, v);
  put(f, double(io.pulse().tMin()));
  put(f, double(io.pulse().fPar0()));
  put(f, double(io.pulse().fPar1()));
  put(f, int64_t(io.pulse().graph().x.size()));
  put(f, int64_t((io.pulse().graph().bits & mfgb::rootio::kIsSortedX) ? 1 : 0));
  // round robin as ecal_data_io::get_n_entries
  const auto ents = io.get_n_entries(int(io.entries()) + 3);
  if (ents.back().first != io.samples()[2]) {
    std::printf("round robin broken\n");
    return 1;
  }
  std::printf("entries %lld\n", (long long)io.entries());
  return 0;
}

int expect_error(const char* path, const char* tree, const char* branch, const char* what) {
  try {
    const mfgb::rootio::RootFile f(path);
    const mfgb::rootio::Tree t = f.tree(tree);
    t.vectors<double>(branch);
  } catch (const mfgb::rootio::FormatError& e) {
    std::printf("error: %s\n", e.what());
    return std::strstr(e.what(), what) ? 0 : 1;
  }
  std::printf("no error\n");
  return 1;
}

int branches(const char* path, const char* out_path) {
  try {
    const mfgb::rootio::RootFile f(path);
    const mfgb::rootio::Tree t = f.tree("Samples");
    const std::vector<double> truth = t.array<double>("amplitudeTruth");
    const std::vector<std::vector<double>> vecs = t.vectors<double>("samples");
    std::ofstream o(out_path, std::ios::binary);
    put(o, int64_t(truth.size()));
    for (double v : truth) put(o, v);
    put(o, int64_t(vecs.size()));
    for (const auto& v : vecs) {
      put(o, int64_t(v.size()));
      for (double x : v) put(o, x);
    }
  } catch (const mfgb::rootio::FormatError& e) {
    std::printf("error: %s\n", e.what());
    return 3;
  }
  return 0;
}

int patch_compression(const char* path, const char* branch) {
  std::vector<uint8_t> d = read_all(path);
  const mfgb::rootio::RootFile f(d, path);
  for (const auto& k : f.walk()) {
    if (k.class_name == "TBasket" && k.name == branch) {
      const size_t p = size_t(k.seek_key + k.keylen);
      if (d[p] != 'Z' || d[p + 1] != 'L') return 1;
      d[p] = 'L';
      d[p + 1] = '4';
      break;
    }
  }
  try {
    const mfgb::rootio::RootFile g(d, "patched");
    g.tree("Samples").vectors<double>(branch);
  } catch (const mfgb::rootio::FormatError& e) {
    std::printf("error: %s\n", e.what());
    return std::strstr(e.what(), "not supported") ? 0 : 1;
  }
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    const std::string mode = argc > 1 ? argv[1] : "";
    if (mode == "inflate" && argc == 3) return inflate_check(argv[2]);
    if (mode == "dump" && argc == 5) return dump(argv[2], argv[3], argv[4]);
    if (mode == "expect-error" && argc == 6) return expect_error(argv[2], argv[3], argv[4], argv[5]);
    if (mode == "patch-compression" && argc == 4) return patch_compression(argv[2], argv[3]);
    if (mode == "branches" && argc == 4) return branches(argv[2], argv[3]);
  } catch (const std::exception& e) {
    std::printf("exception: %s\n", e.what());
    return 2;
  }
  std::fprintf(stderr, "usage: rootio_check inflate|dump|expect-error|patch-compression|branches ...\n");
  return 2;
}
