// Corrupted-file harness for the array-file reader (jams_gb300/csrc/llg_io.cu),
// built by tests/test_io_asan.py with AddressSanitizer and UBSan: any read
// outside the file buffer or undefined behaviour aborts the run.  It writes
// valid files with the library's own writer, then reads back seeded
// corruptions of them (bit flips, zeroed and saturated spans, truncations,
// repeated spans) and counts the status codes.
//
//   io_fuzz_harness <dir> <cases> <seed> [more base files ...]
//
// The optional files (chunked, filtered HDF5 files that the library does
// not write) join the bases; their dataset must be named "spins".
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <random>
#include <string>
#include <vector>

#include "../jams_gb300/csrc/llg_io.h"

static std::vector<uint8_t> slurp(const std::string& p) {
  std::vector<uint8_t> b;
  FILE* f = std::fopen(p.c_str(), "rb");
  if (!f) return b;
  int c;
  while ((c = std::fgetc(f)) != EOF) b.push_back((uint8_t)c);
  std::fclose(f);
  return b;
}

int main(int argc, char** argv) {
  if (argc < 4) return 2;
  const std::string dir = argv[1];
  const long cases = std::atol(argv[2]);
  std::mt19937_64 rng(std::strtoull(argv[3], nullptr, 10));
  std::vector<double> spins(300), flat(37);
  for (size_t i = 0; i < spins.size(); ++i) spins[i] = std::sin(0.37 * (double)i);
  for (size_t i = 0; i < flat.size(); ++i) flat[i] = (double)i;
  struct Base {
    std::string path;
    std::vector<uint8_t> bytes;
  };
  std::vector<Base> bases;
  const struct {
    const char* name;
    const double* data;
    int64_t rows, cols;
  } files[] = {{"spins.h5", spins.data(), 100, 3}, {"flat.h5", flat.data(), 37, 1},
               {"two.h5", spins.data(), 50, 3}, {"spins.txt", spins.data(), 20, 3}};
  for (const auto& f : files) {
    std::string err;
    std::vector<llgio::Dataset> sets{{"spins", f.data, f.rows, f.cols}};
    if (std::string(f.name) == "two.h5") sets.push_back({"other", flat.data(), 37, 1});
    const std::string p = dir + "/" + f.name;
    if (llgio::write_array(p, sets, err)) {
      std::fprintf(stderr, "write %s: %s\n", p.c_str(), err.c_str());
      return 3;
    }
    bases.push_back({p, slurp(p)});
  }
  for (int a = 4; a < argc; ++a) {
    bases.push_back({argv[a], slurp(argv[a])});
    if (bases.back().bytes.empty()) return 3;
  }
  std::map<int, long> codes;
  for (long it = 0; it < cases; ++it) {
    const Base& b = bases[(size_t)it % bases.size()];
    std::vector<uint8_t> d = b.bytes;
    const int nops = 1 + (int)(rng() % 6);
    for (int k = 0; k < nops && !d.empty(); ++k) {
      const size_t i = rng() % d.size();
      const size_t len = 1 + rng() % 16;
      const size_t e = std::min(d.size(), i + len);
      switch (rng() % 6) {
        case 0: d[i] ^= (uint8_t)(1u << (rng() % 8)); break;
        case 1: for (size_t j = i; j < e; ++j) d[j] = 0; break;
        case 2: for (size_t j = i; j < e; ++j) d[j] = 0xff; break;
        case 3: d.resize(i); break;
        case 4: {
          std::vector<uint8_t> span(d.begin() + (long)i, d.begin() + (long)e);
          d.insert(d.begin() + (long)i, span.begin(), span.end());
          break;
        }
        default: d[i] = (uint8_t)(rng() % 256); break;
      }
    }
    const std::string bad = dir + (b.path.size() > 3 && b.path.substr(b.path.size() - 3) == ".h5" ? "/bad.h5" : "/bad.txt");
    FILE* f = std::fopen(bad.c_str(), "wb");
    if (!f) return 4;
    if (!d.empty()) std::fwrite(d.data(), 1, d.size(), f);
    std::fclose(f);
    std::vector<double> out;
    int64_t rows = -1, cols = -1;
    std::string err;
    const int rc = llgio::read_array(bad, "spins", out, rows, cols, err);
    if (rc == 0 && (rows < 0 || cols < 0 || (int64_t)out.size() != rows * cols)) {
      std::fprintf(stderr, "case %ld: %lld x %lld but %zu values\n", it, (long long)rows, (long long)cols,
                   out.size());
      return 5;
    }
    if (rc != 0 && err.empty()) {
      std::fprintf(stderr, "case %ld: error without a message\n", it);
      return 6;
    }
    ++codes[rc];
  }
  std::printf("codes");
  for (auto& c : codes) std::printf(" %d:%ld", c.first, c.second);
  std::printf("\n");
  return 0;
}
