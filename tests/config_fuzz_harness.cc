// Malformed-config harness for the config front end (jams_gb300/csrc/llg_config.cu),
// built by tests/test_config_asan.py with AddressSanitizer and UBSan: any
// out-of-bounds access or undefined behaviour aborts the run.  It reads base
// config texts from files, applies seeded mutations (truncations, deleted,
// repeated and replaced spans, stray grammar characters), sends each through
// llg_config_describe (some with a mutated patch) and counts the status
// codes.  The library entry points the describe path never reaches are
// stubs here.
//
//   config_fuzz_harness <cases> <seed> <config file>...
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "../include/jams_llg.h"

namespace jams_llg {
static std::string g_err;
void set_thread_error(const char* msg) { g_err = msg ? msg : ""; }
void set_max_steps(llg_handle*, int64_t) {}
}  // namespace jams_llg

extern "C" {
int llg_create(const llg_desc*, llg_handle** out) {
  if (out) *out = nullptr;
  return LLG_ERR_NO_DEVICE;
}
void llg_destroy(llg_handle*) {}
int llg_set_state(llg_handle*, int32_t, const double*) { return LLG_ERR_NO_DEVICE; }
}

int main(int argc, char** argv) {
  if (argc < 4) return 2;
  const long cases = std::atol(argv[1]);
  std::mt19937_64 rng(std::strtoull(argv[2], nullptr, 10));
  std::vector<std::string> bases;
  for (int a = 3; a < argc; ++a) {
    std::ifstream f(argv[a]);
    std::stringstream ss;
    ss << f.rdbuf();
    bases.push_back(ss.str());
  }
  const std::string alphabet = "{}()[];:=\",.-+0123456789eE/*#\n\t abcdefghijklmnopqrstuvwxyz_";
  auto mutate = [&](std::string t) {
    const int nops = 1 + (int)(rng() % 4);
    for (int k = 0; k < nops && !t.empty(); ++k) {
      const size_t i = rng() % t.size();
      const size_t len = 1 + rng() % 12;
      switch (rng() % 5) {
        case 0: t.resize(i); break;
        case 1: t.erase(i, len); break;
        case 2: {
          const std::string span = t.substr(i, len);
          const int rep = 2 + (int)(rng() % 3);
          for (int r = 0; r < rep; ++r) t.insert(i, span);
          break;
        }
        case 3: t[i] = alphabet[rng() % alphabet.size()]; break;
        default: {
          std::string ins;
          for (size_t j = 0; j < len; ++j) ins += alphabet[rng() % alphabet.size()];
          t.insert(i, ins);
          break;
        }
      }
    }
    return t;
  };
  const size_t cap = 1 << 20, guard = 4096;
  std::vector<char> buf(cap + guard);
  std::map<int, long> codes;
  for (long it = 0; it < cases; ++it) {
    const std::string text = mutate(bases[(size_t)it % bases.size()]);
    const std::string patch = it % 5 == 0 ? mutate("physics : { temperature = 50.0; };") : std::string();
    std::memset(buf.data() + cap, 0x5a, guard);
    const int rc = llg_config_describe(text.c_str(), patch.c_str(), buf.data(), (int64_t)cap);
    for (size_t j = cap; j < cap + guard; ++j)
      if (buf[j] != 0x5a) {
        std::fprintf(stderr, "case %ld wrote past the buffer\n", it);
        return 5;
      }
    if (rc != 0 && jams_llg::g_err.empty()) {
      std::fprintf(stderr, "case %ld: error %d without a message\n", it, rc);
      return 6;
    }
    jams_llg::g_err.clear();
    ++codes[rc];
  }
  std::printf("codes");
  for (auto& c : codes) std::printf(" %d:%ld", c.first, c.second);
  std::printf("\n");
  return 0;
}
