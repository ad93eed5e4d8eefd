// JAMS config-file front end for libjams_llg.so (host C++).
//
// Reads the libconfig-format configuration JAMS takes on its command line
// (plus optional patch strings, merged as src/jams/interface/config.cc:15-167
// does) and builds the llg_desc of the LLG hot path:
//   materials        src/jams/containers/material.h:29-58
//   unitcell         src/jams/core/lattice.cc:257-290, 356-420 (basis vectors
//                    are the columns of the unit-cell matrix)
//   lattice          src/jams/core/lattice.cc:421-430 (size, periodic)
//   hamiltonians     exchange (src/jams/hamiltonian/exchange.cc:15-171 and
//                    src/jams/core/interactions.cc:128-348), uniaxial
//                    (uniaxial_anisotropy.cc:48-118), cubic
//                    (cubic_anisotropy.cc:40-125), applied-field with
//                    its static / sinc / sinc-cos types
//                    (applied_field.cc:10-124), zeeman dc and ac fields
//                    (zeeman.cc:12-71)
//   solver           t_step / t_max in seconds, module, gilbert_prefactor
//                    (src/jams/solvers/cuda_llg_heun.cu:21-35)
//   physics          temperature (src/jams/core/physics.cc:79-100)
//   sim              seed
// libconfig itself is not available in this image; the parser below reads the
// same grammar (groups, lists, arrays, scalars, comments, string
// concatenation, '=' or ':' assignment, ';' or ',' separators).
//
// Symmetry operations: the reference asks spglib for the space group and
// keeps, per basis site, the rotations of the operations without
// translation that fix the site modulo a lattice vector
// (src/jams/core/lattice.cc:1127-1152).  Here the site point group is found
// directly: integer matrices R (entries -1, 0, 1) in fractional coordinates
// that preserve the lattice metric, for which x -> R x + (p - R p) maps every
// basis site onto a basis site of the same material; the partner of an
// expanded interaction is the site its rotated vector reaches.  On cells
// whose site symmetries need no centring translation (simple cubic, bcc,
// primitive cells, the triangular monolayer) this is the reference's set;
// on centred conventional cells (the 4-site fcc cell) the reference drops
// the operations with a centring translation and keeps the original partner,
// which leaves sites with incomplete or inconsistent neighbour lists.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/jams_llg.h"

namespace jams_llg {
void set_thread_error(const char* msg);
void set_max_steps(llg_handle* h, int64_t max_steps);
}

namespace {

// ---------------------------------------------------------------- parser --

struct CfgError : std::runtime_error {
  explicit CfgError(const std::string& m) : std::runtime_error(m) {}
};

struct Node {
  enum Type { None, Int, Float, Bool, String, Group, Array, List };
  Type type = None;
  std::string name;
  long long i = 0;
  double f = 0.0;
  bool b = false;
  std::string s;
  std::vector<Node> kids;

  bool is_number() const { return type == Int || type == Float; }
  bool is_aggregate() const { return type == Group || type == Array || type == List; }
  const Node* find(const std::string& n) const {
    for (auto& k : kids)
      if (k.name == n) return &k;
    return nullptr;
  }
  Node* find(const std::string& n) {
    for (auto& k : kids)
      if (k.name == n) return &k;
    return nullptr;
  }
  const Node& at(const std::string& n) const {
    const Node* p = find(n);
    if (!p) throw CfgError("setting '" + n + "' not found in '" + name + "'");
    return *p;
  }
  const Node& at(size_t k) const {
    if (k >= kids.size()) throw CfgError("index " + std::to_string(k) + " out of range in '" + name + "'");
    return kids[k];
  }
  size_t size() const { return kids.size(); }
  double num() const {
    if (type == Int) return (double)i;
    if (type == Float) return f;
    if (type == Bool) return b ? 1.0 : 0.0;
    throw CfgError("setting '" + name + "' is not a number");
  }
  bool boolean() const {
    if (type == Bool) return b;
    if (type == Int) return i != 0;
    throw CfgError("setting '" + name + "' is not a boolean");
  }
  const std::string& str() const {
    if (type != String) throw CfgError("setting '" + name + "' is not a string");
    return s;
  }
};

class Parser {
 public:
  explicit Parser(const std::string& t) : t_(t) {}

  Node parse_root() {
    Node root;
    root.type = Node::Group;
    parse_settings(root, '\0');
    return root;
  }

 private:
  const std::string& t_;
  size_t p_ = 0;
  int line_ = 1;

  [[noreturn]] void fail(const std::string& what) {
    throw CfgError("config parse error at line " + std::to_string(line_) + ": " + what);
  }

  void skip() {
    for (;;) {
      while (p_ < t_.size() && std::isspace((unsigned char)t_[p_])) {
        if (t_[p_] == '\n') ++line_;
        ++p_;
      }
      if (p_ >= t_.size()) return;
      if (t_[p_] == '#' || (t_[p_] == '/' && p_ + 1 < t_.size() && t_[p_ + 1] == '/')) {
        while (p_ < t_.size() && t_[p_] != '\n') ++p_;
        continue;
      }
      if (t_[p_] == '/' && p_ + 1 < t_.size() && t_[p_ + 1] == '*') {
        size_t e = t_.find("*/", p_ + 2);
        if (e == std::string::npos) fail("unterminated comment");
        for (size_t k = p_; k < e; ++k)
          if (t_[k] == '\n') ++line_;
        p_ = e + 2;
        continue;
      }
      return;
    }
  }

  char peek() {
    skip();
    return p_ < t_.size() ? t_[p_] : '\0';
  }

  std::string name() {
    skip();
    size_t s = p_;
    if (p_ < t_.size() && (std::isalpha((unsigned char)t_[p_]) || t_[p_] == '*')) {
      ++p_;
      while (p_ < t_.size() &&
             (std::isalnum((unsigned char)t_[p_]) || t_[p_] == '_' || t_[p_] == '-' || t_[p_] == '*'))
        ++p_;
    }
    if (s == p_) fail("expected a setting name");
    return t_.substr(s, p_ - s);
  }

  // settings of a group until `close` ('}' or end of text)
  void parse_settings(Node& g, char close) {
    for (;;) {
      char c = peek();
      if (c == close) {
        if (close) ++p_;
        return;
      }
      if (c == '\0') fail(close ? "missing '}'" : "unexpected end");
      Node n;
      n.name = name();
      c = peek();
      if (c != '=' && c != ':') fail("expected '=' or ':' after '" + n.name + "'");
      ++p_;
      parse_value(n);
      c = peek();
      if (c == ';' || c == ',') ++p_;
      if (g.find(n.name)) fail("duplicate setting '" + n.name + "'");
      g.kids.push_back(std::move(n));
    }
  }

  void parse_value(Node& n) {
    char c = peek();
    if (c == '{') {
      ++p_;
      n.type = Node::Group;
      parse_settings(n, '}');
    } else if (c == '(' || c == '[') {
      const char close = c == '(' ? ')' : ']';
      n.type = c == '(' ? Node::List : Node::Array;
      ++p_;
      for (;;) {
        if (peek() == close) {
          ++p_;
          break;
        }
        Node e;
        parse_value(e);
        if (n.type == Node::Array && e.is_aggregate()) fail("arrays hold scalars only");
        n.kids.push_back(std::move(e));
        char d = peek();
        if (d == ',') {
          ++p_;
        } else if (d != close) {
          fail(std::string("expected ',' or '") + close + "'");
        }
      }
    } else if (c == '"') {
      n.type = Node::String;
      while (peek() == '"') {  // adjacent strings concatenate
        ++p_;
        while (p_ < t_.size() && t_[p_] != '"') {
          if (t_[p_] == '\\' && p_ + 1 < t_.size()) {
            const char e = t_[++p_];
            n.s += e == 'n' ? '\n' : e == 't' ? '\t' : e;
          } else {
            if (t_[p_] == '\n') ++line_;
            n.s += t_[p_];
          }
          ++p_;
        }
        if (p_ >= t_.size()) fail("unterminated string");
        ++p_;
      }
    } else {
      skip();
      size_t s = p_;
      while (p_ < t_.size() && (std::isalnum((unsigned char)t_[p_]) || strchr("+-._", t_[p_]))) ++p_;
      std::string tok = t_.substr(s, p_ - s);
      if (tok.empty()) fail("expected a value");
      std::string low = tok;
      for (auto& ch : low) ch = (char)std::tolower((unsigned char)ch);
      if (low == "true" || low == "false") {
        n.type = Node::Bool;
        n.b = low == "true";
        return;
      }
      const bool is_hex = low.size() > 2 && (low.rfind("0x", 0) == 0);
      const bool is_float = !is_hex && low.find_first_of(".e") != std::string::npos;
      // `end` points into the string parsed, so each branch checks it while
      // that string is alive
      if (is_float) {
        n.type = Node::Float;
        char* end = nullptr;
        n.f = strtod(tok.c_str(), &end);
        if (!end || *end != '\0') fail("bad number '" + tok + "'");
      } else {
        std::string digits = tok;
        while (!digits.empty() && (digits.back() == 'L' || digits.back() == 'l')) digits.pop_back();
        n.type = Node::Int;
        char* end = nullptr;
        n.i = strtoll(digits.c_str(), &end, 0);
        if (!end || *end != '\0') fail("bad number '" + digits + "'");
      }
    }
  }
};

// Patch merge (src/jams/interface/config.cc:15-167): groups merge setting by
// setting; scalars replace; lists and arrays merge element by element.
void merge(Node& orig, const Node& patch) {
  if (patch.type == Node::Group) {
    if (orig.type != Node::Group) {
      orig = patch;
      return;
    }
    for (const auto& pk : patch.kids) {
      Node* o = orig.find(pk.name);
      if (o && pk.is_aggregate() && o->is_aggregate() && o->type == pk.type) {
        merge(*o, pk);
      } else if (o) {
        *o = pk;
      } else {
        orig.kids.push_back(pk);
      }
    }
  } else if (patch.type == Node::List || patch.type == Node::Array) {
    if (orig.type != patch.type) {
      std::string n = orig.name;
      orig = patch;
      orig.name = n;
      return;
    }
    for (size_t k = 0; k < patch.kids.size(); ++k) {
      if (k < orig.kids.size()) {
        if (patch.kids[k].is_aggregate() && orig.kids[k].type == patch.kids[k].type)
          merge(orig.kids[k], patch.kids[k]);
        else
          orig.kids[k] = patch.kids[k];
      } else {
        orig.kids.push_back(patch.kids[k]);
      }
    }
  } else {
    std::string n = orig.name;
    orig = patch;
    orig.name = n;
  }
}

// ---------------------------------------------------------- geometry ---

using V3 = std::array<double, 3>;
using M3 = std::array<std::array<double, 3>, 3>;

// src/jams/helpers/consts.h:24-38
constexpr double kElectronGFactor = 2.0023193043625;
constexpr double kHBarIU = 0.6582119569;
constexpr double kBohrMagnetonIU = 0.0578838181;
constexpr double kGyromagneticRatioIU = kElectronGFactor * kBohrMagnetonIU / kHBarIU;
constexpr double kBoltzmannIU = 0.0861733326;
constexpr double kJoule2meV = 6.24150907e21;
constexpr double kmRyd2meV = 13.605693123;
constexpr double kPi = 3.14159265358979323846264338327950288;
constexpr double kLatticeTolerance = 1e-4;  // src/jams/helpers/defaults.h:40

V3 mul(const M3& m, const V3& v) {
  V3 r{};
  for (int i = 0; i < 3; ++i) r[i] = m[i][0] * v[0] + m[i][1] * v[1] + m[i][2] * v[2];
  return r;
}

M3 inverse(const M3& m) {
  const double det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
                     m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                     m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
  if (std::fabs(det) < 1e-12) throw CfgError("unit cell basis is singular");
  M3 r;
  r[0][0] = (m[1][1] * m[2][2] - m[1][2] * m[2][1]) / det;
  r[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) / det;
  r[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) / det;
  r[1][0] = (m[1][2] * m[2][0] - m[1][0] * m[2][2]) / det;
  r[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) / det;
  r[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) / det;
  r[2][0] = (m[1][0] * m[2][1] - m[1][1] * m[2][0]) / det;
  r[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) / det;
  r[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) / det;
  return r;
}

bool approx_eq(const V3& a, const V3& b, double tol) {
  for (int i = 0; i < 3; ++i)
    if (std::fabs(a[i] - b[i]) > tol) return false;
  return true;
}

// fractional coordinate in [0, 1), values within tol of 1 mapped to 0
// (normalise_fractional_coordinate, src/jams/core/lattice.cc:50-64, applied
// after reducing by whole cells)
V3 wrap_frac(V3 r) {
  for (int i = 0; i < 3; ++i) {
    r[i] -= std::floor(r[i]);
    if (std::fabs(r[i] - 1.0) <= kLatticeTolerance) r[i] = 0.0;
  }
  return r;
}

bool same_site(const V3& a, const V3& b) {
  V3 d;
  for (int i = 0; i < 3; ++i) {
    d[i] = a[i] - b[i];
    d[i] -= std::nearbyint(d[i]);
  }
  return approx_eq(d, V3{0, 0, 0}, kLatticeTolerance);
}

struct Basis {
  std::string material;
  int mat = 0;
  V3 frac{};
};

struct Model {
  // lattice
  M3 cell{};        // columns are a1, a2, a3 (units of the lattice parameter)
  double parameter = 0.0;   // lattice parameter (m)
  M3 cell_inv{};
  std::vector<Basis> basis;
  int L[3] = {1, 1, 1};
  int periodic[3] = {1, 1, 1};
  // materials (by material index)
  std::vector<std::string> mat_names;
  std::vector<double> mat_moment, mat_gyro, mat_alpha;
  std::vector<V3> mat_spin;
  std::vector<bool> mat_random;
  // per basis site arrays for the descriptor
  std::vector<double> mus, gyro, alpha;
  // terms
  struct Term {
    llg_term t{};
    std::string module;
    std::vector<int32_t> bi, bj, T;
    std::vector<double> J, K, axis;
    std::vector<double> vectors, positions;   // dipole geometry
    std::vector<double> dc, ac, freq;         // zeeman fields per basis site
  };
  std::vector<Term> terms;
  // solver / physics / sim
  double t_step = 0.0, t_max = 0.0;
  int64_t max_steps = 0;
  int integrator = LLG_HEUN;
  bool gilbert = false;
  double temperature = 0.0;
  uint64_t seed = 0;
  std::string solver_module;
};

double energy_unit(const Node& h) {
  // src/jams/core/units.h:15-27; Hamiltonian default "joules"
  // (src/jams/helpers/defaults.h:25, src/jams/core/hamiltonian.cc:122-134)
  std::string u = "joules";
  if (const Node* n = h.find("energy_units")) u = n->str();
  if (const Node* n = h.find("unit_name")) u = n->str();
  static const std::map<std::string, double> table = {
      {"joules", kJoule2meV}, {"J", kJoule2meV}, {"milli_electron_volts", 1.0}, {"meV", 1.0},
      {"milli_rydbergs", kmRyd2meV}, {"mRyd", kmRyd2meV}, {"rydbergs", kmRyd2meV * 1e3},
      {"Ryd", kmRyd2meV * 1e3}, {"Kelvin", kBoltzmannIU}, {"K", kBoltzmannIU}};
  auto it = table.find(u);
  if (it == table.end()) throw CfgError("energy units: " + u + " is not known");
  return it->second;
}

V3 vec3(const Node& n) {
  if (n.size() != 3) throw CfgError("setting '" + n.name + "' needs 3 components");
  return V3{n.at(0).num(), n.at(1).num(), n.at(2).num()};
}

std::string lower(std::string s) {
  for (auto& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

int material_index(const Model& m, const std::string& name) {
  for (size_t k = 0; k < m.mat_names.size(); ++k)
    if (m.mat_names[k] == name) return (int)k;
  throw CfgError("material " + name + " is not defined");
}

// point group of basis site `site`: the rotations R (integer matrices in
// fractional coordinates) of the symmetry operations x -> R x + t of the
// crystal that fix the site, as the reference takes them from spglib's
// space group (src/jams/core/lattice.cc:1015-1060)
std::vector<std::array<int, 9>> site_point_group(const Model& m, int site) {
  // metric G = A^T A
  M3 G{};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k) G[i][j] += m.cell[k][i] * m.cell[k][j];
  std::vector<std::array<int, 9>> ops;
  std::array<int, 9> R;
  for (int code = 0; code < 19683; ++code) {
    int c = code;
    for (int e = 0; e < 9; ++e) {
      R[e] = c % 3 - 1;
      c /= 3;
    }
    const int det = R[0] * (R[4] * R[8] - R[5] * R[7]) - R[1] * (R[3] * R[8] - R[5] * R[6]) +
                    R[2] * (R[3] * R[7] - R[4] * R[6]);
    if (det != 1 && det != -1) continue;
    // R^T G R == G
    bool metric = true;
    for (int i = 0; i < 3 && metric; ++i)
      for (int j = 0; j < 3 && metric; ++j) {
        double v = 0.0;
        for (int k = 0; k < 3; ++k)
          for (int l = 0; l < 3; ++l) v += R[3 * k + i] * G[k][l] * R[3 * l + j];
        if (std::fabs(v - G[i][j]) > kLatticeTolerance) metric = false;
      }
    if (!metric) continue;
    auto rot = [&](const V3& p) {
      return V3{R[0] * p[0] + R[1] * p[1] + R[2] * p[2], R[3] * p[0] + R[4] * p[1] + R[5] * p[2],
                R[6] * p[0] + R[7] * p[1] + R[8] * p[2]};
    };
    // the operation x -> R x + t that fixes the site: t = p - R p (every
    // symmetry fixing the site has this translation, modulo lattice vectors,
    // including the centring translations of conventional cells)
    const V3 ps = m.basis[site].frac;
    const V3 rp = rot(ps);
    const V3 t{ps[0] - rp[0], ps[1] - rp[1], ps[2] - rp[2]};
    bool maps = true;
    for (auto& b : m.basis) {
      const V3 r = rot(b.frac);
      const V3 q{r[0] + t[0], r[1] + t[1], r[2] + t[2]};
      bool found = false;
      for (auto& b2 : m.basis)
        if (b2.mat == b.mat && same_site(q, b2.frac)) found = true;
      if (!found) {
        maps = false;
        break;
      }
    }
    if (!maps) continue;
    ops.push_back(R);
  }
  return ops;
}

struct Interaction {
  int bi = -1, bj = -1;
  std::string ti, tj;
  V3 r{};  // cartesian, lattice-parameter units
  std::array<double, 9> J{};
};

// A line the interaction-file reader skips (src/jams/helpers/utils.h:115-126):
// fewer than two non-blank characters, or the first of them '#', or the
// first two "//".
bool interaction_line_is_comment(const std::string& line) {
  char c[2];
  int n = 0;
  for (char ch : line)
    if (!std::isspace((unsigned char)ch)) {
      c[n++] = ch;
      if (n == 2) break;
    }
  return n < 2 || c[0] == '#' || (c[0] == '/' && c[1] == '/');
}

// exc_file (src/jams/hamiltonian/exchange.cc:117-131), read as
// discover_interaction_file_format and interactions_from_file
// (src/jams/core/interactions.cc:127-246): the first data line fixes the
// layout for the whole file, 6 columns for a scalar J or 14 for a 3x3
// tensor, and its first two tokens, both integers (KKR: 1-based basis
// sites) or both names (JAMS: material names).  Each data line is read
// token by token; a line that does not read is an error.
std::vector<Interaction> interactions_from_file(const std::string& path, const Model& m, bool& kkr) {
  std::ifstream f(path);
  if (!f) throw CfgError("exchange: failed to open exc_file " + path);
  std::vector<std::string> lines;
  for (std::string line; std::getline(f, line);) lines.push_back(line);
  int ncols = 0;
  for (const std::string& line : lines) {
    if (interaction_line_is_comment(line)) continue;
    std::istringstream is(line);
    std::vector<std::string> tok;
    for (std::string t; is >> t;) tok.push_back(t);
    if (tok.size() != 6 && tok.size() != 14) throw CfgError("interaction file has an incorrect number of columns");
    auto is_int = [](const std::string& s) { return s.find_first_not_of("0123456789") == std::string::npos; };
    if (is_int(tok[0]) != is_int(tok[1])) throw CfgError("failed to discover interaction file format");
    kkr = is_int(tok[0]);
    ncols = (int)tok.size();
    break;
  }
  if (ncols == 0) throw CfgError("failed to discover interaction file format");
  std::vector<Interaction> in;
  for (size_t k = 0; k < lines.size(); ++k) {
    if (interaction_line_is_comment(lines[k])) continue;
    std::istringstream is(lines[k]);
    Interaction I;
    if (kkr) {
      is >> I.bi >> I.bj;
      --I.bi;
      --I.bj;
    } else {
      is >> I.ti >> I.tj;
    }
    is >> I.r[0] >> I.r[1] >> I.r[2];
    if (ncols == 6) {
      double J = 0.0;
      is >> J;
      I.J = {J, 0, 0, 0, J, 0, 0, 0, J};
    } else {
      for (int a = 0; a < 9; ++a) is >> I.J[a];
    }
    if (is.fail()) throw CfgError("failed to read line " + std::to_string(k + 1) + " of interaction file " + path);
    if (kkr && (I.bi < 0 || I.bi >= (int)m.basis.size() || I.bj < 0 || I.bj >= (int)m.basis.size()))
      throw CfgError("interaction basis index out of range");
    in.push_back(I);
  }
  return in;
}

void build_exchange(Model& m, const Node& h, Model::Term& out) {
  const double conv = energy_unit(h);
  bool symops = true;
  if (const Node* n = h.find("symops")) symops = n->boolean();
  double energy_cutoff = 0.0, radius_cutoff = 100.0, prefactor = 1.0, distance_tolerance = kLatticeTolerance;
  if (const Node* n = h.find("energy_cutoff")) energy_cutoff = n->num();
  if (const Node* n = h.find("radius_cutoff")) radius_cutoff = n->num();
  if (const Node* n = h.find("interaction_prefactor")) prefactor = n->num();
  if (const Node* n = h.find("distance_tolerance")) distance_tolerance = n->num();
  std::string coord = "CARTESIAN";
  if (const Node* n = h.find("coordinate_format")) coord = n->str();
  coord = lower(coord);
  if (coord != "cartesian" && coord != "fractional") throw CfgError("Unknown coordinate format " + coord);
  std::vector<Interaction> in;
  bool kkr = false;
  // exc_file first, as the reference checks it first; else the inline list
  const Node* file = h.find("exc_file");
  const Node no_list;
  if (file) in = interactions_from_file(file->str(), m, kkr);
  const Node& list = file ? no_list : h.at("interactions");
  if (!file && (list.type != Node::List || list.size() == 0)) throw CfgError("exchange settings must be a list");

  // interactions_from_settings (src/jams/core/interactions.cc:221-257)
  if (!file) kkr = list.at(0).at(0).is_number();
  for (size_t k = 0; k < list.size(); ++k) {
    const Node& e = list.at(k);
    Interaction I;
    if (kkr) {
      I.bi = (int)e.at(0).num() - 1;
      I.bj = (int)e.at(1).num() - 1;
      if (I.bi < 0 || I.bi >= (int)m.basis.size() || I.bj < 0 || I.bj >= (int)m.basis.size())
        throw CfgError("interaction basis index out of range");
    } else {
      I.ti = e.at(0).str();
      I.tj = e.at(1).str();
    }
    I.r = vec3(e.at(2));
    if (e.size() == 4 && e.at(3).is_number()) {
      const double J = e.at(3).num();
      I.J = {J, 0, 0, 0, J, 0, 0, 0, J};
    } else if (e.size() == 4 && e.at(3).type == Node::Array && e.at(3).size() == 9) {
      for (int a = 0; a < 9; ++a) I.J[a] = e.at(3).at(a).num();
    } else if (e.size() == 12) {
      for (int a = 0; a < 9; ++a) I.J[a] = e.at(3 + a).num();
    } else {
      throw CfgError("interaction energy format is incorrect");
    }
    in.push_back(I);
  }

  // post_process_interactions (src/jams/core/interactions.cc:292-348)
  if (coord == "fractional")
    for (auto& I : in) I.r = mul(m.cell, I.r);
  std::vector<Interaction> done;
  if (!kkr) {
    // every basis site of type_i whose partner at r is of type_j
    for (auto& I : in)
      for (int i = 0; i < (int)m.basis.size(); ++i) {
        if (m.basis[i].material != I.ti) continue;
        const V3 q = mul(m.cell_inv, I.r);
        V3 p{m.basis[i].frac[0] + q[0], m.basis[i].frac[1] + q[1], m.basis[i].frac[2] + q[2]};
        int jj = -1;
        for (int j = 0; j < (int)m.basis.size(); ++j)
          if (same_site(p, m.basis[j].frac)) jj = j;
        if (jj < 0 || m.basis[jj].material != I.tj) continue;
        Interaction J = I;
        J.bi = i;
        J.bj = jj;
        done.push_back(J);
      }
  } else {
    for (auto& I : in) {
      Interaction J = I;
      J.ti = m.basis[I.bi].material;
      J.tj = m.basis[I.bj].material;
      done.push_back(J);
    }
  }
  if (symops) {
    std::vector<Interaction> sym;
    for (auto& I : done) {
      std::vector<V3> pts{I.r};
      const V3 rf = mul(m.cell_inv, I.r);
      for (auto& R : site_point_group(m, I.bi)) {
        const V3 f{R[0] * rf[0] + R[1] * rf[1] + R[2] * rf[2], R[3] * rf[0] + R[4] * rf[1] + R[5] * rf[2],
                   R[6] * rf[0] + R[7] * rf[1] + R[8] * rf[2]};
        const V3 c = mul(m.cell, f);
        bool seen = false;
        for (auto& q : pts)
          if (approx_eq(q, c, kLatticeTolerance)) seen = true;
        if (!seen) pts.push_back(c);
      }
      for (auto& q : pts) {
        Interaction J = I;
        J.r = q;
        // the partner is the site the rotated vector reaches.  The reference
        // keeps the original partner (apply_symops, interactions.cc:24-37),
        // which is the same site whenever the point group maps the partner's
        // sublattice onto itself (bcc, primitive cells) and, in cells where
        // a rotation reaches another sublattice (the conventional fcc cell),
        // gives a non-integer translation that only an assert checks.
        const V3 qf = mul(m.cell_inv, q);
        const V3 p{m.basis[I.bi].frac[0] + qf[0], m.basis[I.bi].frac[1] + qf[1], m.basis[I.bi].frac[2] + qf[2]};
        for (int j = 0; j < (int)m.basis.size(); ++j)
          if (same_site(p, m.basis[j].frac) && m.basis[j].material == I.tj) J.bj = j;
        sym.push_back(J);
      }
    }
    done.swap(sym);
  }
  // predicates: energy and radius cut-offs
  std::vector<Interaction> kept;
  for (auto& I : done) {
    double mx = 0.0;
    for (double v : I.J) mx = std::max(mx, std::fabs(v));
    if (energy_cutoff > 0.0 && mx < energy_cutoff * (1.0 - 1e-15)) continue;
    const double rn = std::sqrt(I.r[0] * I.r[0] + I.r[1] * I.r[1] + I.r[2] * I.r[2]);
    if (radius_cutoff > 0.0 && rn > radius_cutoff * (1.0 + kLatticeTolerance)) continue;
    kept.push_back(I);
  }
  // lattice translation vectors: T = r_frac + p_i - p_j
  for (auto& I : kept) {
    const V3 rf = mul(m.cell_inv, I.r);
    int T[3];
    for (int l = 0; l < 3; ++l) {
      const double v = rf[l] + m.basis[I.bi].frac[l] - m.basis[I.bj].frac[l];
      const double n = std::nearbyint(v);
      if (std::fabs(v - n) > distance_tolerance)
        throw CfgError("interaction vector does not join two lattice sites");
      T[l] = (int)n;
    }
    // value in meV (exchange.cc:162-169): prefactor x unit conversion x J
    double mx = 0.0;
    std::array<double, 9> Jm;
    for (int a = 0; a < 9; ++a) {
      Jm[a] = prefactor * conv * I.J[a];
      mx = std::max(mx, std::fabs(Jm[a]));
    }
    if (!(mx > energy_cutoff * conv)) continue;
    out.bi.push_back(I.bi);
    out.bj.push_back(I.bj);
    for (int l = 0; l < 3; ++l) out.T.push_back(T[l]);
    for (int a = 0; a < 9; ++a) out.J.push_back(Jm[a]);
  }
  out.t.kind = LLG_TERM_EXCHANGE;
}

void build_uniaxial(Model& m, const Node& h, Model::Term& out) {
  if (h.find("d2z") || h.find("d4z") || h.find("d6z") || h.find("K1") || h.find("K2") || h.find("K3"))
    throw CfgError("UniaxialHamiltonian: anisotropy should only be specified for a single K1, K2 or K3");
  const std::string order = h.at("order").str();
  const int power = order == "K1" ? 2 : order == "K2" ? 4 : order == "K3" ? 6 : 0;
  if (!power) throw CfgError("Unsupported anisotropy: " + order);
  const double conv = energy_unit(h);
  const size_t nb = m.basis.size();
  out.K.assign(nb, 0.0);
  out.axis.assign(3 * nb, 0.0);
  const Node& an = h.at("anisotropies");
  for (size_t k = 0; k < an.size(); ++k) {
    const Node& e = an.at(k);
    V3 ax = vec3(e.at(1));
    const double nrm = std::sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
    for (auto& c : ax) c = c / nrm;
    const double K = e.at(2).num() * conv;
    for (size_t b = 0; b < nb; ++b) {
      const bool hit = e.at(0).is_number() ? (int)b == (int)e.at(0).num() - 1 : m.basis[b].material == e.at(0).str();
      if (!hit) continue;
      out.K[b] = K;
      for (int c = 0; c < 3; ++c) out.axis[3 * b + c] = ax[c];
    }
  }
  out.t.kind = LLG_TERM_UNIAXIAL;
  out.t.order = power;
}

void build_cubic(Model& m, const Node& h, Model::Term& out) {
  const bool k1 = h.find("K1") != nullptr, k2 = h.find("K2") != nullptr;
  if (k1 && k2) throw CfgError("Input only one order of cubic anisotropy");
  if (!k1 && !k2) throw CfgError("Unsupported cubic anisotropy");
  const Node& list = h.at(k1 ? "K1" : "K2");
  const double conv = energy_unit(h);
  const size_t nb = m.basis.size();
  out.K.assign(nb, 0.0);
  out.axis.assign(9 * nb, 0.0);
  // one entry per material, in material order (cubic_anisotropy.cc:108-124)
  for (size_t b = 0; b < nb; ++b) {
    const size_t mi = (size_t)m.basis[b].mat;
    if (mi >= list.size()) throw CfgError("cubic anisotropy: one entry per material is needed");
    const Node& e = list.at(mi);
    V3 u{1, 0, 0}, v{0, 1, 0}, w{0, 0, 1};
    double K;
    if (e.type == Node::List) {
      K = e.at(0).num();
      u = vec3(e.at(1));
      v = vec3(e.at(2));
      w = vec3(e.at(3));
    } else {
      K = e.num();
    }
    for (V3* a : {&u, &v, &w}) {
      const double n = std::sqrt((*a)[0] * (*a)[0] + (*a)[1] * (*a)[1] + (*a)[2] * (*a)[2]);
      for (auto& c : *a) c = c / n;
    }
    out.K[b] = K * conv;
    for (int c = 0; c < 3; ++c) {
      out.axis[9 * b + c] = u[c];
      out.axis[9 * b + 3 + c] = v[c];
      out.axis[9 * b + 6 + c] = w[c];
    }
  }
  out.t.kind = LLG_TERM_CUBIC;
  out.t.order = k1 ? 1 : 2;
}

uint64_t splitmix64(uint64_t& x) {
  uint64_t z = (x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

Model build_model(const Node& root) {
  Model m;
  // materials (src/jams/containers/material.h:40-57)
  const Node& mats = root.at("materials");
  for (size_t k = 0; k < mats.size(); ++k) {
    const Node& g = mats.at(k);
    m.mat_names.push_back(g.at("name").str());
    m.mat_moment.push_back(g.at("moment").num() * kBohrMagnetonIU);
    m.mat_gyro.push_back((g.find("gyro") ? g.at("gyro").num() : 1.0) * kGyromagneticRatioIU);
    m.mat_alpha.push_back(g.find("alpha") ? g.at("alpha").num() : 0.01);
    V3 spin{0, 0, 1};
    bool random = false;
    if (const Node* s = g.find("spin")) {
      if (s->type == Node::String && lower(s->str()) == "random") {
        random = true;
      } else if (s->type == Node::Array && s->size() == 3) {
        spin = vec3(*s);
      } else if (s->type == Node::Array && s->size() == 2) {
        const double th = s->at(0).num() * kPi / 180.0, ph = s->at(1).num() * kPi / 180.0;
        spin = V3{std::sin(th) * std::cos(ph), std::sin(th) * std::sin(ph), std::cos(th)};
      } else {
        throw CfgError("spin setting array is not length 2 or 3");
      }
    }
    m.mat_spin.push_back(spin);
    m.mat_random.push_back(random);
  }
  // unit cell
  const Node& uc = root.at("unitcell");
  const Node& bas = uc.at("basis");
  if (bas.size() != 3) throw CfgError("unitcell basis needs 3 rows");
  for (int i = 0; i < 3; ++i) {
    const V3 row = vec3(bas.at(i));
    for (int j = 0; j < 3; ++j) m.cell[i][j] = row[j];
  }
  m.cell_inv = inverse(m.cell);
  if (const Node* n = uc.find("parameter")) m.parameter = n->num();
  std::string pos_format = "fractional";
  if (const Node* n = uc.find("coordinate_format")) pos_format = lower(n->str());
  const Node& pos = uc.at("positions");
  for (size_t k = 0; k < pos.size(); ++k) {
    Basis b;
    b.material = pos.at(k).at(0).str();
    b.mat = material_index(m, b.material);
    V3 p = vec3(pos.at(k).at(1));
    if (pos_format == "cartesian") p = mul(m.cell_inv, p);
    b.frac = wrap_frac(p);
    m.basis.push_back(b);
  }
  if (m.basis.empty()) throw CfgError("unitcell has no positions");
  // lattice
  const Node& lat = root.at("lattice");
  const V3 size = vec3(lat.at("size"));
  for (int l = 0; l < 3; ++l) {
    m.L[l] = (int)size[l];
    if (m.L[l] < 1) throw CfgError("lattice size must be positive");
  }
  if (const Node* p = lat.find("periodic"))
    for (int l = 0; l < 3; ++l) m.periodic[l] = p->at(l).boolean() ? 1 : 0;
  // solver
  const Node& sol = root.at("solver");
  m.solver_module = lower(sol.at("module").str());
  if (m.solver_module == "llg-heun-gpu" || m.solver_module == "llg-heun-cpu")
    m.integrator = LLG_HEUN;
  else if (m.solver_module == "llg-rk4-gpu")
    m.integrator = LLG_RK4;
  else
    throw CfgError("unknown solver " + m.solver_module + " for the LLG path");
  m.t_step = sol.at("t_step").num();
  m.t_max = sol.at("t_max").num();
  if (const Node* g = sol.find("gilbert_prefactor")) m.gilbert = g->boolean();
  // src/jams/solvers/cuda_llg_heun.cu:23-29
  const double step_ps = m.t_step / 1e-12;
  const double max_ps = m.t_max / 1e-12;
  if (!(step_ps > 0.0)) throw CfgError("solver t_step must be positive");
  m.max_steps = (int64_t)(max_ps / step_ps);
  // per basis site parameters (src/jams/core/lattice.cc:688-700)
  for (auto& b : m.basis) {
    const double mo = m.mat_moment[b.mat], g = m.mat_gyro[b.mat], a = m.mat_alpha[b.mat];
    m.mus.push_back(mo);
    m.alpha.push_back(a);
    m.gyro.push_back(m.gilbert ? g / (1.0 + a * a) : g);
  }
  // physics, sim
  if (const Node* ph = root.find("physics"))
    if (const Node* t = ph->find("temperature")) m.temperature = t->num();
  if (const Node* sim = root.find("sim"))
    if (const Node* s = sim->find("seed")) m.seed = (uint64_t)s->num();
  // hamiltonians, in list order (Solver::compute_fields sums them in order)
  const Node& hs = root.at("hamiltonians");
  for (size_t k = 0; k < hs.size(); ++k) {
    const Node& h = hs.at(k);
    Model::Term t;
    t.module = lower(h.at("module").str());
    if (t.module == "exchange") {
      build_exchange(m, h, t);
    } else if (t.module == "uniaxial" || t.module == "uniaxial-anisotropy") {
      build_uniaxial(m, h, t);
    } else if (t.module == "cubic" || t.module == "cubic-anisotropy") {
      build_cubic(m, h, t);
    } else if (t.module == "applied-field") {
      // static, sinc or sinc-cos field (applied_field.cc:82-110); time_center
      // in seconds, freq_bandwidth and freq_center in hertz, converted to ps
      // and THz as the reference does (:36-38, 64-67)
      const V3 B = vec3(h.at("field"));
      t.t.kind = LLG_TERM_APPLIED_FIELD;
      for (int c = 0; c < 3; ++c) t.t.B[c] = B[c];
      t.t.pulse = LLG_PULSE_STATIC;
      if (h.find("type")) {
        const std::string type = lower(h.at("type").str());
        if (type == "sinc") t.t.pulse = LLG_PULSE_SINC;
        else if (type == "sinc-cos") t.t.pulse = LLG_PULSE_SINC_COS;
        else if (type != "static") throw CfgError("applied-field: unknown field pulse type " + type);
      }
      if (t.t.pulse != LLG_PULSE_STATIC) {
        t.t.time_center = h.at("time_center").num() / 1e-12;
        t.t.freq_bandwidth = h.at("freq_bandwidth").num() / 1e12;
        if (t.t.pulse == LLG_PULSE_SINC_COS) t.t.freq_center = h.at("freq_center").num() / 1e12;
      }
    } else if (t.module == "zeeman") {
      // dc field, ac field and ac frequency per material (zeeman.cc:12-71)
      t.t.kind = LLG_TERM_ZEEMAN;
      const size_t nm = m.mat_names.size(), nb = m.basis.size();
      const Node* dc = h.find("dc_local_field");
      const Node* ac = h.find("ac_local_field");
      const Node* fr = h.find("ac_local_frequency");
      if (dc && dc->size() != nm) throw CfgError("zeeman: dc_local_field must be specified for every material");
      if ((ac != nullptr) != (fr != nullptr)) throw CfgError("zeeman: ac_local_field must have a field and a frequency");
      if (ac && (ac->size() != nm || fr->size() != nm))
        throw CfgError("zeeman: ac_local_field and ac_local_frequency must be specified for every material");
      t.dc.assign(3 * nb, 0.0);
      if (ac) {
        t.ac.assign(3 * nb, 0.0);
        t.freq.assign(nb, 0.0);
      }
      for (size_t b = 0; b < nb; ++b) {
        const size_t mi = (size_t)m.basis[b].mat;
        if (dc) {
          const V3 v = vec3(dc->at(mi));
          for (int c = 0; c < 3; ++c) t.dc[3 * b + c] = v[c];
        }
        if (ac) {
          const V3 v = vec3(ac->at(mi));
          for (int c = 0; c < 3; ++c) t.ac[3 * b + c] = v[c];
          t.freq[b] = fr->at(mi).num();
        }
      }
    } else if (t.module == "dipole-fft" || t.module == "dipole-bruteforce" || t.module == "dipole-tensor" ||
               t.module == "dipole-neighbour-list" || t.module == "dipole-neartree") {
      // the same sum by every method (docs/source/hamiltonians/dipole.rst);
      // here always by FFT convolution
      t.t.kind = LLG_TERM_DIPOLE;
      t.t.r_cutoff = h.at("r_cutoff").num();
      t.t.distance_tolerance = 1e-4;   // jams::defaults::lattice_tolerance
      if (const Node* n = h.find("distance_tolerance")) t.t.distance_tolerance = n->num();
      if (!(m.parameter > 0.0)) throw CfgError(t.module + ": unitcell.parameter (m) is required");
      t.t.lattice_parameter = m.parameter;
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) t.vectors.push_back(m.cell[c][r]);   // rows a1, a2, a3
      for (const Basis& b : m.basis)
        for (int c = 0; c < 3; ++c) t.positions.push_back(b.frac[c]);
    } else {
      throw CfgError("hamiltonian module '" + t.module + "' is not on the LLG hot path");
    }
    m.terms.push_back(std::move(t));
  }
  return m;
}

void fill_desc(Model& m, llg_desc& d, llg_replica& rep, std::vector<llg_term>& terms, int precision, int device) {
  terms.clear();
  for (auto& t : m.terms) {
    llg_term lt = t.t;
    lt.n_int = (int32_t)t.bi.size();
    lt.bi = t.bi.data();
    lt.bj = t.bj.data();
    lt.T = t.T.data();
    lt.J = t.J.data();
    lt.K = t.K.empty() ? nullptr : t.K.data();
    lt.axis = t.axis.empty() ? nullptr : t.axis.data();
    lt.lattice_vectors = t.vectors.empty() ? nullptr : t.vectors.data();
    lt.positions = t.positions.empty() ? nullptr : t.positions.data();
    lt.dc_field = t.dc.empty() ? nullptr : t.dc.data();
    lt.ac_field = t.ac.empty() ? nullptr : t.ac.data();
    lt.ac_frequency = t.freq.empty() ? nullptr : t.freq.data();
    terms.push_back(lt);
  }
  d = llg_desc{};
  d.abi_version = LLG_ABI_VERSION;
  d.nb = (int32_t)m.basis.size();
  for (int l = 0; l < 3; ++l) {
    d.periodic[l] = m.periodic[l];
    rep.L[l] = m.L[l];
  }
  rep.temperature = m.temperature;
  rep.use_B = 0;
  d.mus = m.mus.data();
  d.gyro = m.gyro.data();
  d.alpha = m.alpha.data();
  d.n_terms = (int32_t)terms.size();
  d.terms = terms.data();
  d.dt = m.t_step / 1e-12;
  d.gilbert_prefactor = m.gilbert ? 1 : 0;
  d.integrator = m.integrator;
  d.precision = precision;
  d.seed = m.seed;
  d.n_replicas = 1;
  d.replicas = &rep;
  d.device = device;
}

// initial spins: material spin, unit length; "random" materials draw
// uniform directions (Marsaglia, as uniform_random_sphere,
// src/jams/helpers/random.h:12-26) from a generator seeded by sim.seed
std::vector<double> initial_spins(const Model& m) {
  const int64_t nb = (int64_t)m.basis.size();
  const int64_t n = (int64_t)m.L[0] * m.L[1] * m.L[2] * nb;
  std::vector<double> s((size_t)(3 * n));
  uint64_t state = m.seed ^ 0x6A09E667F3BCC909ull;
  for (int64_t i = 0; i < n; ++i) {
    const int mat = m.basis[(size_t)(i % nb)].mat;
    V3 v = m.mat_spin[mat];
    if (m.mat_random[mat]) {
      double v1, v2, q;
      do {
        v1 = 2.0 * ((splitmix64(state) >> 11) * 0x1.0p-53) - 1.0;
        v2 = 2.0 * ((splitmix64(state) >> 11) * 0x1.0p-53) - 1.0;
        q = v1 * v1 + v2 * v2;
      } while (q > 1.0);
      const double ss = 2.0 * std::sqrt(1.0 - q);
      v = V3{v1 * ss, v2 * ss, 1.0 - 2.0 * q};
    }
    const double len = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int c = 0; c < 3; ++c) s[(size_t)(3 * i + c)] = len > 0.0 ? v[c] / len : 0.0;
  }
  return s;
}

Node parse_with_patch(const char* text, const char* patch) {
  if (!text) throw CfgError("config text is null");
  std::string t(text);
  Node root = Parser(t).parse_root();
  if (patch && *patch) {
    std::string p(patch);
    Node pr = Parser(p).parse_root();
    merge(root, pr);
  }
  return root;
}

void json_num(std::ostringstream& o, double v) {
  char buf[40];
  snprintf(buf, sizeof buf, "%.17g", v);
  o << buf;
}

}  // namespace

extern "C" {

int llg_create_from_config(const char* config_text, const char* patch_text, int32_t precision, int32_t device,
                           llg_handle** out) {
  if (!out) {
    jams_llg::set_thread_error("out is null");
    return LLG_ERR_BAD_DESC;
  }
  *out = nullptr;
  try {
    Node root = parse_with_patch(config_text, patch_text);
    Model m = build_model(root);
    llg_desc d;
    llg_replica rep{};
    std::vector<llg_term> terms;
    fill_desc(m, d, rep, terms, precision, device);
    llg_handle* h = nullptr;
    int rc = llg_create(&d, &h);
    if (rc) return rc;
    std::vector<double> s = initial_spins(m);
    rc = llg_set_state(h, 0, s.data());
    if (rc) {
      llg_destroy(h);
      return rc;
    }
    jams_llg::set_max_steps(h, m.max_steps);
    *out = h;
    return 0;
  } catch (const std::exception& e) {
    jams_llg::set_thread_error(e.what());
    return LLG_ERR_BAD_DESC;
  }
}

int llg_config_describe(const char* config_text, const char* patch_text, char* json, int64_t json_len) {
  try {
    Node root = parse_with_patch(config_text, patch_text);
    Model m = build_model(root);
    std::ostringstream o;
    o << "{\"nb\":" << m.basis.size() << ",\"L\":[" << m.L[0] << "," << m.L[1] << "," << m.L[2]
      << "],\"periodic\":[" << m.periodic[0] << "," << m.periodic[1] << "," << m.periodic[2] << "]";
    auto arr = [&](const char* name, const std::vector<double>& v) {
      o << ",\"" << name << "\":[";
      for (size_t k = 0; k < v.size(); ++k) {
        if (k) o << ",";
        json_num(o, v[k]);
      }
      o << "]";
    };
    std::vector<double> basis_material;
    for (const Basis& b : m.basis) basis_material.push_back((double)b.mat);
    arr("basis_material", basis_material);   // material index of each basis site (magnetisation grouping)
    arr("mus", m.mus);
    arr("gyro", m.gyro);
    arr("alpha", m.alpha);
    o << ",\"dt\":";
    json_num(o, m.t_step / 1e-12);
    o << ",\"t_step\":";
    json_num(o, m.t_step);
    o << ",\"max_steps\":" << m.max_steps << ",\"integrator\":" << m.integrator << ",\"gilbert_prefactor\":"
      << (m.gilbert ? 1 : 0) << ",\"temperature\":";
    json_num(o, m.temperature);
    o << ",\"seed\":" << m.seed << ",\"terms\":[";
    for (size_t k = 0; k < m.terms.size(); ++k) {
      const auto& t = m.terms[k];
      if (k) o << ",";
      o << "{\"module\":\"" << t.module << "\",\"kind\":" << t.t.kind << ",\"order\":" << t.t.order;
      std::vector<double> bi(t.bi.begin(), t.bi.end()), bj(t.bj.begin(), t.bj.end()), T(t.T.begin(), t.T.end());
      arr("bi", bi);
      arr("bj", bj);
      arr("T", T);
      arr("J", t.J);
      arr("K", t.K);
      arr("axis", t.axis);
      arr("B", std::vector<double>{t.t.B[0], t.t.B[1], t.t.B[2]});
      if (t.t.kind == LLG_TERM_APPLIED_FIELD)
        arr("pulse", std::vector<double>{(double)t.t.pulse, t.t.time_center, t.t.freq_bandwidth, t.t.freq_center});
      if (t.t.kind == LLG_TERM_ZEEMAN) {
        arr("dc_field", t.dc);
        arr("ac_field", t.ac);
        arr("ac_frequency", t.freq);
      }
      if (t.t.kind == LLG_TERM_DIPOLE) {
        arr("dipole", std::vector<double>{t.t.r_cutoff, t.t.distance_tolerance, t.t.lattice_parameter});
        arr("lattice_vectors", t.vectors);
        arr("positions", t.positions);
      }
      o << "}";
    }
    o << "]}";
    const std::string s = o.str();
    if (!json || json_len < (int64_t)s.size() + 1) {
      const std::string msg = "llg_config_describe: buffer too small, need " + std::to_string(s.size() + 1) + " bytes";
      jams_llg::set_thread_error(msg.c_str());
      return LLG_ERR_BAD_DESC;
    }
    memcpy(json, s.c_str(), s.size() + 1);
    return 0;
  } catch (const std::exception& e) {
    jams_llg::set_thread_error(e.what());
    return LLG_ERR_BAD_DESC;
  }
}

}  // extern "C"
