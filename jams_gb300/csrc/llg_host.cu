// Host runtime of libjams_llg.so: validates an llg_desc, builds the stencil
// tables, owns the device buffers and streams, runs blocks of steps as CUDA
// graphs and exposes the C ABI declared in include/jams_llg.h.
//
// Stencil tables.  The reference expands the interaction template into a
// 3N x 3N CSR matrix (src/jams/core/interactions.cc:350-396,
// src/jams/containers/sparse_matrix_builder.h:186-248).  On a periodic or
// open lattice without impurities the neighbour of site (c, b) through
// template entry e is site (c + T_e wrapped, bj_e), so j - i depends only on
// which axes wrap at c.  Cells are grouped into boundary classes per axis
// (c < R, interior, c >= L - R, with R the stencil reach; every coordinate is
// its own class when L <= 2R + 1) and one table of offsets j - i per (basis
// site, class) describes the whole matrix.  For the FP64 form the entries of
// each class are stored in ascending j, the order in which the CSR row sum
// visits them.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/jams_llg.h"
#include "llg_internal.h"

#include "llg_dipole.h"
#include "llg_families.h"
#include "llg_io.h"
#include "llg_kernels.h"

using namespace jams_llg;

namespace jams_llg {
void set_max_steps(llg_handle* h, int64_t max_steps);
}

namespace {
thread_local std::string g_tls_error;
}

namespace jams_llg {
// thread-local message for llg_last_error(NULL), used by entry points without a handle
void set_thread_error(const char* msg) { g_tls_error = msg; }
}  // namespace jams_llg

namespace {

// src/jams/helpers/consts.h:16,32
constexpr double kPi = 3.14159265358979323846;
constexpr double kBoltzmannIU = 0.0861733326;

struct ExchangeHost {
  int term;
  int zmax = 0;        // FP64 list length per (b, class)
  int nslot_max = 0;   // FP32 slots per (b, class)
  // FP32 slot layout per basis site: entry index of each slot, groups, rest
  std::vector<int> slot_entry[kMaxBasis];
  std::vector<int> group_end[kMaxBasis];
  std::vector<double> group_j[kMaxBasis];
  std::vector<float> rest_j;  // [nb][kMaxSlots][9]
  std::vector<double> J64;    // [n_entries][9]
  std::vector<uint16_t> mask; // [n_entries]
};

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  ~DevBuf() { reset(); }
  void reset() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t alloc(size_t count) {
    reset();
    n = count;
    if (count == 0) return cudaSuccess;
    return cudaMalloc((void**)&p, count * sizeof(T));
  }
};

// a pinned host buffer (staging of host -> device copies)
struct PinnedBuf {
  unsigned char* p = nullptr;
  ~PinnedBuf() {
    if (p) cudaFreeHost(p);
  }
  cudaError_t alloc(size_t bytes) { return cudaHostAlloc((void**)&p, bytes, cudaHostAllocDefault); }
};

// a pinned host word the status flag is copied into
struct PinnedWord {
  unsigned int* p = nullptr;
  ~PinnedWord() {
    if (p) cudaFreeHost(p);
  }
  cudaError_t alloc() { return p ? cudaSuccess : cudaHostAlloc((void**)&p, sizeof(unsigned int), cudaHostAllocDefault); }
};

struct GraphKey {
  int parity;
  int nsteps;
  bool operator<(const GraphKey& o) const { return parity != o.parity ? parity < o.parity : nsteps < o.nsteps; }
};

}  // namespace

struct llg_handle {
  std::string err;
  int device = 0;
  bool fp64 = false;
  int integrator = LLG_HEUN;
  int nb = 1;
  int nterms = 0;
  int steps_per_graph = 100;
  std::vector<llg_term> terms_copy;
  std::vector<double> term_B;  // applied-field B of the desc (per term, 3)
  std::vector<ReplicaDev> reps;
  std::vector<double> rep_T;
  std::vector<int2> tiles;
  std::vector<int> rep_first_tile, rep_ntiles;
  int64_t npad = 0;
  double mus[kMaxBasis], gyro[kMaxBasis], alpha[kMaxBasis];
  bool gilbert = false;
  double dt = 0.0;
  Params P{};
  // device
  DevBuf<unsigned char> state[3];  // spin planes (float or double)
  DevBuf<unsigned char> aux;       // FP64 Heun ds / RK4 accumulator
  DevBuf<float> noise;             // stored-noise mode: the step's thermal field planes
  DevBuf<ReplicaDev> d_rep;
  DevBuf<int2> d_tiles;
  DevBuf<int32_t> d_tab32;
  DevBuf<int2> d_tab64;
  DevBuf<int32_t> d_cnt64;
  DevBuf<float> d_rest[kMaxExchange];
  DevBuf<double> d_J64[kMaxExchange];
  DevBuf<uint16_t> d_mask[kMaxExchange];
  DevBuf<unsigned int> d_status;
  PinnedWord h_status;
  DevBuf<uint64_t> d_step_base;
  DevBuf<unsigned int> d_ticket;
  DevBuf<double> d_scratch;        // N x 3 doubles for host transfers
  DevBuf<double> d_partials;
  std::vector<double> h_partials;
  int cur = 0;                     // index of the buffer holding the state
  int64_t iteration = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  std::map<GraphKey, cudaGraphExec_t> graphs;
  int64_t last_launches = 0;
  bool params_dirty = false;
  int64_t max_steps = -1;    // from a config file's solver section
  // tiled FP32 path (lattice matched a stencil family)
  int family = kFamNone;
  bool tiled = false;
  bool store_noise = false;  // Heun, stored-rhs mode: the predictor stores the thermal field for the corrector
  bool store_mode = false;   // Heun: predictor stores s0 + dt/2 rhs(s0) instead of the corrector recomputing rhs(s0)
  int occupancy = 2;         // tiled kernels compiled for >= 2, 3 or 4 CTAs per SM
  int tz = 0, ty = 0;
  int rpt = 1;               // rows per thread of the tiled kernels (1 or 2)
  uint64_t model_hash = 0;   // the descriptor's Hamiltonian and material parameters (checkpoint fingerprint)
  bool tma = false;          // tiled kernels: planes arrive by TMA box loads (tmaps: one per state buffer)
  CUtensorMap tmaps[3];
  bool fused = false;        // Heun: one fused step kernel (predictor over tile + halo in shared memory)
  bool fused_wide = true;    // its wide tile (fused_rows)
  TiledParams TP{};
  DevBuf<int4> d_tiles4;
  // dipole-dipole term: FFT convolution state and the field planes of the
  // stage input (0: start-of-step state, 1: Heun predictor state)
  bool has_dipole = false;
  DipoleGeometry dip_geom{};
  DipoleField* dipole = nullptr;
  DevBuf<unsigned char> d_hdip[2];
  // time-dependent fields (applied-field pulse, zeeman ac field): their
  // parameters, a device table of the time factors of every stage of up to
  // pulse_cap steps ([iteration of entry 0][pad][doubles][floats]), filled
  // per llg_step chunk through two pinned staging buffers, and the factors
  // at the current solver time for fields and energies
  bool pulsed = false;
  int pulse_type = LLG_PULSE_STATIC;
  double pulse_tc = 0.0, pulse_fbw = 0.0, pulse_fc = 0.0;
  bool zeeman_ac = false;
  double zeeman_w[kMaxBasis] = {};
  int pulse_cap = 0;
  DevBuf<unsigned char> d_pulse;
  PinnedBuf pulse_host[2];
  cudaEvent_t pulse_ev[2] = {nullptr, nullptr};
  int pulse_slot = 0;
  DevBuf<unsigned char> d_pulse_now;
  PinnedBuf pulse_now_host;
  std::string async_err;     // a failure inside an enqueue (reported by llg_step)

  ~llg_handle() {
    for (auto& e : pulse_ev)
      if (e) cudaEventDestroy(e);
    if (dipole) dipole_destroy(dipole);
    for (auto& g : graphs) cudaGraphExecDestroy(g.second);
    if (own_stream) cudaStreamDestroy(own_stream);
  }
  int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    err = buf;
    g_tls_error = buf;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* what) {
    return fail(e == cudaErrorMemoryAllocation ? LLG_ERR_OOM : LLG_ERR_CUDA, "%s: %s", what,
                cudaGetErrorString(e));
  }
};

namespace {

int tls_fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_tls_error = buf;
  return code;
}

size_t real_size(const llg_handle* h) { return h->fp64 ? sizeof(double) : sizeof(float); }

int axis_classes(int L, int R) { return (L <= 2 * R + 1) ? L : 2 * R + 1; }

int class_rep(int k, int L, int R, int ncls) {
  if (ncls == L) return k;
  if (k <= R) return k;
  return L - R + (k - R - 1);
}

// builds FP32 slot layout (groups of equal isotropic J, then anisotropic rests)
int build_slots(llg_handle* h, const llg_term& t, ExchangeHost& X) {
  const int nb = h->nb;
  X.rest_j.assign((size_t)nb * kMaxSlots * 9, 0.f);
  for (int b = 0; b < nb; ++b) {
    std::vector<double> iso_vals;
    std::vector<std::vector<int>> iso_members;
    std::vector<int> rest_members;
    for (int e = 0; e < t.n_int; ++e) {
      if (t.bi[e] != b) continue;
      const double* J = t.J + 9 * e;
      double mx = 0.0;
      for (int a = 0; a < 9; ++a) mx = std::max(mx, std::fabs(J[a]));
      if (!(mx > 0.0)) continue;  // exchange.cc:166: only tensors with max|J| > 0
      double iso = 0.0;
      if (J[0] == J[4] && J[4] == J[8]) iso = J[0];
      bool rest = false;
      for (int a = 0; a < 9; ++a) {
        const double r = J[a] - ((a % 4 == 0) ? iso : 0.0);
        if (r != 0.0) rest = true;
      }
      if (iso != 0.0) {
        size_t g = 0;
        for (; g < iso_vals.size(); ++g)
          if (iso_vals[g] == iso) break;
        if (g == iso_vals.size()) {
          iso_vals.push_back(iso);
          iso_members.emplace_back();
        }
        iso_members[g].push_back(e);
      }
      if (rest) rest_members.push_back(e);
    }
    if ((int)iso_vals.size() > kMaxGroups)
      return h->fail(LLG_ERR_UNSUPPORTED, "more than %d distinct isotropic exchange values on basis site %d",
                     kMaxGroups, b);
    size_t iso_slots = 0;
    for (auto& g : iso_members) iso_slots += g.size();
    if (iso_slots > (size_t)kMaxSlots)
      return h->fail(LLG_ERR_UNSUPPORTED, "more than %d neighbour slots on basis site %d", kMaxSlots, b);
    for (size_t g = 0; g < iso_vals.size(); ++g) {
      for (int e : iso_members[g]) X.slot_entry[b].push_back(e);
      X.group_end[b].push_back((int)X.slot_entry[b].size());
      X.group_j[b].push_back(iso_vals[g]);
    }
    for (int e : rest_members) {
      const int slot = (int)X.slot_entry[b].size();
      if (slot >= kMaxSlots)
        return h->fail(LLG_ERR_UNSUPPORTED, "more than %d neighbour slots on basis site %d", kMaxSlots, b);
      X.slot_entry[b].push_back(e);
      const double* J = t.J + 9 * e;
      const double iso = (J[0] == J[4] && J[4] == J[8]) ? J[0] : 0.0;
      for (int a = 0; a < 9; ++a)
        X.rest_j[((size_t)b * kMaxSlots + slot) * 9 + a] = (float)(J[a] - ((a % 4 == 0) ? iso : 0.0));
    }
    X.nslot_max = std::max<int>(X.nslot_max, (int)X.slot_entry[b].size());
  }
  X.J64.assign((size_t)t.n_int * 9, 0.0);
  X.mask.assign((size_t)t.n_int, 0);
  for (int e = 0; e < t.n_int; ++e) {
    uint16_t m = 0;
    for (int a = 0; a < 9; ++a) {
      X.J64[(size_t)e * 9 + a] = t.J[9 * e + a];
      if (t.J[9 * e + a] != 0.0) m |= (uint16_t)(1u << a);
    }
    X.mask[e] = m;
  }
  for (int b = 0; b < nb; ++b) {
    int z = 0;
    for (int e = 0; e < t.n_int; ++e)
      if (t.bi[e] == b) ++z;
    X.zmax = std::max(X.zmax, z);
  }
  return 0;
}

// Matches an exchange interaction template against a compile-time stencil
// family: the same (basis site, translation, partner) set per basis site,
// one isotropic J per shell (families without remainders) and nothing else.
template <class F>
bool match_family(const llg_desc* d, const llg_term& t, TiledParams& TP) {
  if (d->nb != F::NB) return false;
  for (int r = 0; r < d->n_replicas; ++r) {
    if (F::TWO_D && d->replicas[r].L[2] != 1) return false;
    for (int l = 0; l < 3; ++l)
      if (d->periodic[l] && d->replicas[r].L[l] < 3 && !(F::TWO_D && l == 2)) return false;
  }
  std::map<std::vector<int>, int> idx;
  for (int e = 0; e < t.n_int; ++e) {
    double mx = 0.0;
    for (int a = 0; a < 9; ++a) mx = std::max(mx, std::fabs(t.J[9 * e + a]));
    if (!(mx > 0.0)) continue;
    const int* T = t.T + 3 * e;
    const int dX = T[0], dY = F::TWO_D ? T[2] : T[1], dZ = F::TWO_D ? T[1] : T[2];
    std::vector<int> key = {t.bi[e], dX, dY, dZ, t.bj[e]};
    if (idx.count(key)) return false;
    idx[key] = e;
  }
  if ((int)idx.size() != F::NB * F::Z) return false;
  TiledParams tp = TP;
  for (int b = 0; b < F::NB; ++b) {
    double shell_j[4] = {0, 0, 0, 0};
    for (int k = 0; k < F::Z; ++k) {
      const Slot sl = F::slot(b, k);
      auto it = idx.find(std::vector<int>{b, sl.dx, sl.dy, sl.dz, sl.bj});
      if (it == idx.end()) return false;
      const double* J = t.J + 9 * it->second;
      int g = 0;
      while (k >= F::shell_end(b, g)) ++g;
      const bool diag_equal = J[0] == J[4] && J[4] == J[8];
      double iso = diag_equal ? J[0] : 0.0;
      if (!F::REST) {
        if (!diag_equal) return false;
        for (int a = 0; a < 9; ++a)
          if (a % 4 != 0 && J[a] != 0.0) return false;
      }
      const bool first = k == (g == 0 ? 0 : F::shell_end(b, g - 1));
      if (first) shell_j[g] = iso;
      else if (shell_j[g] != iso) return false;
      if (F::REST) {
        if (k >= 8) return false;
        for (int a = 0; a < 9; ++a) tp.rest[b][k][a] = (float)(J[a] - ((a % 4 == 0) ? iso : 0.0));
      }
    }
    for (int g = 0; g < F::NSHELL; ++g) {
      const float hi = (float)shell_j[g];
      tp.shell_hi[b][g] = hi;
      tp.shell_lo[b][g] = (float)(shell_j[g] - (double)hi);
    }
  }
  TP = tp;
  return true;
}

int find_family(const llg_desc* d, const llg_term& t, TiledParams& TP) {
  if (match_family<FamSC>(d, t, TP)) return kFamSC;
  if (match_family<FamBCC>(d, t, TP)) return kFamBCC;
  if (match_family<FamBCC3>(d, t, TP)) return kFamBCC3;
  if (match_family<FamTRI>(d, t, TP)) return kFamTRI;
  if (match_family<FamFCC>(d, t, TP)) return kFamFCC;
  if (match_family<FamFCC2>(d, t, TP)) return kFamFCC2;
  return kFamNone;
}

// tile work-list of the tiled kernels for the current TX
int build_tiles4(llg_handle* h) {
  std::vector<int4> t4;
  for (size_t r = 0; r < h->reps.size(); ++r) {
    const ReplicaDev& R = h->reps[r];
    for (int x0 = 0; x0 < R.vL[0]; x0 += h->TP.TX)
      for (int y0 = 0; y0 < R.vL[1]; y0 += h->ty)
        for (int z0 = 0; z0 < R.vL[2]; z0 += h->tz) t4.push_back(make_int4((int)r, x0, y0, z0));
  }
  cudaError_t ce = h->d_tiles4.alloc(t4.size());
  if (ce == cudaSuccess)
    ce = cudaMemcpy(h->d_tiles4.p, t4.data(), t4.size() * sizeof(int4), cudaMemcpyHostToDevice);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "uploading tiles");
  h->TP.tiles = h->d_tiles4.p;
  h->TP.ntiles = (int)t4.size();
  return 0;
}

void drop_graphs(llg_handle* h) {
  for (auto& g : h->graphs) cudaGraphExecDestroy(g.second);
  h->graphs.clear();
}

// cuTensorMapEncodeTiled, from the driver through the runtime (the library
// links the runtime only)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// whether the tiled kernels can take their planes by TMA: one replica, a
// family with 32-cell-wide tiles, rows whose byte stride is a multiple of
// 16, and the driver's encoder; the reason when not
const char* tma_unsupported(const llg_handle* h) {
  if (!h->tiled || h->fp64) return "the tiled FP32 kernels only";
  if (h->dipole) return "not with a dipole term";
  if (h->reps.size() != 1) return "one replica only";
  int lo, width, rows;
  if (!tma_box(h->family, h->ty, &lo, &width, &rows)) return "not for this lattice family";
  const ReplicaDev& R = h->reps[0];
  if (R.vs[2] != h->nb || R.vs[1] != (int64_t)R.vL[2] * h->nb || (R.vs[1] * 4) % 16 != 0)
    return "rows must be contiguous with a byte stride that is a multiple of 16";
  if (!tensor_map_encoder()) return "the driver has no cuTensorMapEncodeTiled";
  return nullptr;
}

// the tensor map of state buffer k: (z x basis, y, x, component) of
// replica 0, box (width, rows, 1 plane, 3 components)
int build_tensor_maps(llg_handle* h) {
  int lo, width, rows;
  tma_box(h->family, h->ty, &lo, &width, &rows);
  const ReplicaDev& R = h->reps[0];
  const cuuint64_t dims[4] = {(cuuint64_t)R.vL[2] * h->nb, (cuuint64_t)R.vL[1], (cuuint64_t)R.vL[0], 3};
  const cuuint64_t strides[3] = {(cuuint64_t)R.vs[1] * 4, (cuuint64_t)R.vs[0] * 4, (cuuint64_t)h->npad * 4};
  const cuuint32_t box[4] = {(cuuint32_t)width, (cuuint32_t)rows, 1, 3};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  for (int k = 0; k < 3; ++k) {
    float* base = reinterpret_cast<float*>(h->state[k].p) + R.offset;
    const CUresult r = tensor_map_encoder()(&h->tmaps[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, dims, strides, box,
                                            estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return h->fail(LLG_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  }
  return 0;
}

// FNV-1a over the values that define a model's physics besides the lattice
// sizes: materials, periodicity, dt convention, and every term's parameters
// (interaction templates, anisotropy constants and axes, fields, pulses,
// dipole geometry), in term order
struct ModelHasher {
  uint64_t h = 1469598103934665603ull;
  void bytes(const void* p, size_t n) {
    const unsigned char* c = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) h = (h ^ c[i]) * 1099511628211ull;
  }
  template <class T>
  void val(T v) { bytes(&v, sizeof v); }
  template <class T>
  void arr(const T* p, size_t n) {
    val((uint64_t)(p ? n : 0));
    if (p && n) bytes(p, n * sizeof(T));
  }
};

uint64_t model_hash(const llg_desc* d) {
  ModelHasher m;
  m.val(d->nb);
  m.arr(d->periodic, 3);
  m.arr(d->mus, (size_t)d->nb);
  m.arr(d->gyro, (size_t)d->nb);
  m.arr(d->alpha, (size_t)d->nb);
  m.val(d->gilbert_prefactor);
  m.val(d->rk4_normalise_stages);
  m.val(d->n_terms);
  for (int t = 0; t < d->n_terms; ++t) {
    const llg_term& T = d->terms[t];
    const size_t nb = (size_t)d->nb;
    m.val(T.kind);
    m.val(T.order);
    switch (T.kind) {
      case LLG_TERM_EXCHANGE: {
        const size_t ni = T.n_int > 0 ? (size_t)T.n_int : 0;
        m.arr(T.bi, ni);
        m.arr(T.bj, ni);
        m.arr(T.T, 3 * ni);
        m.arr(T.J, 9 * ni);
        break;
      }
      case LLG_TERM_UNIAXIAL:
      case LLG_TERM_CUBIC:
        m.arr(T.K, nb);
        m.arr(T.axis, nb * (T.kind == LLG_TERM_CUBIC ? 9 : 3));
        break;
      case LLG_TERM_APPLIED_FIELD:
        m.arr(T.B, 3);
        m.val(T.pulse);
        m.val(T.time_center);
        m.val(T.freq_bandwidth);
        m.val(T.freq_center);
        break;
      case LLG_TERM_DIPOLE:
        m.val(T.r_cutoff);
        m.val(T.distance_tolerance);
        m.val(T.lattice_parameter);
        m.arr(T.lattice_vectors, 9);
        m.arr(T.positions, 3 * nb);
        break;
      case LLG_TERM_ZEEMAN:
        m.arr(T.dc_field, 3 * nb);
        m.arr(T.ac_field, 3 * nb);
        if (T.ac_field) m.arr(T.ac_frequency, nb);
        break;
      default:
        break;
    }
  }
  return m.h;
}

int build(llg_handle* h, const llg_desc* d) {
  if (!d) return h->fail(LLG_ERR_BAD_DESC, "null descriptor");
  if (d->abi_version != LLG_ABI_VERSION)
    return h->fail(LLG_ERR_BAD_DESC, "abi_version %d, library has %d", d->abi_version, LLG_ABI_VERSION);
  if (d->nb < 1 || d->nb > kMaxBasis) return h->fail(LLG_ERR_BAD_DESC, "nb must be in [1, %d]", kMaxBasis);
  if (d->n_terms < 0 || d->n_terms > kMaxTerms)
    return h->fail(LLG_ERR_BAD_DESC, "n_terms must be in [0, %d]", kMaxTerms);
  if (d->n_terms > 0 && !d->terms) return h->fail(LLG_ERR_BAD_DESC, "terms is null");
  if (d->n_replicas < 1 || !d->replicas) return h->fail(LLG_ERR_BAD_DESC, "need at least one replica");
  if (!(d->dt > 0.0) || !std::isfinite(d->dt)) return h->fail(LLG_ERR_BAD_DESC, "dt must be positive");
  if (!d->mus || !d->gyro || !d->alpha) return h->fail(LLG_ERR_BAD_DESC, "material arrays are null");
  if (d->precision != LLG_FP64 && d->precision != LLG_FP32C)
    return h->fail(LLG_ERR_BAD_DESC, "unknown precision %d", d->precision);
  if (d->integrator != LLG_HEUN && d->integrator != LLG_RK4)
    return h->fail(LLG_ERR_BAD_DESC, "unknown integrator %d", d->integrator);
  h->fp64 = d->precision == LLG_FP64;
  h->integrator = d->integrator;
  h->nb = d->nb;
  h->nterms = d->n_terms;
  h->dt = d->dt;
  h->gilbert = d->gilbert_prefactor != 0;
  h->steps_per_graph = d->steps_per_graph > 0 ? d->steps_per_graph : 100;
  for (int b = 0; b < d->nb; ++b) {
    h->mus[b] = d->mus[b];
    h->gyro[b] = d->gyro[b];
    h->alpha[b] = d->alpha[b];
    if (!(d->mus[b] > 0.0)) return h->fail(LLG_ERR_BAD_DESC, "mu_s of basis site %d must be positive", b);
  }

  Params& P = h->P;
  P = Params{};
  P.nb = d->nb;
  P.nterms = d->n_terms;
  P.dt = d->dt;
  P.dt32 = (float)d->dt;
  P.seed = d->seed;
  {
    uint32_t k0 = (uint32_t)d->seed, k1 = (uint32_t)(d->seed >> 32);
    for (int r = 0; r < 10; ++r) {
      P.philox_keys[2 * r] = k0;
      P.philox_keys[2 * r + 1] = k1;
      k0 += 0x9E3779B9u;  // Weyl key schedule of Philox4x32
      k1 += 0xBB67AE85u;
    }
  }
  P.rk4_normalise_stages = d->rk4_normalise_stages;
  for (int b = 0; b < d->nb; ++b) {
    P.mus[b] = d->mus[b];
    P.gyro[b] = d->gyro[b];
    P.alpha[b] = d->alpha[b];
    // src/jams/solvers/cpu_llg_heun.cc:36-43
    double denominator = 1.0;
    if (h->gilbert) denominator = 1.0 + d->alpha[b] * d->alpha[b];
    P.sigma[b] = std::sqrt((2.0 * kBoltzmannIU * d->alpha[b]) / (d->mus[b] * d->gyro[b] * d->dt * denominator));
    P.inv_mus32[b] = (float)(1.0 / d->mus[b]);
    P.mus32[b] = (float)d->mus[b];
    P.gyro32[b] = (float)d->gyro[b];
    P.alpha32[b] = (float)d->alpha[b];
  }

  // terms
  std::vector<ExchangeHost> ex;
  h->term_B.assign((size_t)d->n_terms * 3, 0.0);
  int field_terms = 0, zeeman_terms = 0;
  for (int t = 0; t < d->n_terms; ++t) {
    const llg_term& T = d->terms[t];
    TermDev& TD = P.term[t];
    TD.kind = T.kind;
    TD.order = T.order;
    TD.exch = -1;
    switch (T.kind) {
      case LLG_TERM_EXCHANGE: {
        if ((int)ex.size() >= kMaxExchange)
          return h->fail(LLG_ERR_UNSUPPORTED, "more than %d exchange terms", kMaxExchange);
        if (T.n_int < 0 || (T.n_int > 0 && (!T.bi || !T.bj || !T.T || !T.J)))
          return h->fail(LLG_ERR_BAD_DESC, "exchange term %d has null arrays", t);
        for (int e = 0; e < T.n_int; ++e) {
          if (T.bi[e] < 0 || T.bi[e] >= d->nb || T.bj[e] < 0 || T.bj[e] >= d->nb)
            return h->fail(LLG_ERR_BAD_DESC, "exchange term %d entry %d: basis index outside [0, %d)", t, e,
                           d->nb);
          for (int a = 0; a < 9; ++a)
            if (!std::isfinite(T.J[9 * e + a]))
              return h->fail(LLG_ERR_BAD_DESC, "exchange term %d entry %d: non-finite J", t, e);
        }
        ExchangeHost X;
        X.term = t;
        int rc = build_slots(h, T, X);
        if (rc) return rc;
        TD.exch = (int)ex.size();
        ex.push_back(std::move(X));
        break;
      }
      case LLG_TERM_UNIAXIAL:
      case LLG_TERM_CUBIC: {
        if (!T.K || !T.axis) return h->fail(LLG_ERR_BAD_DESC, "anisotropy term %d has null arrays", t);
        if (T.kind == LLG_TERM_UNIAXIAL && !(T.order == 2 || T.order == 4 || T.order == 6))
          return h->fail(LLG_ERR_BAD_DESC, "uniaxial power must be 2, 4 or 6");
        if (T.kind == LLG_TERM_CUBIC && !(T.order == 1 || T.order == 2))
          return h->fail(LLG_ERR_BAD_DESC, "cubic order must be 1 or 2");
        const int na = T.kind == LLG_TERM_UNIAXIAL ? 3 : 9;
        for (int b = 0; b < d->nb; ++b) {
          TD.K[b] = T.K[b];
          TD.Kf[b] = (float)T.K[b];
          for (int a = 0; a < na; ++a) {
            TD.axis[b][a] = T.axis[na * b + a];
            TD.axisf[b][a] = (float)T.axis[na * b + a];
          }
        }
        break;
      }
      case LLG_TERM_APPLIED_FIELD:
        for (int a = 0; a < 3; ++a) h->term_B[3 * t + a] = T.B[a];
        if (T.pulse < LLG_PULSE_STATIC || T.pulse > LLG_PULSE_SINC_COS)
          return h->fail(LLG_ERR_BAD_DESC, "applied-field term %d: unknown pulse type %d", t, T.pulse);
        if (!std::isfinite(T.time_center) || !std::isfinite(T.freq_bandwidth) || !std::isfinite(T.freq_center))
          return h->fail(LLG_ERR_BAD_DESC, "applied-field term %d: non-finite pulse parameters", t);
        h->pulse_type = T.pulse;
        h->pulse_tc = T.time_center;
        h->pulse_fbw = T.freq_bandwidth;
        h->pulse_fc = T.freq_center;
        if (T.pulse != LLG_PULSE_STATIC) h->pulsed = true;
        ++field_terms;
        break;
      case LLG_TERM_ZEEMAN: {
        // mu_s B_dc and mu_s B_ac per basis site, as dc_local_field and
        // ac_local_field (src/jams/hamiltonian/zeeman.cc:26-71)
        if (!T.dc_field || (T.ac_field && !T.ac_frequency))
          return h->fail(LLG_ERR_BAD_DESC, "zeeman term %d: dc field per basis site, ac field with its frequency", t);
        TD.order = T.ac_field ? 1 : 0;
        for (int b = 0; b < d->nb; ++b) {
          for (int a = 0; a < 3; ++a) {
            const double dc = T.dc_field[3 * b + a] * d->mus[b];
            const double ac = T.ac_field ? T.ac_field[3 * b + a] * d->mus[b] : 0.0;
            if (!std::isfinite(dc) || !std::isfinite(ac))
              return h->fail(LLG_ERR_BAD_DESC, "zeeman term %d: non-finite field", t);
            TD.axis[b][a] = dc;
            TD.axis[b][3 + a] = ac;
            TD.axisf[b][a] = (float)dc;
            TD.axisf[b][3 + a] = (float)ac;
          }
          if (T.ac_field) {
            if (!std::isfinite(T.ac_frequency[b]))
              return h->fail(LLG_ERR_BAD_DESC, "zeeman term %d: non-finite frequency", t);
            h->zeeman_w[b] = 2.0 * kPi * T.ac_frequency[b];
          }
        }
        if (T.ac_field) h->zeeman_ac = h->pulsed = true;
        ++zeeman_terms;
        break;
      }
      case LLG_TERM_DIPOLE: {
        if (h->has_dipole) return h->fail(LLG_ERR_UNSUPPORTED, "more than one dipole term");
        if (!T.lattice_vectors || !T.positions)
          return h->fail(LLG_ERR_BAD_DESC, "dipole term %d needs lattice_vectors and positions", t);
        if (!(T.r_cutoff > 0.0) || !(T.lattice_parameter > 0.0) || !(T.distance_tolerance >= 0.0) ||
            !std::isfinite(T.r_cutoff) || !std::isfinite(T.lattice_parameter))
          return h->fail(LLG_ERR_BAD_DESC, "dipole term %d: r_cutoff and lattice_parameter must be positive", t);
        DipoleGeometry& G = h->dip_geom;
        G.r_cutoff = T.r_cutoff;
        G.tolerance = T.distance_tolerance;
        G.a = T.lattice_parameter;
        for (int a = 0; a < 9; ++a) G.A[a] = T.lattice_vectors[a];
        for (int b = 0; b < d->nb; ++b)
          for (int a = 0; a < 3; ++a) G.frac[b][a] = T.positions[3 * b + a];
        h->has_dipole = true;
        break;
      }
      default:
        return h->fail(LLG_ERR_BAD_DESC, "unknown term kind %d", T.kind);
    }
  }
  if (field_terms > 1) return h->fail(LLG_ERR_UNSUPPORTED, "at most one applied-field term");
  if (zeeman_terms > 1) return h->fail(LLG_ERR_UNSUPPORTED, "at most one zeeman term");
  P.nexch = (int)ex.size();

  // stencil reach over all exchange terms
  int reach[3] = {0, 0, 0};
  for (auto& X : ex) {
    const llg_term& T = d->terms[X.term];
    for (int e = 0; e < T.n_int; ++e)
      for (int l = 0; l < 3; ++l) reach[l] = std::max(reach[l], std::abs(T.T[3 * e + l]));
  }

  // replicas, tiles and tables
  std::vector<int32_t> tab32;
  std::vector<int2> tab64;
  std::vector<int32_t> cnt64;
  int64_t offset = 0;
  h->reps.resize(d->n_replicas);
  h->rep_T.resize(d->n_replicas);
  h->rep_first_tile.resize(d->n_replicas);
  h->rep_ntiles.resize(d->n_replicas);
  for (int r = 0; r < d->n_replicas; ++r) {
    const llg_replica& rp = d->replicas[r];
    ReplicaDev R{};
    int64_t n = (int64_t)d->nb;
    for (int l = 0; l < 3; ++l) {
      if (rp.L[l] < 1) return h->fail(LLG_ERR_BAD_DESC, "replica %d: lattice size must be positive", r);
      if (reach[l] > rp.L[l] && d->periodic[l])
        return h->fail(LLG_ERR_BAD_DESC, "replica %d: interaction reach %d exceeds lattice size %d on axis %d",
                       r, reach[l], rp.L[l], l);
      R.L[l] = rp.L[l];
      R.R[l] = reach[l];
      R.ncls[l] = axis_classes(rp.L[l], reach[l]);
      n *= rp.L[l];
    }
    if (n > (int64_t)INT32_MAX / 2) return h->fail(LLG_ERR_UNSUPPORTED, "replica %d has too many spins", r);
    if (!(rp.temperature >= 0.0) || !std::isfinite(rp.temperature))
      return h->fail(LLG_ERR_BAD_DESC, "replica %d: temperature must be >= 0", r);
    R.n = (int32_t)n;
    R.offset = offset;
    offset += (n + 63) / 64 * 64;
    h->rep_T[r] = rp.temperature;
    for (int a = 0; a < 3; ++a) {
      double B = 0.0;
      for (int t = 0; t < d->n_terms; ++t)
        if (d->terms[t].kind == LLG_TERM_APPLIED_FIELD) B = d->terms[t].B[a];
      if (rp.use_B) B = rp.B[a];
      R.B[a] = B;
      R.Bf[a] = (float)B;
    }
    const int ncl = R.ncls[0] * R.ncls[1] * R.ncls[2];
    for (size_t x = 0; x < ex.size(); ++x) {
      ExchangeHost& X = ex[x];
      const llg_term& T = d->terms[X.term];
      R.tab32[x] = (int64_t)tab32.size();
      R.tab64[x] = (int64_t)tab64.size();
      R.cnt64[x] = (int64_t)cnt64.size();
      tab32.resize(tab32.size() + (size_t)d->nb * ncl * std::max(X.nslot_max, 1), kMissing);
      tab64.resize(tab64.size() + (size_t)d->nb * ncl * std::max(X.zmax, 1), make_int2(0, 0));
      cnt64.resize(cnt64.size() + (size_t)d->nb * ncl, 0);
      for (int b = 0; b < d->nb; ++b)
        for (int k1 = 0; k1 < R.ncls[0]; ++k1)
          for (int k2 = 0; k2 < R.ncls[1]; ++k2)
            for (int k3 = 0; k3 < R.ncls[2]; ++k3) {
              const int q = (k1 * R.ncls[1] + k2) * R.ncls[2] + k3;
              const int c[3] = {class_rep(k1, R.L[0], R.R[0], R.ncls[0]), class_rep(k2, R.L[1], R.R[1], R.ncls[1]),
                                class_rep(k3, R.L[2], R.R[2], R.ncls[2])};
              const int64_t i = (((int64_t)c[0] * R.L[1] + c[1]) * R.L[2] + c[2]) * d->nb + b;
              // neighbour offset of every entry of this basis site (INT64_MIN: outside)
              std::vector<std::pair<int64_t, int>> nbrs;
              std::map<int, int64_t> off_of_entry;
              for (int e = 0; e < T.n_int; ++e) {
                if (T.bi[e] != b) continue;
                int64_t w[3];
                bool outside = false;
                for (int l = 0; l < 3; ++l) {
                  int64_t v = (int64_t)c[l] + T.T[3 * e + l];
                  if (!d->periodic[l] && (v < 0 || v >= R.L[l])) {
                    outside = true;
                    break;
                  }
                  v = ((v % R.L[l]) + R.L[l]) % R.L[l];
                  w[l] = v;
                }
                if (outside) continue;
                const int64_t j = ((w[0] * R.L[1] + w[1]) * R.L[2] + w[2]) * d->nb + T.bj[e];
                nbrs.push_back({j, e});
                off_of_entry[e] = j - i;
              }
              std::sort(nbrs.begin(), nbrs.end());
              for (size_t k = 1; k < nbrs.size(); ++k)
                if (nbrs[k].first == nbrs[k - 1].first)
                  return h->fail(LLG_ERR_BAD_DESC,
                                 "Multiple interactions for sites %lld and %lld (replica %d, term %d)",
                                 (long long)i, (long long)nbrs[k].first, r, X.term);
              // FP64 list in ascending j (zero tensors skipped as the reference does)
              const size_t base64 = R.tab64[x] + ((size_t)b * ncl + q) * std::max(X.zmax, 1);
              int cnt = 0;
              for (auto& nj : nbrs) {
                if (X.mask[nj.second] == 0) continue;
                tab64[base64 + cnt] = make_int2((int)(nj.first - i), nj.second);
                ++cnt;
              }
              cnt64[R.cnt64[x] + (size_t)b * ncl + q] = cnt;
              // FP32 slots
              const size_t base32 = R.tab32[x] + ((size_t)b * ncl + q) * std::max(X.nslot_max, 1);
              for (size_t s = 0; s < X.slot_entry[b].size(); ++s) {
                auto it = off_of_entry.find(X.slot_entry[b][s]);
                tab32[base32 + s] = it == off_of_entry.end() ? kMissing : (int32_t)it->second;
              }
            }
    }
    h->rep_first_tile[r] = (int)h->tiles.size();
    for (int64_t s = 0; s < n; s += kBlock) h->tiles.push_back(make_int2(r, (int)s));
    h->rep_ntiles[r] = (int)h->tiles.size() - h->rep_first_tile[r];
    h->reps[r] = R;
  }
  // tile views (X, Y, Z) of every replica
  for (auto& R : h->reps) {
    const int64_t nbl = d->nb;
    R.vL[0] = R.L[0];
    R.vL[1] = R.L[1];
    R.vL[2] = R.L[2];
    R.vs[0] = (int64_t)R.L[1] * R.L[2] * nbl;
    R.vs[1] = (int64_t)R.L[2] * nbl;
    R.vs[2] = nbl;
    R.vper[0] = d->periodic[0];
    R.vper[1] = d->periodic[1];
    R.vper[2] = d->periodic[2];
  }
  int n_uni = 0, n_cub = 0;
  for (int t = 0; t < d->n_terms; ++t) {
    n_uni += d->terms[t].kind == LLG_TERM_UNIAXIAL;
    n_cub += d->terms[t].kind == LLG_TERM_CUBIC;
  }
  // FP32C: several exchange terms (isotropic exchange and DMI given as
  // separate modules, say) are summed per (site, translation, partner) into
  // one template, in term order and in FP64, which then has to match a
  // stencil family.  The reference sums their fields term by term
  // (src/jams/core/solver.cc:43-57); the FP32C form rounds once.
  std::vector<int32_t> m_bi, m_bj, m_T;
  std::vector<double> m_J;
  llg_term merged{};
  if (!h->fp64 && ex.size() > 1) {
    std::map<std::array<int32_t, 5>, size_t> at;
    for (const ExchangeHost& X : ex) {
      const llg_term& t = d->terms[X.term];
      for (int e = 0; e < t.n_int; ++e) {
        const std::array<int32_t, 5> key = {t.bi[e], t.T[3 * e], t.T[3 * e + 1], t.T[3 * e + 2], t.bj[e]};
        auto it = at.find(key);
        if (it == at.end()) {
          it = at.emplace(key, m_bi.size()).first;
          m_bi.push_back(key[0]);
          m_T.insert(m_T.end(), {key[1], key[2], key[3]});
          m_bj.push_back(key[4]);
          m_J.insert(m_J.end(), 9, 0.0);
        }
        for (int a = 0; a < 9; ++a) m_J[9 * it->second + a] += t.J[9 * e + a];
      }
    }
    merged.kind = LLG_TERM_EXCHANGE;
    merged.n_int = (int32_t)m_bi.size();
    merged.bi = m_bi.data();
    merged.bj = m_bj.data();
    merged.T = m_T.data();
    merged.J = m_J.data();
  }
  if (!h->fp64 && !ex.empty() && n_uni <= 1 && n_cub <= 1) {
    const llg_term& T = ex.size() == 1 ? d->terms[ex[0].term] : merged;
    h->family = find_family(d, T, h->TP);
    if (h->family != kFamNone) {
      h->tiled = true;
      h->TP.exch_term = ex[0].term;
      tiled_geometry(h->family, &h->tz, &h->ty);
      if (h->family == kFamTRI) {
        // monolayer: the contiguous axis is a2, the trivial axis a3
        for (auto& R : h->reps) {
          R.vL[1] = R.L[2];
          R.vL[2] = R.L[1];
          std::swap(R.vs[1], R.vs[2]);
          R.vper[1] = d->periodic[2];
          R.vper[2] = d->periodic[1];
        }
      }
      int maxL = 1;
      for (auto& R : h->reps) maxL = std::max(maxL, R.vL[0]);
      h->TP.TX = std::min(8, maxL + (maxL & 1));
    }
  }
  h->npad = std::max<int64_t>(offset, 64);
  P.npad = h->npad;
  P.ntiles = (int)h->tiles.size();
  for (size_t x = 0; x < ex.size(); ++x) {
    ExchangeHost& X = ex[x];
    P.nslot_max[x] = std::max(X.nslot_max, 1);
    P.zmax[x] = std::max(X.zmax, 1);
    ExchangeF32& E = P.ex32[x];
    for (int b = 0; b < d->nb; ++b) {
      E.nslot[b] = (int)X.slot_entry[b].size();
      E.ngroup[b] = (int)X.group_end[b].size();
      for (size_t g = 0; g < X.group_end[b].size(); ++g) {
        E.group_end[b][g] = X.group_end[b][g];
        const float hi = (float)X.group_j[b][g];
        E.group_j_hi[b][g] = hi;
        E.group_j_lo[b][g] = (float)(X.group_j[b][g] - (double)hi);
      }
      E.nrest[b] = E.nslot[b] - (E.ngroup[b] ? E.group_end[b][E.ngroup[b] - 1] : 0);
    }
  }

  // device
  cudaError_t ce = cudaSetDevice(d->device);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "cudaSetDevice");
  h->device = d->device;
  cudaDeviceProp prop;
  ce = cudaGetDeviceProperties(&prop, d->device);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "cudaGetDeviceProperties");
  if (prop.major != 10 || prop.minor != 3)
    return h->fail(LLG_ERR_NO_DEVICE, "device %d is sm_%d%d; this library is built for sm_103a", d->device,
                   prop.major, prop.minor);
  ce = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "cudaStreamCreate");
  h->stream = h->own_stream;

  const size_t rs = real_size(h);
  for (int k = 0; k < 3; ++k) {
    ce = h->state[k].alloc((size_t)3 * h->npad * rs);
    if (ce != cudaSuccess) return h->cuda_fail(ce, "allocating spin planes");
    cudaMemsetAsync(h->state[k].p, 0, (size_t)3 * h->npad * rs, h->stream);
  }
  const bool need_aux = true;  // FP64 Heun ds, RK4 k sum, tiled Heun stored rhs
  if (need_aux) {
    ce = h->aux.alloc((size_t)3 * h->npad * rs);
    if (ce != cudaSuccess) return h->cuda_fail(ce, "allocating integrator scratch");
    cudaMemsetAsync(h->aux.p, 0, (size_t)3 * h->npad * rs, h->stream);
  }
  struct Up {
    void* dst;
    const void* src;
    size_t bytes;
  };
  std::vector<Up> ups;
  if ((ce = h->d_rep.alloc(h->reps.size())) != cudaSuccess) return h->cuda_fail(ce, "alloc");
  if ((ce = h->d_tiles.alloc(h->tiles.size())) != cudaSuccess) return h->cuda_fail(ce, "alloc");
  if ((ce = h->d_tab32.alloc(std::max<size_t>(tab32.size(), 1))) != cudaSuccess) return h->cuda_fail(ce, "alloc");
  if ((ce = h->d_tab64.alloc(std::max<size_t>(tab64.size(), 1))) != cudaSuccess) return h->cuda_fail(ce, "alloc");
  if ((ce = h->d_cnt64.alloc(std::max<size_t>(cnt64.size(), 1))) != cudaSuccess) return h->cuda_fail(ce, "alloc");
  if ((ce = h->d_status.alloc(1)) != cudaSuccess) return h->cuda_fail(ce, "alloc");
  if ((ce = h->h_status.alloc()) != cudaSuccess) return h->cuda_fail(ce, "alloc");
  if ((ce = h->d_step_base.alloc(1)) != cudaSuccess) return h->cuda_fail(ce, "alloc");
  if ((ce = h->d_ticket.alloc(1)) != cudaSuccess) return h->cuda_fail(ce, "alloc");
  ups.push_back({h->d_tiles.p, h->tiles.data(), h->tiles.size() * sizeof(int2)});
  if (!tab32.empty()) ups.push_back({h->d_tab32.p, tab32.data(), tab32.size() * sizeof(int32_t)});
  if (!tab64.empty()) ups.push_back({h->d_tab64.p, tab64.data(), tab64.size() * sizeof(int2)});
  if (!cnt64.empty()) ups.push_back({h->d_cnt64.p, cnt64.data(), cnt64.size() * sizeof(int32_t)});
  for (size_t x = 0; x < ex.size(); ++x) {
    if ((ce = h->d_rest[x].alloc(ex[x].rest_j.size())) != cudaSuccess) return h->cuda_fail(ce, "alloc");
    if ((ce = h->d_J64[x].alloc(std::max<size_t>(ex[x].J64.size(), 1))) != cudaSuccess)
      return h->cuda_fail(ce, "alloc");
    if ((ce = h->d_mask[x].alloc(std::max<size_t>(ex[x].mask.size(), 1))) != cudaSuccess)
      return h->cuda_fail(ce, "alloc");
    ups.push_back({h->d_rest[x].p, ex[x].rest_j.data(), ex[x].rest_j.size() * sizeof(float)});
    if (!ex[x].J64.empty()) ups.push_back({h->d_J64[x].p, ex[x].J64.data(), ex[x].J64.size() * sizeof(double)});
    if (!ex[x].mask.empty())
      ups.push_back({h->d_mask[x].p, ex[x].mask.data(), ex[x].mask.size() * sizeof(uint16_t)});
    P.ex32[x].rest_j = h->d_rest[x].p;
    P.ex64[x].J = h->d_J64[x].p;
    P.ex64[x].mask = h->d_mask[x].p;
  }
  for (auto& u : ups) {
    ce = cudaMemcpy(u.dst, u.src, u.bytes, cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) return h->cuda_fail(ce, "uploading tables");
  }
  cudaMemsetAsync(h->d_status.p, 0, sizeof(unsigned int), h->stream);
  cudaMemsetAsync(h->d_step_base.p, 0, sizeof(uint64_t), h->stream);
  cudaMemsetAsync(h->d_ticket.p, 0, sizeof(unsigned int), h->stream);
  P.tab32 = h->d_tab32.p;
  P.tab64 = h->d_tab64.p;
  P.cnt64 = h->d_cnt64.p;
  P.tiles = h->d_tiles.p;
  P.rep = h->d_rep.p;
  P.status = h->d_status.p;
  P.step_base = h->d_step_base.p;
  P.ticket = h->d_ticket.p;
  if (h->pulsed) {
    // factor table of pulse_cap steps (a multiple of the even graph block)
    const int ns = h->integrator == LLG_HEUN ? 2 : 4;
    const int K = h->steps_per_graph + (h->steps_per_graph & 1);
    h->pulse_cap = K * std::max(1, 4096 / K);
    const size_t nv = (size_t)h->pulse_cap * ns * kPulseVals;
    const size_t bytes = 16 + nv * (sizeof(double) + sizeof(float));
    if ((ce = h->d_pulse.alloc(bytes)) != cudaSuccess) return h->cuda_fail(ce, "alloc");
    for (int k = 0; k < 2; ++k) {
      if ((ce = h->pulse_host[k].alloc(bytes)) != cudaSuccess) return h->cuda_fail(ce, "pinned alloc");
      if ((ce = cudaEventCreateWithFlags(&h->pulse_ev[k], cudaEventDisableTiming)) != cudaSuccess)
        return h->cuda_fail(ce, "cudaEventCreate");
    }
    P.pulse_base = reinterpret_cast<const uint64_t*>(h->d_pulse.p);
    P.pulse64 = reinterpret_cast<const double*>(h->d_pulse.p + 16);
    P.pulse32 = reinterpret_cast<const float*>(h->d_pulse.p + 16 + nv * sizeof(double));
    P.pulse_stages = ns;
    const size_t now_bytes = kPulseVals * (sizeof(double) + sizeof(float));
    if ((ce = h->d_pulse_now.alloc(now_bytes)) != cudaSuccess) return h->cuda_fail(ce, "alloc");
    if ((ce = h->pulse_now_host.alloc(now_bytes)) != cudaSuccess) return h->cuda_fail(ce, "pinned alloc");
    P.pulse_now64 = reinterpret_cast<const double*>(h->d_pulse_now.p);
    P.pulse_now32 = reinterpret_cast<const float*>(h->d_pulse_now.p + kPulseVals * sizeof(double));
  }
  size_t maxn = 0;
  for (auto& R : h->reps) maxn = std::max<size_t>(maxn, (size_t)R.n);
  if ((ce = h->d_scratch.alloc(3 * maxn)) != cudaSuccess) return h->cuda_fail(ce, "alloc");
  size_t max_tiles = 0;
  for (int r = 0; r < d->n_replicas; ++r) max_tiles = std::max<size_t>(max_tiles, h->rep_ntiles[r]);
  const size_t nq = 4 + (size_t)kMaxTerms + 4 * (size_t)kMaxBasis;
  if ((ce = h->d_partials.alloc(std::max<size_t>(max_tiles, 1) * nq)) != cudaSuccess) return h->cuda_fail(ce, "alloc");
  h->h_partials.resize(std::max<size_t>(max_tiles, 1) * nq);
  h->params_dirty = true;
  if (h->tiled) {
    int rc = build_tiles4(h);
    if (rc) return rc;
  }
  if (h->has_dipole) {
    std::vector<DipoleReplicaSpec> specs;
    for (auto& R : h->reps) {
      DipoleReplicaSpec sp;
      for (int a = 0; a < 3; ++a) sp.L[a] = R.L[a];
      sp.offset = R.offset;
      specs.push_back(sp);
    }
    std::string err;
    h->dipole = dipole_create(h->dip_geom, d->nb, d->periodic, d->mus, specs, h->fp64, err);
    if (!h->dipole) return h->fail(LLG_ERR_BAD_DESC, "%s", err.c_str());
    for (auto& b : h->d_hdip)
      if ((ce = b.alloc((size_t)3 * h->npad * real_size(h))) != cudaSuccess) return h->cuda_fail(ce, "alloc");
  }
  return 0;
}

// Params of one launch: the dipole field planes of the launch's input state
// (computed here, on the stream, when the model has a dipole term) and of
// the start-of-step state
Params launch_params(llg_handle* h, const void* input, int slot) {
  Params P = h->P;
  if (!h->dipole) return P;
  if (input) {
    const std::string err = dipole_compute(h->dipole, input, h->d_hdip[slot].p, h->npad, h->stream);
    if (!err.empty() && h->async_err.empty()) h->async_err = err;
  }
  if (h->fp64) {
    P.hdip64 = reinterpret_cast<const double*>(h->d_hdip[slot].p);
    P.hdip64_s0 = reinterpret_cast<const double*>(h->d_hdip[0].p);
  } else {
    P.hdip32 = reinterpret_cast<const float*>(h->d_hdip[slot].p);
    P.hdip32_s0 = reinterpret_cast<const float*>(h->d_hdip[0].p);
  }
  return P;
}

// uploads replica records (temperature- and field-dependent parts)
// zeros in the stored-noise planes of every replica at 0 K
cudaError_t clear_cold_noise(llg_handle* h) {
  if (!h->noise.p) return cudaSuccess;
  for (size_t r = 0; r < h->reps.size(); ++r) {
    if (h->rep_T[r] > 0.0) continue;
    for (int m = 0; m < 3; ++m) {
      const cudaError_t ce = cudaMemsetAsync(h->noise.p + (size_t)m * h->npad + h->reps[r].offset, 0,
                                             (size_t)h->reps[r].n * sizeof(float), h->stream);
      if (ce != cudaSuccess) return ce;
    }
  }
  return cudaSuccess;
}

int sync_replicas(llg_handle* h) {
  if (!h->params_dirty) return 0;
  for (size_t r = 0; r < h->reps.size(); ++r) {
    ReplicaDev& R = h->reps[r];
    const double T = h->rep_T[r];
    R.thermal = T > 0.0 ? 1 : 0;
    R.sqrt_t = std::sqrt(T);
    for (int b = 0; b < h->nb; ++b) R.amp32[b] = (float)(h->P.sigma[b] * R.sqrt_t);
  }
  cudaError_t ce = cudaMemcpyAsync(h->d_rep.p, h->reps.data(), h->reps.size() * sizeof(ReplicaDev),
                                   cudaMemcpyHostToDevice, h->stream);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "uploading replica records");
  // stored noise: the predictor writes the thermal field of replicas above
  // 0 K only, and the corrector reads every replica's, so a replica at 0 K
  // reads zeros
  ce = clear_cold_noise(h);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "clearing the noise planes");
  // pageable source: make sure the copy has consumed it before the vector changes
  ce = cudaStreamSynchronize(h->stream);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "uploading replica records");
  h->params_dirty = false;
  return 0;
}

template <typename Real>
Real* buf(llg_handle* h, int k) {
  return reinterpret_cast<Real*>(h->state[k].p);
}

int num_stages(const llg_handle* h) { return h->integrator == LLG_HEUN ? 2 : 4; }
// launches per stage: the stage kernel and, where the model has a dipole
// term, the transform kernels of the field evaluation before it
int64_t stage_launches(const llg_handle* h) { return 1 + (h->dipole ? dipole_launches(h->dipole) : 0); }

// time factors at solver time t (ps), the reference's double expressions:
// f[0] = sinc(pi f_bw (t - t_c)), f[1] = cos(2 pi f_c (t - t_c)) of the
// applied-field pulse (src/jams/hamiltonian/applied_field.cc:17-78,
// src/jams/helpers/maths.h:437-446; 1 where the pulse has no such factor),
// f[2 + b] = cos(w_b t) of the zeeman ac field (zeeman.cc:115-117)
void pulse_factors(const llg_handle* h, double t, double* f) {
  f[0] = 1.0;
  f[1] = 1.0;
  if (h->pulse_type != LLG_PULSE_STATIC) {
    const double x = kPi * h->pulse_fbw * (t - h->pulse_tc);
    f[0] = x == 0.0 ? 1.0 : std::sin(x) / x;
    if (h->pulse_type == LLG_PULSE_SINC_COS) f[1] = std::cos(2.0 * kPi * h->pulse_fc * (t - h->pulse_tc));
  }
  for (int b = 0; b < kMaxBasis; ++b) f[2 + b] = (h->zeeman_ac && b < h->nb) ? std::cos(h->zeeman_w[b] * t) : 1.0;
}

// the solver time of each stage of iteration n: Heun t0, t0 + dt
// (src/jams/solvers/cuda_llg_heun.cu:64-122); RK4 t0, t0 + dt/2, t0 + dt/2,
// t0 + dt (cuda_rk4_base.cu:50-108); t0 = n dt
void stage_times(const llg_handle* h, int64_t n, double* ts) {
  const double dt = h->dt, t0 = (double)n * dt;
  if (h->integrator == LLG_HEUN) {
    ts[0] = t0;
    ts[1] = t0 + dt;
  } else {
    ts[0] = t0;
    ts[1] = t0 + 0.5 * dt;
    ts[2] = t0 + 0.5 * dt;
    ts[3] = t0 + dt;
  }
}

// the factor table for iterations it0 .. it0 + nsteps - 1 (nsteps <=
// pulse_cap), enqueued on the stream before the launches that read it
int upload_pulse_table(llg_handle* h, int64_t it0, int nsteps) {
  const int ns = num_stages(h);
  const size_t nv = (size_t)h->pulse_cap * ns * kPulseVals;
  const size_t used = (size_t)nsteps * ns * kPulseVals;
  const int slot = h->pulse_slot;
  h->pulse_slot ^= 1;
  // the copy that last read this staging buffer has finished
  cudaError_t ce = cudaEventSynchronize(h->pulse_ev[slot]);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "pulse table");
  unsigned char* host = h->pulse_host[slot].p;
  const uint64_t base = (uint64_t)it0;
  std::memcpy(host, &base, sizeof base);
  double* f64 = reinterpret_cast<double*>(host + 16);
  float* f32 = reinterpret_cast<float*>(host + 16 + nv * sizeof(double));
  double ts[4];
  for (int k = 0; k < nsteps; ++k) {
    stage_times(h, it0 + k, ts);
    for (int st = 0; st < ns; ++st) {
      double* f = f64 + ((size_t)k * ns + st) * kPulseVals;
      pulse_factors(h, ts[st], f);
      for (int v = 0; v < kPulseVals; ++v) f32[((size_t)k * ns + st) * kPulseVals + v] = (float)f[v];
    }
  }
  unsigned char* dev = h->d_pulse.p;
  ce = cudaMemcpyAsync(dev, host, 16 + used * sizeof(double), cudaMemcpyHostToDevice, h->stream);
  if (ce == cudaSuccess)
    ce = cudaMemcpyAsync(dev + 16 + nv * sizeof(double), host + 16 + nv * sizeof(double), used * sizeof(float),
                         cudaMemcpyHostToDevice, h->stream);
  if (ce == cudaSuccess) ce = cudaEventRecord(h->pulse_ev[slot], h->stream);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "uploading the pulse table");
  return 0;
}

// the factors at the current solver time (iteration dt), for fields and
// energies; the caller synchronises the stream before it returns
int upload_pulse_now(llg_handle* h) {
  if (!h->pulsed) return 0;
  double* f = reinterpret_cast<double*>(h->pulse_now_host.p);
  float* f32 = reinterpret_cast<float*>(h->pulse_now_host.p + kPulseVals * sizeof(double));
  pulse_factors(h, (double)h->iteration * h->dt, f);
  for (int v = 0; v < kPulseVals; ++v) f32[v] = (float)f[v];
  cudaError_t ce = cudaMemcpyAsync(h->d_pulse_now.p, h->pulse_now_host.p,
                                   kPulseVals * (sizeof(double) + sizeof(float)), cudaMemcpyHostToDevice, h->stream);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "uploading the pulse factors");
  return 0;
}

// launches stage `stage` of step `ks` of a block; `cur` is the buffer that
// holds the state at the start of the step (FP32 Heun alternates 0 and 2).
// advance > 0: the tiled kernels advance the noise step counter by that
// much at the end of the launch (returns true; other kernels leave it to
// the caller)
bool launch_stage(llg_handle* h, int stage, uint32_t ks, int cur, cudaEvent_t after_dipole = nullptr,
                  uint32_t advance = 0) {
  // the stage's input state (whose dipole field the stage needs)
  const void* input;
  if (h->integrator == LLG_HEUN)
    input = stage == 0 ? h->state[h->fp64 ? 0 : cur].p : h->state[1].p;
  else
    input = stage == 0 ? h->state[0].p : (stage == 2 ? h->state[2].p : h->state[1].p);
  const Params P = launch_params(h, input, (h->integrator == LLG_HEUN && stage == 1) ? 1 : 0);
  if (after_dipole) cudaEventRecord(after_dipole, h->stream);
  const unsigned grid = (unsigned)P.ntiles;
  cudaStream_t st = h->stream;
  if (h->tiled) {
    const unsigned g4 = (unsigned)h->TP.ntiles;
    float* aux = reinterpret_cast<float*>(h->aux.p);
    if (h->fused) {
      // the whole step in the launch of stage 0; stage 1 has nothing to do
      if (stage == 0) {
        const cudaError_t e = launch_fused(h->family, h->fused_wide, h->occupancy, g4, st, P, h->TP,
                                           buf<float>(h, cur), buf<float>(h, 2 - cur), ks, advance);
        if (e != cudaSuccess && h->async_err.empty()) h->async_err = std::string("fused step: ") + cudaGetErrorString(e);
      }
      return true;
    }
    if (h->integrator == LLG_HEUN) {
      float* s0 = buf<float>(h, cur);
      float* sp = buf<float>(h, 1);
      // TMA: the tensor map of the buffer the stage gathers from
      const CUtensorMap* m0 = h->tma ? &h->tmaps[cur] : nullptr;
      const CUtensorMap* m1 = h->tma ? &h->tmaps[1] : nullptr;
      // stored-noise mode: stages 7 and 8 are stages 0 and 2 that write /
      // read the thermal field planes
      Params PN = P;
      if (h->store_noise) PN.noise32 = h->noise.p;
      if (stage == 0)
        launch_tiled(h->family, h->tz, h->ty, h->rpt, h->occupancy, h->store_noise ? 7 : 0, g4, st, PN, h->TP, s0, nullptr, sp, h->store_mode ? aux : nullptr, ks, advance, h->dipole != nullptr, m0);
      else if (h->store_mode)
        launch_tiled(h->family, h->tz, h->ty, h->rpt, h->occupancy, h->store_noise ? 8 : 2, g4, st, PN, h->TP, s0, sp, s0, aux, ks, advance, h->dipole != nullptr, m1);
      else
        launch_tiled(h->family, h->tz, h->ty, h->rpt, h->occupancy, 1, g4, st, P, h->TP, s0, sp, buf<float>(h, 2 - cur), nullptr, ks, advance, h->dipole != nullptr, m1);
    } else {
      float* s0 = buf<float>(h, 0);
      float* a = buf<float>(h, 1);
      float* b = buf<float>(h, 2);
      float* in = stage == 0 ? s0 : (stage == 2 ? b : a);
      float* out = stage == 0 ? a : (stage == 1 ? b : (stage == 2 ? a : s0));
      const CUtensorMap* m = h->tma ? &h->tmaps[stage == 0 ? 0 : (stage == 2 ? 2 : 1)] : nullptr;
      launch_tiled(h->family, h->tz, h->ty, h->rpt, h->occupancy, 3 + stage, g4, st, P, h->TP, s0, in, out, aux, ks, advance, h->dipole != nullptr, m);
    }
    return true;
  }
  if (h->integrator == LLG_HEUN) {
    if (h->fp64) {
      // state stays in buffer 0; 1 = predictor, aux = ds
      double* s0 = buf<double>(h, 0);
      double* sp = buf<double>(h, 1);
      double* ds = reinterpret_cast<double*>(h->aux.p);
      if (stage == 0)
        heun_predict_f64<<<grid, kBlock, 0, st>>>(P, s0, sp, ds, ks);
      else
        heun_correct_f64<<<grid, kBlock, 0, st>>>(P, s0, sp, ds, s0, ks);
    } else {
      // state alternates between buffers 0 and 2; 1 = predictor
      float* s0 = buf<float>(h, cur);
      float* sp = buf<float>(h, 1);
      float* s1 = buf<float>(h, 2 - cur);
      // s0 + dt/2 rhs(s0) stored by the predictor for the corrector
      float* rhs0 = reinterpret_cast<float*>(h->aux.p);
      if (stage == 0)
        heun_predict_f32<<<grid, kBlock, 0, st>>>(P, s0, sp, rhs0, ks);
      else
        heun_correct_f32<<<grid, kBlock, 0, st>>>(P, s0, sp, s1, rhs0, ks);
    }
  } else {
    // state stays in buffer 0; 1 and 2 hold stage states, aux the k sum
    void* s0 = h->state[0].p;
    void* a = h->state[1].p;
    void* b = h->state[2].p;
    void* in = stage == 0 ? s0 : (stage == 2 ? b : a);
    void* out = stage == 0 ? a : (stage == 1 ? b : (stage == 2 ? a : s0));
    if (h->fp64)
      launch_rk4_f64(stage + 1, grid, st, P, (const double*)s0, (const double*)in, (double*)h->aux.p,
                     (double*)out, ks);
    else
      launch_rk4_f32(stage + 1, grid, st, P, (const float*)s0, (const float*)in, (float*)h->aux.p,
                     (float*)out, ks);
  }
  return false;
}

int next_buffer(const llg_handle* h, int cur) {
  return (!h->fp64 && h->integrator == LLG_HEUN && !(h->tiled && h->store_mode)) ? 2 - cur : cur;
}

// launches `nsteps` steps starting with the state in buffer `cur`; returns
// the number of kernel launches.  The last launch advances the noise step
// counter (tiled kernels), else one more kernel does.
int64_t enqueue_steps(llg_handle* h, int nsteps, int cur) {
  const int ns = num_stages(h);
  bool advanced = false;
  if (h->fused) {
    // one launch per step; the last advances the noise step counter
    for (int k = 0; k < nsteps; ++k) {
      launch_stage(h, 0, (uint32_t)k, cur, nullptr, k == nsteps - 1 ? (uint32_t)nsteps : 0u);
      cur = next_buffer(h, cur);
    }
    return nsteps;
  }
  for (int k = 0; k < nsteps; ++k) {
    for (int stg = 0; stg < ns; ++stg) {
      const bool last = k == nsteps - 1 && stg == ns - 1;
      advanced = launch_stage(h, stg, (uint32_t)k, cur, nullptr, last ? (uint32_t)nsteps : 0u) && last;
    }
    cur = next_buffer(h, cur);
  }
  if (advanced) return (int64_t)nsteps * ns * stage_launches(h);
  advance_step_base<<<1, 1, 0, h->stream>>>(h->d_step_base.p, (uint32_t)nsteps);
  return (int64_t)nsteps * ns * stage_launches(h) + 1;
}

int state_buffer(const llg_handle* h) { return (h->fp64 || h->integrator == LLG_RK4) ? 0 : h->cur; }

}  // namespace

// =================================================================== ABI ==

extern "C" {

int llg_create(const llg_desc* desc, llg_handle** out) {
  if (!out) return tls_fail(LLG_ERR_BAD_DESC, "out is null");
  *out = nullptr;
  llg_handle* h = new (std::nothrow) llg_handle();
  if (!h) return tls_fail(LLG_ERR_OOM, "host allocation failed");
  cudaGetLastError();   // a launch error found below is this handle's own
  int rc = build(h, desc);
  if (rc == 0) h->model_hash = model_hash(desc);
  if (rc == 0) rc = sync_replicas(h);
  if (rc == 0) {
    // all spins +z
    for (int r = 0; r < (int)h->reps.size() && rc == 0; ++r) {
      std::vector<double> s((size_t)h->reps[r].n * 3, 0.0);
      for (int64_t i = 0; i < h->reps[r].n; ++i) s[3 * i + 2] = 1.0;
      rc = llg_set_state(h, r, s.data());
    }
  }
  if (rc != 0) {
    g_tls_error = h->err;
    delete h;
    return rc;
  }
  *out = h;
  return 0;
}

void llg_destroy(llg_handle* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  delete h;
}

const char* llg_last_error(const llg_handle* h) { return h ? h->err.c_str() : g_tls_error.c_str(); }

int64_t llg_num_spins(const llg_handle* h, int32_t replica) {
  if (!h) return -1;
  if (replica < 0) {
    int64_t n = 0;
    for (auto& R : h->reps) n += R.n;
    return n;
  }
  if (replica >= (int32_t)h->reps.size()) return -1;
  return h->reps[replica].n;
}

int32_t llg_num_replicas(const llg_handle* h) { return h ? (int32_t)h->reps.size() : -1; }

// the device address of a pinned, mapped host buffer (the unpack kernel then
// reads it in place over the host link, in one pass with the layout
// conversion), or null for pageable memory (copied by the DMA engines through
// the device scratch buffer)
static void* mapped_host(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

static int transfer_state(llg_handle* h, int32_t replica, const double* src, double* dst, bool device_ptr) {
  if (!h) return tls_fail(LLG_ERR_BAD_DESC, "null handle");
  if (replica >= (int32_t)h->reps.size()) return h->fail(LLG_ERR_BAD_DESC, "replica %d out of range", replica);
  cudaSetDevice(h->device);
  const int r0 = replica < 0 ? 0 : replica;
  const int r1 = replica < 0 ? (int)h->reps.size() : replica + 1;
  int64_t host_off = 0;
  const int sb = state_buffer(h);
  for (int r = r0; r < r1; ++r) {
    const ReplicaDev& R = h->reps[r];
    const size_t bytes = (size_t)R.n * 3 * sizeof(double);
    double* dev_aos = h->d_scratch.p;
    cudaError_t ce = cudaSuccess;
    if (src) {
      const double* s = src + 3 * host_off;
      if (device_ptr) {
        dev_aos = const_cast<double*>(s);
      } else if (void* m = mapped_host(s)) {
        dev_aos = static_cast<double*>(m);
      } else {
        ce = cudaMemcpyAsync(dev_aos, s, bytes, cudaMemcpyHostToDevice, h->stream);
        if (ce != cudaSuccess) return h->cuda_fail(ce, "copying spins to the device");
      }
      launch_unpack(h->fp64, h->stream, dev_aos, h->state[sb].p, R.offset, R.n, h->npad);
      if (!device_ptr) {
        ce = cudaStreamSynchronize(h->stream);
        if (ce != cudaSuccess) return h->cuda_fail(ce, "setting spins");
      }
    } else {
      // results go back through the copy engines: the pack kernel's own
      // stores into pinned host memory were as fast (78 us for 12.6 MB) on
      // some runs and 7x slower on others
      double* d = dst + 3 * host_off;
      if (device_ptr) dev_aos = d;
      launch_pack(h->fp64, h->stream, h->state[sb].p, dev_aos, R.offset, R.n, h->npad);
      if (!device_ptr) {
        ce = cudaMemcpyAsync(d, dev_aos, bytes, cudaMemcpyDeviceToHost, h->stream);
        if (ce != cudaSuccess) return h->cuda_fail(ce, "copying spins to the host");
        ce = cudaStreamSynchronize(h->stream);
        if (ce != cudaSuccess) return h->cuda_fail(ce, "getting spins");
      }
    }
    ce = cudaGetLastError();
    if (ce != cudaSuccess) return h->cuda_fail(ce, "state transfer kernel");
    host_off += R.n;
  }
  return 0;
}

int llg_set_state(llg_handle* h, int32_t replica, const double* s_host) {
  if (!s_host) return h ? h->fail(LLG_ERR_BAD_DESC, "null buffer") : tls_fail(LLG_ERR_BAD_DESC, "null buffer");
  return transfer_state(h, replica, s_host, nullptr, false);
}
int llg_get_state(llg_handle* h, int32_t replica, double* s_host) {
  if (!s_host) return h ? h->fail(LLG_ERR_BAD_DESC, "null buffer") : tls_fail(LLG_ERR_BAD_DESC, "null buffer");
  return transfer_state(h, replica, nullptr, s_host, false);
}
int llg_set_state_device(llg_handle* h, int32_t replica, const double* s_dev) {
  if (!s_dev) return h ? h->fail(LLG_ERR_BAD_DESC, "null buffer") : tls_fail(LLG_ERR_BAD_DESC, "null buffer");
  return transfer_state(h, replica, s_dev, nullptr, true);
}
int llg_get_state_device(llg_handle* h, int32_t replica, double* s_dev) {
  if (!s_dev) return h ? h->fail(LLG_ERR_BAD_DESC, "null buffer") : tls_fail(LLG_ERR_BAD_DESC, "null buffer");
  return transfer_state(h, replica, nullptr, s_dev, true);
}

// nsteps steps as CUDA-graph blocks (the pulse table, if any, covers them)
static int step_blocks(llg_handle* h, int32_t nsteps) {
  h->last_launches = 0;
  const bool alternates = next_buffer(h, 0) != 0;
  int K = h->steps_per_graph;
  if (alternates && (K & 1)) K += 1;  // full blocks return the state to the buffer they found it in
  int remaining = nsteps;
  // blocks of K steps, then the remainder, each as one CUDA-graph launch
  // (graphs cached per buffer parity, tiling and step count; remainders are
  // cached while fewer than kMaxGraphs graphs exist, else launched directly)
  constexpr size_t kMaxGraphs = 64;
  while (remaining > 0) {
    const int n = remaining >= K && K > 1 ? K : remaining;
    GraphKey key{h->cur + 4 * (h->store_mode ? 1 : 0) + 8 * h->occupancy + 64 * h->TP.TX + 8192 * h->ty +
                     131072 * h->rpt + 524288 * (h->fused ? 1 : 0) + 1048576 * (h->tma ? 1 : 0) + 2097152 * (h->store_noise ? 1 : 0) +
                     4194304 * (h->tz == 16 ? 1 : 0),
                 n};
    auto it = h->graphs.find(key);
    if (it == h->graphs.end() && (n == K || h->graphs.size() < kMaxGraphs)) {
      cudaGraph_t g;
      cudaError_t ce = cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal);
      if (ce != cudaSuccess) return h->cuda_fail(ce, "cudaStreamBeginCapture");
      enqueue_steps(h, n, h->cur);
      ce = cudaStreamEndCapture(h->stream, &g);
      if (ce != cudaSuccess) return h->cuda_fail(ce, "cudaStreamEndCapture");
      cudaGraphExec_t ge;
      ce = cudaGraphInstantiate(&ge, g, 0);
      cudaGraphDestroy(g);
      if (ce != cudaSuccess) return h->cuda_fail(ce, "cudaGraphInstantiate");
      it = h->graphs.emplace(key, ge).first;
    }
    if (it != h->graphs.end()) {
      cudaError_t ce = cudaGraphLaunch(it->second, h->stream);
      if (ce != cudaSuccess) return h->cuda_fail(ce, "cudaGraphLaunch");
      // per step: one fused kernel, or one kernel per stage (each stage
      // after the dipole term's transform kernels, where the model has one);
      // the other kernels' blocks end with the step-counter kernel
      h->last_launches += (int64_t)n * (h->fused ? 1 : num_stages(h) * stage_launches(h)) + (h->tiled ? 0 : 1);
    } else {
      h->last_launches += enqueue_steps(h, n, h->cur);
    }
    if (n & 1) h->cur = next_buffer(h, h->cur);
    remaining -= n;
    h->iteration += n;
  }
  if (!h->async_err.empty()) {
    const std::string e = h->async_err;
    h->async_err.clear();
    return h->fail(LLG_ERR_CUDA, "%s", e.c_str());
  }
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return h->cuda_fail(ce, "launching LLG steps");
  return 0;
}

int llg_step(llg_handle* h, int32_t nsteps) {
  if (!h) return tls_fail(LLG_ERR_BAD_DESC, "null handle");
  if (nsteps < 0) return h->fail(LLG_ERR_BAD_DESC, "nsteps must be >= 0");
  cudaSetDevice(h->device);
  int rc = sync_replicas(h);
  if (rc) return rc;
  if (!h->pulsed) return step_blocks(h, nsteps);
  // time-dependent fields: chunks of at most pulse_cap steps, each after
  // the upload of its factor table
  int64_t launches = 0;
  h->last_launches = 0;
  for (int done = 0; done < nsteps;) {
    const int c = std::min(nsteps - done, h->pulse_cap);
    rc = upload_pulse_table(h, h->iteration, c);
    if (rc) return rc;
    rc = step_blocks(h, c);
    launches += h->last_launches;
    if (rc) return rc;
    done += c;
  }
  h->last_launches = launches;
  return 0;
}

int llg_synchronize(llg_handle* h) {
  if (!h) return tls_fail(LLG_ERR_BAD_DESC, "null handle");
  cudaSetDevice(h->device);
  // the status word comes back with the stream's work: one synchronisation
  cudaError_t ce = cudaMemcpyAsync(h->h_status.p, h->d_status.p, sizeof(unsigned int), cudaMemcpyDeviceToHost,
                                   h->stream);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "reading status");
  ce = cudaStreamSynchronize(h->stream);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "cudaStreamSynchronize");
  if (*h->h_status.p & 2u)
    return h->fail(LLG_ERR_BOUNDS, "a kernel met an index outside its array (bounds-checked build; access skipped)");
  if (*h->h_status.p & 1u) return h->fail(LLG_ERR_NONFINITE, "a spin became NaN or infinite");
  return 0;
}

int64_t llg_iteration(const llg_handle* h) { return h ? h->iteration : -1; }

int llg_set_iteration(llg_handle* h, int64_t iteration) {
  if (!h) return tls_fail(LLG_ERR_BAD_DESC, "null handle");
  if (iteration < 0) return h->fail(LLG_ERR_BAD_DESC, "iteration must be >= 0");
  cudaSetDevice(h->device);
  uint64_t v = (uint64_t)iteration;
  cudaError_t ce = cudaMemcpyAsync(h->d_step_base.p, &v, sizeof v, cudaMemcpyHostToDevice, h->stream);
  // the completion ticket of the launch that advances the counter starts at 0
  if (ce == cudaSuccess) ce = cudaMemsetAsync(h->d_ticket.p, 0, sizeof(unsigned int), h->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(h->stream);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "setting the iteration");
  h->iteration = iteration;
  return 0;
}

int llg_set_temperature(llg_handle* h, int32_t replica, double temperature) {
  if (!h) return tls_fail(LLG_ERR_BAD_DESC, "null handle");
  if (replica < 0 || replica >= (int32_t)h->reps.size())
    return h->fail(LLG_ERR_BAD_DESC, "replica %d out of range", replica);
  if (!(temperature >= 0.0) || !std::isfinite(temperature))
    return h->fail(LLG_ERR_BAD_DESC, "temperature must be >= 0");
  h->rep_T[replica] = temperature;
  h->params_dirty = true;
  return 0;
}

int llg_set_field(llg_handle* h, int32_t replica, const double B[3]) {
  if (!h) return tls_fail(LLG_ERR_BAD_DESC, "null handle");
  if (replica < 0 || replica >= (int32_t)h->reps.size() || !B)
    return h->fail(LLG_ERR_BAD_DESC, "replica %d out of range", replica);
  for (int a = 0; a < 3; ++a) {
    h->reps[replica].B[a] = B[a];
    h->reps[replica].Bf[a] = (float)B[a];
  }
  h->params_dirty = true;
  return 0;
}

int llg_fields(llg_handle* h, int32_t replica, double* h_host) {
  if (!h) return tls_fail(LLG_ERR_BAD_DESC, "null handle");
  if (replica < 0 || replica >= (int32_t)h->reps.size() || !h_host)
    return h->fail(LLG_ERR_BAD_DESC, "replica %d out of range", replica);
  cudaSetDevice(h->device);
  int rc = sync_replicas(h);
  if (rc) return rc;
  const ReplicaDev& R = h->reps[replica];
  const dim3 grid((unsigned)h->P.ntiles);
  const int sb = state_buffer(h);
  rc = upload_pulse_now(h);   // fields at the solver time
  if (rc) return rc;
  const Params P = launch_params(h, h->state[sb].p, 0);
  if (!h->async_err.empty()) {
    const std::string e = h->async_err;
    h->async_err.clear();
    return h->fail(LLG_ERR_CUDA, "%s", e.c_str());
  }
  if (h->fp64)
    fields_f64<<<grid, kBlock, 0, h->stream>>>(P, buf<double>(h, sb), h->d_scratch.p, replica);
  else
    fields_f32<<<grid, kBlock, 0, h->stream>>>(P, buf<float>(h, sb), h->d_scratch.p, replica);
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return h->cuda_fail(ce, "fields kernel");
  ce = cudaMemcpyAsync(h_host, h->d_scratch.p, (size_t)R.n * 3 * sizeof(double), cudaMemcpyDeviceToHost,
                       h->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(h->stream);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "copying fields");
  return 0;
}

// one term's field at the current state into `out` (host or device memory)
static int term_fields(llg_handle* h, int32_t replica, int32_t term, double* out, bool device_out) {
  if (!h) return tls_fail(LLG_ERR_BAD_DESC, "null handle");
  if (replica < 0 || replica >= (int32_t)h->reps.size() || !out)
    return h->fail(LLG_ERR_BAD_DESC, "replica %d out of range", replica);
  if (term < 0 || term >= h->nterms) return h->fail(LLG_ERR_BAD_DESC, "term %d outside [0, %d)", term, h->nterms);
  cudaSetDevice(h->device);
  int rc = sync_replicas(h);
  if (rc) return rc;
  const ReplicaDev& R = h->reps[replica];
  const dim3 grid((unsigned)h->P.ntiles);
  const int sb = state_buffer(h);
  rc = upload_pulse_now(h);   // fields at the solver time
  if (rc) return rc;
  const Params P = launch_params(h, h->state[sb].p, 0);
  if (!h->async_err.empty()) {
    const std::string e = h->async_err;
    h->async_err.clear();
    return h->fail(LLG_ERR_CUDA, "%s", e.c_str());
  }
  if (h->fp64)
    term_fields_f64<<<grid, kBlock, 0, h->stream>>>(P, buf<double>(h, sb), h->d_scratch.p, replica, term);
  else
    term_fields_f32<<<grid, kBlock, 0, h->stream>>>(P, buf<float>(h, sb), h->d_scratch.p, replica, term);
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) return h->cuda_fail(ce, "term fields kernel");
  ce = cudaMemcpyAsync(out, h->d_scratch.p, (size_t)R.n * 3 * sizeof(double),
                       device_out ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(h->stream);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "copying term fields");
  return 0;
}

int llg_term_fields(llg_handle* h, int32_t replica, int32_t term, double* h_host) {
  return term_fields(h, replica, term, h_host, false);
}

int llg_term_fields_device(llg_handle* h, int32_t replica, int32_t term, double* h_dev) {
  return term_fields(h, replica, term, h_dev, true);
}

// the replica's observable sums in the observe kernel's layout: mu_s S and
// mu_s (0..3), the energy of every term (4..), mu_s S and mu_s per basis site
// (4 + nterms + 4 b ..)
static int observe_sums(llg_handle* h, int32_t replica, std::vector<double>& sum) {
  if (!h) return tls_fail(LLG_ERR_BAD_DESC, "null handle");
  if (replica < 0 || replica >= (int32_t)h->reps.size())
    return h->fail(LLG_ERR_BAD_DESC, "replica %d out of range", replica);
  cudaSetDevice(h->device);
  int rc = sync_replicas(h);
  if (rc) return rc;
  const int nq = 4 + h->nterms + 4 * h->nb;
  const int sb = state_buffer(h);
  rc = upload_pulse_now(h);   // energies at the solver time
  if (rc) return rc;
  const Params P = launch_params(h, h->state[sb].p, 0);
  if (!h->async_err.empty()) {
    const std::string e = h->async_err;
    h->async_err.clear();
    return h->fail(LLG_ERR_CUDA, "%s", e.c_str());
  }
  rc = observe(P, h->state[sb].p, h->fp64, replica, h->rep_first_tile[replica], h->rep_ntiles[replica],
               h->d_partials.p, h->h_partials.data(), nq, h->stream);
  if (rc) return h->cuda_fail(cudaGetLastError(), "observables");
  // ordered sums over tiles (deterministic), Neumaier compensation
  sum.assign(nq, 0.0);
  std::vector<double> comp(nq, 0.0);
  for (int t = 0; t < h->rep_ntiles[replica]; ++t)
    for (int q = 0; q < nq; ++q) {
      const double x = h->h_partials[(size_t)t * nq + q];
      const double s = sum[q] + x;
      comp[q] += std::fabs(sum[q]) >= std::fabs(x) ? (sum[q] - s) + x : (x - s) + sum[q];
      sum[q] = s;
    }
  for (int q = 0; q < nq; ++q) sum[q] += comp[q];
  return 0;
}

int llg_observables(llg_handle* h, int32_t replica, double* m4, double* e_terms) {
  std::vector<double> sum;
  const int rc = observe_sums(h, replica, sum);
  if (rc) return rc;
  if (m4) {
    m4[0] = sum[0] / sum[3];
    m4[1] = sum[1] / sum[3];
    m4[2] = sum[2] / sum[3];
    m4[3] = std::sqrt(sum[0] * sum[0] + sum[1] * sum[1] + sum[2] * sum[2]) / sum[3];
  }
  if (e_terms)
    for (int t = 0; t < h->nterms; ++t) e_terms[t] = sum[4 + t];
  return 0;
}

int llg_magnetisation_groups(llg_handle* h, int32_t replica, const int32_t* group_of_basis, int32_t ngroups,
                             int32_t normalize, double* m4) {
  if (!h) return tls_fail(LLG_ERR_BAD_DESC, "null handle");
  if (!group_of_basis || !m4 || ngroups < 1) return h->fail(LLG_ERR_BAD_DESC, "bad group arguments");
  for (int b = 0; b < h->nb; ++b)
    if (group_of_basis[b] < 0 || group_of_basis[b] >= ngroups)
      return h->fail(LLG_ERR_BAD_DESC, "basis site %d: group %d outside [0, %d)", b, group_of_basis[b], ngroups);
  std::vector<double> sum;
  const int rc = observe_sums(h, replica, sum);
  if (rc) return rc;
  constexpr double kBohrMagnetonIU = 0.0578838181;   // meV/T, src/jams/helpers/consts.h:30
  std::vector<double> g(4 * (size_t)ngroups, 0.0);
  for (int b = 0; b < h->nb; ++b)
    for (int k = 0; k < 4; ++k) g[4 * (size_t)group_of_basis[b] + k] += sum[4 + h->nterms + 4 * b + k];
  for (int q = 0; q < ngroups; ++q) {
    const double* x = &g[4 * (size_t)q];
    const double f = normalize ? 1.0 / x[3] : 1.0 / kBohrMagnetonIU;
    m4[4 * q] = x[0] * f;
    m4[4 * q + 1] = x[1] * f;
    m4[4 * q + 2] = x[2] * f;
    m4[4 * q + 3] = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]) * f;
  }
  return 0;
}

int llg_topological_charge(llg_handle* h, int32_t replica, double* q) {
  if (!h) return tls_fail(LLG_ERR_BAD_DESC, "null handle");
  if (replica < 0 || replica >= (int32_t)h->reps.size() || !q)
    return h->fail(LLG_ERR_BAD_DESC, "replica %d out of range", replica);
  if (h->nb != 1 || h->reps[replica].L[2] != 1)
    return h->fail(LLG_ERR_UNSUPPORTED, "topological charge needs a one-site monolayer");
  cudaSetDevice(h->device);
  const int sb = state_buffer(h);
  int rc = topological_charge(h->P, h->state[sb].p, h->fp64, replica, (int)(h->d_partials.n / (4 + kMaxTerms)),
                              h->d_partials.p, h->h_partials.data(), h->stream, q);
  if (rc) return h->cuda_fail(cudaGetLastError(), "topological charge");
  return 0;
}

int llg_set_stream(llg_handle* h, void* cuda_stream) {
  if (!h) return tls_fail(LLG_ERR_BAD_DESC, "null handle");
  cudaSetDevice(h->device);
  cudaStreamSynchronize(h->stream);
  h->stream = cuda_stream ? (cudaStream_t)cuda_stream : h->own_stream;
  return 0;
}

int64_t llg_last_launch_count(const llg_handle* h) { return h ? h->last_launches : -1; }

int64_t llg_max_steps(const llg_handle* h) { return h ? h->max_steps : -1; }

}  // extern "C"

void jams_llg::set_max_steps(llg_handle* h, int64_t max_steps) { h->max_steps = max_steps; }

extern "C" {

int llg_kernel_info(const llg_handle* h, int32_t* info) {
  if (!h || !info) return tls_fail(LLG_ERR_BAD_DESC, "null argument");
  info[0] = h->tiled ? h->family : 0;
  info[1] = h->tiled ? h->TP.TX : 0;
  info[2] = h->store_mode ? 1 : 0;
  info[3] = h->tz;
  info[4] = h->ty;
  info[5] = h->fp64 ? 1 : 0;
  info[6] = h->occupancy;
  info[7] = h->tiled ? h->rpt : 0;
  info[8] = h->fused ? 1 : 0;
  info[9] = h->tma ? 1 : 0;
  info[10] = h->store_noise ? 1 : 0;
  return 0;
}

static std::string tuning_key(const llg_handle* h) {
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, h->device);
  std::string k = std::string(prop.name) + "|fam" + std::to_string(h->family) + "|int" +
                  std::to_string(h->integrator) + "|nb" + std::to_string(h->nb) + "|nt" + std::to_string(h->nterms) + "|k4";
  for (auto& R : h->reps)
    k += "|" + std::to_string(R.L[0]) + "x" + std::to_string(R.L[1]) + "x" + std::to_string(R.L[2]) +
         (R.thermal ? "T" : "0");
  // long replica lists: keep the key short
  if (k.size() > 400) {
    uint64_t hsh = 1469598103934665603ull;
    for (char c : k) hsh = (hsh ^ (unsigned char)c) * 1099511628211ull;
    k = k.substr(0, 120) + "|h" + std::to_string(hsh);
  }
  return k;
}

static std::string tuning_cache_path() {
  const char* p = getenv("JAMS_LLG_TUNE_CACHE");
  if (p) return p;
  const char* home = getenv("HOME");
  return home ? std::string(home) + "/.cache/jams_llg_tuning.txt" : std::string();
}

static bool tuning_lookup(const std::string& key, int* tx, int* store) {
  const std::string path = tuning_cache_path();
  if (path.empty()) return false;
  FILE* f = fopen(path.c_str(), "r");
  if (!f) return false;
  char line[1024];
  bool found = false;
  while (fgets(line, sizeof line, f)) {
    char* tab = strchr(line, '\t');
    if (!tab) continue;
    *tab = 0;
    if (key == line && sscanf(tab + 1, "%d %d", tx, store) == 2) found = true;
  }
  fclose(f);
  return found;
}

static void tuning_store(const std::string& key, int tx, int store) {
  const std::string path = tuning_cache_path();
  if (path.empty()) return;
  FILE* f = fopen(path.c_str(), "a");
  if (!f) return;
  fprintf(f, "%s\t%d %d\n", key.c_str(), tx, store);
  fclose(f);
}

int llg_set_tuning(llg_handle* h, int32_t planes_per_cta, int32_t store_rhs) {
  if (!h) return tls_fail(LLG_ERR_BAD_DESC, "null handle");
  if (!h->tiled) return 0;
  if (planes_per_cta < 1) return h->fail(LLG_ERR_BAD_DESC, "planes_per_cta must be >= 1");
  // each thread computes two consecutive planes, the pair starting at an even
  // x (the pair shares one noise counter): the count is rounded up to even
  planes_per_cta += planes_per_cta & 1;
  cudaSetDevice(h->device);
  cudaError_t ce = cudaStreamSynchronize(h->stream);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "cudaStreamSynchronize");
  drop_graphs(h);
  // bit 2: two rows per thread (wide tile, no dipole term)
  const bool pair = (store_rhs & 4) != 0;
  if (pair && (!pair_rows_supported(h->family) || h->dipole || (store_rhs & 2)))
    return h->fail(LLG_ERR_BAD_DESC, "two rows per thread: only for the wide tile of sc, bcc and fcc lattices "
                                     "without a dipole term");
  // bit 3: the fused Heun step (bit 1 then picks its narrow tile; bits 0
  // and 2 do not apply)
  const bool fused = (store_rhs & 8) != 0;
  if (fused && (h->integrator != LLG_HEUN || !fused_supported(h->family) || h->dipole || (store_rhs & 5)))
    return h->fail(LLG_ERR_BAD_DESC, "fused step: Heun on sc, bcc or fcc lattices without a dipole term, "
                                     "without stored rhs or two rows per thread");
  h->fused = fused;
  h->fused_wide = (store_rhs & 2) == 0;
  h->store_mode = (store_rhs & 1) != 0 && h->integrator == LLG_HEUN;
  // bit 8: TMA plane loads (the two-pass tiled kernels)
  const bool tma = (store_rhs & 256) != 0;
  if (tma && fused) return h->fail(LLG_ERR_BAD_DESC, "TMA plane loads: the two-pass tiled kernels only");
  const int occ = (store_rhs >> 4) & 7;
  h->occupancy = occ >= 4 ? 4 : (occ == 3 ? 3 : 2);
  if (pair) h->occupancy = 2;   // two rows per thread need up to 128 registers
  h->rpt = pair ? 2 : 1;
  // bit 1: the narrow tile (half the rows, twice the CTAs)
  int wide_tz = 0, wide_ty = 0;
  tiled_geometry(h->family, &wide_tz, &wide_ty);
  const int ty = fused ? fused_rows(h->family, h->fused_wide)
                       : ((store_rhs & 2) ? narrow_tile_rows(h->family) : wide_ty);
  // bit 10: the half-width simple-cubic tile (16 cells along z, wide rows)
  const bool half = (store_rhs & 1024) != 0;
  if (half && (h->family != kFamSC || fused || tma || h->dipole || (store_rhs & 2)))
    return h->fail(LLG_ERR_BAD_DESC, "half-width tile: simple-cubic lattices without a dipole term, the wide rows, "
                                     "not with the fused step or TMA");
  const int tz = half ? 16 : wide_tz;
  const bool retile = ty != h->ty || tz != h->tz;
  h->ty = ty;
  h->tz = tz;
  if (planes_per_cta != h->TP.TX || retile) {
    h->TP.TX = planes_per_cta;
    int rc = build_tiles4(h);
    if (rc) return rc;
  }
  h->tma = false;
  if (tma) {
    const char* why = tma_unsupported(h);
    if (why) return h->fail(LLG_ERR_BAD_DESC, "TMA plane loads: %s", why);
    int rc = build_tensor_maps(h);
    if (rc) return rc;
    h->tma = true;
  }
  // bit 9: stored noise (the Heun predictor stores the thermal field for
  // the stored-rhs corrector)
  h->store_noise = false;
  if (store_rhs & 512) {
    if (!h->store_mode || fused)
      return h->fail(LLG_ERR_BAD_DESC, "stored noise: the two-pass Heun kernels in stored-rhs mode only");
    if (!h->noise.p) {
      ce = h->noise.alloc((size_t)3 * h->npad);
      if (ce != cudaSuccess) return h->cuda_fail(ce, "alloc noise planes");
      ce = clear_cold_noise(h);
      if (ce != cudaSuccess) return h->cuda_fail(ce, "clearing the noise planes");
    }
    h->store_noise = true;
  }
  return 0;
}

int llg_profile_stages(llg_handle* h, int32_t nsteps, double* ms) {
  if (!h) return tls_fail(LLG_ERR_BAD_DESC, "null handle");
  if (nsteps < 1 || !ms) return h->fail(LLG_ERR_BAD_DESC, "nsteps must be >= 1 and ms non-null");
  cudaSetDevice(h->device);
  int rc = sync_replicas(h);
  if (rc) return rc;
  if (h->pulsed) {
    if (nsteps > h->pulse_cap) return h->fail(LLG_ERR_BAD_DESC, "profile at most %d steps", h->pulse_cap);
    rc = upload_pulse_table(h, h->iteration, nsteps);
    if (rc) return rc;
  }
  const int ns = num_stages(h);
  // per stage: start, after the dipole field evaluation, end
  std::vector<cudaEvent_t> ev((size_t)nsteps * ns * 3);
  for (auto& e : ev) {
    cudaError_t ce = cudaEventCreate(&e);
    if (ce != cudaSuccess) return h->cuda_fail(ce, "cudaEventCreate");
  }
  int cur = h->cur;
  for (int k = 0; k < nsteps; ++k) {
    for (int stg = 0; stg < ns; ++stg) {
      cudaEvent_t* e = &ev[((size_t)k * ns + stg) * 3];
      cudaEventRecord(e[0], h->stream);
      launch_stage(h, stg, (uint32_t)k, cur, e[1]);
      cudaEventRecord(e[2], h->stream);
    }
    cur = next_buffer(h, cur);
  }
  advance_step_base<<<1, 1, 0, h->stream>>>(h->d_step_base.p, (uint32_t)nsteps);
  h->cur = cur;
  h->iteration += nsteps;
  h->last_launches = (int64_t)nsteps * ns * stage_launches(h) + 1;
  cudaError_t ce = cudaStreamSynchronize(h->stream);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "profiling stages");
  for (int stg = 0; stg < 2 * ns; ++stg) ms[stg] = 0.0;
  for (int k = 0; k < nsteps; ++k)
    for (int stg = 0; stg < ns; ++stg) {
      const cudaEvent_t* e = &ev[((size_t)k * ns + stg) * 3];
      float t = 0.f;
      cudaEventElapsedTime(&t, e[1], e[2]);
      ms[stg] += t / nsteps;
      cudaEventElapsedTime(&t, e[0], e[1]);
      ms[ns + stg] += t / nsteps;
    }
  for (auto& e : ev) cudaEventDestroy(e);
  if (!h->async_err.empty()) {
    const std::string e = h->async_err;
    h->async_err.clear();
    return h->fail(LLG_ERR_CUDA, "%s", e.c_str());
  }
  return 0;
}

int llg_autotune(llg_handle* h, int32_t trial_steps, int32_t use_cache) {
  if (!h) return tls_fail(LLG_ERR_BAD_DESC, "null handle");
  if (!h->tiled) return 0;
  if (trial_steps < 1) trial_steps = 10;
  cudaSetDevice(h->device);
  int rc = sync_replicas(h);
  if (rc) return rc;
  const std::string key = tuning_key(h);
  int tx = 0, st = 0;
  if (use_cache && tuning_lookup(key, &tx, &st)) return llg_set_tuning(h, tx, st);
  // keep the state: the trials advance a copy
  const size_t bytes = (size_t)3 * h->npad * real_size(h);
  DevBuf<unsigned char> save;
  cudaError_t ce = save.alloc(bytes);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "autotune scratch");
  const int sb0 = state_buffer(h);
  ce = cudaMemcpyAsync(save.p, h->state[sb0].p, bytes, cudaMemcpyDeviceToDevice, h->stream);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "autotune save");
  const int64_t it0 = h->iteration;
  const int cur0 = h->cur;
  int maxL = 1;
  for (auto& R : h->reps) maxL = std::max(maxL, R.vL[0]);
  std::vector<std::pair<int, int>> cands;   // (planes per CTA, store flag | occupancy << 4)
  for (int t : {2, 4, 8, 16, 32, 64})
    if (t <= std::max(2, maxL))
      for (int occ : {2, 3, 4})
        for (int narrow : {0, 2}) {   // the family's wide tile, or the narrow one where it differs
          int wide_tz = 0, wide_ty = 0;
          tiled_geometry(h->family, &wide_tz, &wide_ty);
          if (narrow && narrow_tile_rows(h->family) == wide_ty) continue;
          cands.push_back({t, narrow | (occ << 4)});
          if (h->integrator == LLG_HEUN) cands.push_back({t, 1 | narrow | (occ << 4)});
          // two rows per thread: wide tile, occupancy 2
          if (!narrow && occ == 2 && pair_rows_supported(h->family) && !h->dipole) {
            cands.push_back({t, 4 | (occ << 4)});
            if (h->integrator == LLG_HEUN) cands.push_back({t, 5 | (occ << 4)});
          }
        }
  // TMA plane loads: the same tilings again (where supported: the tile
  // rows of a candidate decide the box)
  {
    const size_t n0 = cands.size();
    const int ty0 = h->ty;
    for (size_t c = 0; c < n0; ++c) {
      int wide_tz = 0, wide_ty = 0;
      tiled_geometry(h->family, &wide_tz, &wide_ty);
      h->ty = (cands[c].second & 2) ? narrow_tile_rows(h->family) : wide_ty;
      if (!tma_unsupported(h)) cands.push_back({cands[c].first, cands[c].second | 256});
    }
    h->ty = ty0;
  }
  // stored noise: the stored-rhs Heun candidates again, where some replica
  // is above 0 K (at 0 K there is no noise to store)
  if (h->integrator == LLG_HEUN && std::any_of(h->rep_T.begin(), h->rep_T.end(), [](double T) { return T > 0.0; })) {
    const size_t n0 = cands.size();
    for (size_t c = 0; c < n0; ++c)
      if (cands[c].second & 1) cands.push_back({cands[c].first, cands[c].second | 512});
  }
  // the half-width simple-cubic tile: the wide-row candidates again, without
  // TMA
  if (h->family == kFamSC && !h->dipole) {
    const size_t n0 = cands.size();
    for (size_t c = 0; c < n0; ++c)
      if (!(cands[c].second & (2 | 256))) cands.push_back({cands[c].first, cands[c].second | 1024});
  }
  // the fused Heun step: wide or narrow tile, occupancy 2 or 4 (x 256 threads)
  if (h->integrator == LLG_HEUN && fused_supported(h->family) && !h->dipole)
    for (int t : {2, 4, 8, 16, 32, 64})
      if (t <= std::max(2, maxL))
        for (int occ : {2, 4})
          for (int narrow : {0, 2}) {
            if (narrow && fused_rows(h->family, false) == fused_rows(h->family, true)) continue;
            cands.push_back({t, 8 | narrow | (occ << 4)});
          }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  int wide_tz0 = 0, wide_ty0 = 0;
  tiled_geometry(h->family, &wide_tz0, &wide_ty0);
  std::pair<int, int> choice = {h->TP.TX, h->fused ? (8 | (h->fused_wide ? 0 : 2) | (h->occupancy << 4))
                                                   : ((h->store_mode ? 1 : 0) | (h->ty != wide_ty0 ? 2 : 0) |
                                                      (h->rpt == 2 ? 4 : 0) | (h->occupancy << 4) |
                                                      (h->tma ? 256 : 0) | (h->store_noise ? 512 : 0) |
                                                      (h->tz == 16 ? 1024 : 0))};
  // each trial runs as llg_step runs steps: one CUDA graph of trial_steps
  // steps (captured and run once untimed, then timed)
  const int spg0 = h->steps_per_graph;
  trial_steps += trial_steps & 1;
  h->steps_per_graph = trial_steps;
  for (auto& c : cands) {
    rc = llg_set_tuning(h, c.first, c.second);
    if (!rc) rc = llg_step(h, trial_steps);
    if (rc) break;
    cudaEventRecord(e0, h->stream);
    rc = llg_step(h, trial_steps);
    cudaEventRecord(e1, h->stream);
    if (rc) break;
    ce = cudaEventSynchronize(e1);
    if (ce != cudaSuccess) {
      rc = h->cuda_fail(ce, "autotune trial");
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) {
      best = ms;
      choice = c;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  h->steps_per_graph = spg0;
  if (rc) return rc;
  // restore state, buffer parity and the noise counter
  h->cur = cur0;
  rc = llg_set_tuning(h, choice.first, choice.second);
  if (rc) return rc;
  ce = cudaMemcpyAsync(h->state[state_buffer(h)].p, save.p, bytes, cudaMemcpyDeviceToDevice, h->stream);
  if (ce != cudaSuccess) return h->cuda_fail(ce, "autotune restore");
  rc = llg_set_iteration(h, it0);
  if (rc) return rc;
  tuning_store(key, choice.first, choice.second);
  return 0;
}

}  // extern "C"

// ------------------------------------------------- spin files, checkpoints --

namespace {

constexpr char kCkptMagic[8] = {'J', 'L', 'L', 'G', 'C', 'K', 'P', 'T'};
constexpr uint32_t kCkptVersion = 2;   // 2: the fingerprint holds the model hash

struct Bytes {
  std::vector<uint8_t> b;
  void u32(uint64_t v) { for (int i = 0; i < 4; ++i) b.push_back((uint8_t)(v >> (8 * i))); }
  void u64(uint64_t v) { for (int i = 0; i < 8; ++i) b.push_back((uint8_t)(v >> (8 * i))); }
  void f64(double x) {
    uint64_t u;
    std::memcpy(&u, &x, 8);
    u64(u);
  }
};

struct Reader {
  const std::vector<uint8_t>& b;
  size_t p = 0;
  bool ok = true;
  uint64_t un(int n) {
    if (p + n > b.size()) {
      ok = false;
      return 0;
    }
    uint64_t v = 0;
    for (int i = 0; i < n; ++i) v |= (uint64_t)b[p + i] << (8 * i);
    p += n;
    return v;
  }
  double f64() {
    const uint64_t u = un(8);
    double x;
    std::memcpy(&x, &u, 8);
    return x;
  }
};

// FNV-1a, 64 bit
uint64_t fnv1a(const uint8_t* p, size_t n) {
  uint64_t h = 1469598103934665603ull;
  for (size_t i = 0; i < n; ++i) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}

// header fields that must match between the writing and the loading solver
void ckpt_fingerprint(const llg_handle* h, Bytes& o) {
  o.u64(h->model_hash);
  o.u32(h->fp64 ? LLG_FP64 : LLG_FP32C);
  o.u32(h->integrator);
  o.u32(h->nb);
  o.u32(h->reps.size());
  o.f64(h->dt);
  o.u64(h->P.seed);
  for (const ReplicaDev& R : h->reps) {
    o.u32(R.L[0]);
    o.u32(R.L[1]);
    o.u32(R.L[2]);
    o.u32(R.n);
  }
}

}  // namespace

extern "C" {

int llg_write_array_file(const char* path, const char* dataset, const double* data, int64_t rows, int64_t cols) {
  if (!path || !data || rows < 0 || cols < 1) return tls_fail(LLG_ERR_BAD_DESC, "bad array file arguments");
  std::string err;
  std::vector<llgio::Dataset> sets{{llgio::dataset_name(dataset ? dataset : "data"), data, rows, cols}};
  if (llgio::write_array(path, sets, err)) return tls_fail(LLG_ERR_IO, "%s", err.c_str());
  return 0;
}

int llg_read_array_file(const char* path, const char* dataset, double* data, int64_t capacity, int64_t* rows,
                        int64_t* cols) {
  if (!path || !rows || !cols) return tls_fail(LLG_ERR_BAD_DESC, "bad array file arguments");
  std::string err;
  std::vector<double> v;
  int64_t r = 0, c = 0;
  if (llgio::read_array(path, dataset ? dataset : "data", v, r, c, err)) return tls_fail(LLG_ERR_IO, "%s", err.c_str());
  *rows = r;
  *cols = c;
  if (!data) return 0;
  if ((int64_t)v.size() > capacity)
    return tls_fail(LLG_ERR_BAD_DESC, "%s holds %lld values, the buffer %lld", path, (long long)v.size(),
                    (long long)capacity);
  std::memcpy(data, v.data(), v.size() * sizeof(double));
  return 0;
}

int llg_write_spins(llg_handle* h, int32_t replica, const char* path) {
  if (!h) return tls_fail(LLG_ERR_BAD_DESC, "null handle");
  if (replica < 0 || replica >= (int32_t)h->reps.size() || !path)
    return h->fail(LLG_ERR_BAD_DESC, "replica %d out of range", replica);
  const int64_t n = h->reps[replica].n;
  std::vector<double> s((size_t)n * 3);
  int rc = llg_get_state(h, replica, s.data());
  if (rc) return rc;
  std::string err;
  std::vector<llgio::Dataset> sets{{"spins", s.data(), n, 3}};
  if (llgio::write_array(path, sets, err)) return h->fail(LLG_ERR_IO, "%s", err.c_str());
  return 0;
}

int llg_read_spins(llg_handle* h, int32_t replica, const char* path) {
  if (!h) return tls_fail(LLG_ERR_BAD_DESC, "null handle");
  if (replica < 0 || replica >= (int32_t)h->reps.size() || !path)
    return h->fail(LLG_ERR_BAD_DESC, "replica %d out of range", replica);
  const int64_t n = h->reps[replica].n;
  std::string err;
  std::vector<double> v;
  int64_t r = 0, c = 0;
  if (llgio::read_array(path, "spins", v, r, c, err)) return h->fail(LLG_ERR_IO, "%s", err.c_str());
  if ((int64_t)v.size() != 3 * n)
    return h->fail(LLG_ERR_IO, "loading array from file: '%s' expected size: %lld actual size: %lld", path,
                   (long long)(3 * n), (long long)v.size());
  return llg_set_state(h, replica, v.data());
}

int llg_save_checkpoint(llg_handle* h, const char* path) {
  if (!h) return tls_fail(LLG_ERR_BAD_DESC, "null handle");
  if (!path) return h->fail(LLG_ERR_BAD_DESC, "null path");
  Bytes o;
  o.b.insert(o.b.end(), kCkptMagic, kCkptMagic + 8);
  o.u32(kCkptVersion);
  ckpt_fingerprint(h, o);
  o.u64((uint64_t)h->iteration);
  for (size_t r = 0; r < h->reps.size(); ++r) {
    o.f64(h->rep_T[r]);
    for (int a = 0; a < 3; ++a) o.f64(h->reps[r].B[a]);
  }
  std::vector<double> s;
  for (size_t r = 0; r < h->reps.size(); ++r) {
    s.resize((size_t)h->reps[r].n * 3);
    int rc = llg_get_state(h, (int32_t)r, s.data());
    if (rc) return rc;
    for (double x : s) o.f64(x);
  }
  o.u64(fnv1a(o.b.data(), o.b.size()));
  const std::string tmp = std::string(path) + ".tmp";
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) return h->fail(LLG_ERR_IO, "cannot open %s for writing", tmp.c_str());
  bool ok = std::fwrite(o.b.data(), 1, o.b.size(), f) == o.b.size();
  ok = std::fflush(f) == 0 && ok;
  ok = std::fclose(f) == 0 && ok;
  if (!ok || std::rename(tmp.c_str(), path) != 0) {
    std::remove(tmp.c_str());
    return h->fail(LLG_ERR_IO, "writing checkpoint %s failed", path);
  }
  return 0;
}

int llg_load_checkpoint(llg_handle* h, const char* path) {
  if (!h) return tls_fail(LLG_ERR_BAD_DESC, "null handle");
  if (!path) return h->fail(LLG_ERR_BAD_DESC, "null path");
  std::vector<uint8_t> b;
  {
    FILE* f = std::fopen(path, "rb");
    if (!f) return h->fail(LLG_ERR_IO, "cannot open checkpoint %s", path);
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    b.resize(n > 0 ? (size_t)n : 0);
    const bool ok = n > 0 && std::fread(b.data(), 1, b.size(), f) == b.size();
    std::fclose(f);
    if (!ok) return h->fail(LLG_ERR_IO, "cannot read checkpoint %s", path);
  }
  if (b.size() < 8 + 4 + 8 || std::memcmp(b.data(), kCkptMagic, 8) != 0)
    return h->fail(LLG_ERR_IO, "%s is not a checkpoint of this library", path);
  {
    Reader t{b, b.size() - 8};
    if (t.un(8) != fnv1a(b.data(), b.size() - 8)) return h->fail(LLG_ERR_IO, "checkpoint %s: checksum mismatch", path);
  }
  Reader rd{b, 8};
  if (rd.un(4) != kCkptVersion) return h->fail(LLG_ERR_IO, "checkpoint %s: unknown format version", path);
  Bytes fp;
  ckpt_fingerprint(h, fp);
  if (rd.p + fp.b.size() > b.size() || std::memcmp(&b[rd.p], fp.b.data(), fp.b.size()) != 0)
    return h->fail(LLG_ERR_BAD_DESC,
                   "checkpoint %s was written by a different model (Hamiltonian terms or their parameters, "
                   "materials, replicas, sizes, basis, precision, integrator, dt or seed differ)",
                   path);
  rd.p += fp.b.size();
  const int64_t iteration = (int64_t)rd.un(8);
  std::vector<double> T(h->reps.size()), B(3 * h->reps.size());
  for (size_t r = 0; r < h->reps.size(); ++r) {
    T[r] = rd.f64();
    for (int a = 0; a < 3; ++a) B[3 * r + a] = rd.f64();
  }
  size_t need = 0;
  for (const ReplicaDev& R : h->reps) need += (size_t)R.n * 3 * 8;
  if (!rd.ok || rd.p + need + 8 != b.size()) return h->fail(LLG_ERR_IO, "checkpoint %s: truncated", path);
  // everything is read and checked before anything is applied
  for (size_t r = 0; r < h->reps.size(); ++r) {
    if (!(T[r] >= 0.0) || !std::isfinite(T[r]))
      return h->fail(LLG_ERR_IO, "checkpoint %s: replica %zu has temperature %g", path, r, T[r]);
    for (int a = 0; a < 3; ++a)
      if (!std::isfinite(B[3 * r + a])) return h->fail(LLG_ERR_IO, "checkpoint %s: replica %zu field", path, r);
  }
  if (iteration < 0) return h->fail(LLG_ERR_IO, "checkpoint %s: negative iteration", path);
  std::vector<std::vector<double>> states(h->reps.size());
  for (size_t r = 0; r < h->reps.size(); ++r) {
    states[r].resize((size_t)h->reps[r].n * 3);
    for (double& x : states[r]) x = rd.f64();
    for (double x : states[r])
      if (!std::isfinite(x)) return h->fail(LLG_ERR_IO, "checkpoint %s: replica %zu holds a non-finite spin", path, r);
  }
  for (size_t r = 0; r < h->reps.size(); ++r) {
    int rc = llg_set_state(h, (int32_t)r, states[r].data());
    if (rc) return rc;
  }
  for (size_t r = 0; r < h->reps.size(); ++r) {
    int rc = llg_set_temperature(h, (int32_t)r, T[r]);
    if (!rc) rc = llg_set_field(h, (int32_t)r, &B[3 * r]);
    if (rc) return rc;
  }
  return llg_set_iteration(h, iteration);
}

}  // extern "C"
