// Harness that runs the REFERENCE's own CPU LLG path, compiled from the
// reference sources by oracle/Makefile.ref into oracle/_ref/libjams_ref.so.
// TEST INFRASTRUCTURE ONLY, built in the development container (the
// reference sources are not shipped): it pins the C restatement in
// llg_oracle.c and generates the golden vectors in tests/golden/.
//
// Compiled from the reference (unmodified): src/jams/solvers/cpu_llg_heun.cc,
// src/jams/core/solver.cc, src/jams/hamiltonian/sparse_interaction.cc,
// src/jams/hamiltonian/uniaxial_anisotropy.cc,
// src/jams/hamiltonian/cubic_anisotropy.cc,
// src/jams/hamiltonian/applied_field.cc, src/jams/hamiltonian/zeeman.cc,
// src/jams/hamiltonian/dipole_bruteforce.cc, src/jams/lattice/minimum_image.cc,
// src/jams/containers/cell.cc, src/jams/core/physics.cc,
// src/jams/core/base.cc, src/jams/common.cc, and the header-only CSR builder
// and Xcsrmv_general (src/jams/containers/sparse_matrix*.h,
// src/jams/interface/sparse_blas.h).
//
// Supplied here because their own translation units pull in spglib, HDF5,
// FFTW or the whole plugin factory set:
//   - globals storage (src/jams/core/globals.h with GLOBALORIGIN),
//   - the handful of Lattice accessors the anisotropy and dipole terms call
//     (lattice parameter, supercell, cartesian site positions, and the
//     supercell inradius of jams::maximum_interaction_length,
//     src/jams/core/lattice.cc:1155-1200, restated),
//   - LAPACK's dgetrf_/dgetri_ for the Mat3 inverse (mat3.h:232-257),
//   - the Hamiltonian base constructor (energy-unit lookup and name only,
//     src/jams/core/hamiltonian.cc:116-165),
//   - an exchange term that inserts 3x3 blocks for the neighbour list of an
//     interaction template (loop of src/jams/core/interactions.cc:350-396)
//     through the reference's own SparseInteractionHamiltonian,
//   - cblas_daxpy as y[i] += a * x[i].
#define GLOBALORIGIN
#include <jams/core/globals.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include <jams/core/hamiltonian.h>
#include <jams/core/lattice.h>
#include <jams/core/units.h>
#include <jams/hamiltonian/applied_field.h>
#include <jams/containers/cell.h>
#include <jams/hamiltonian/cubic_anisotropy.h>
#include <jams/hamiltonian/dipole_bruteforce.h>
#include <jams/hamiltonian/sparse_interaction.h>
#include <jams/hamiltonian/uniaxial_anisotropy.h>
#include <jams/hamiltonian/zeeman.h>
#include <jams/physics/empty.h>
#include <jams/solvers/cpu_llg_heun.h>

#include "llg_oracle.h"

using libconfig::Setting;

extern "C" void cblas_daxpy(int n, double a, const double* x, int incx, double* y, int incy) {
  for (int i = 0; i < n; ++i) y[i * incy] += a * x[i * incx];
}

// LU factorisation with partial pivoting and the inverse from it, column-major
// (the LAPACK routines the reference's Mat3 inverse calls)
extern "C" void dgetrf_(const int* m, const int* n, double* a, const int* lda, int* ipiv, int* info) {
  const int M = *m, N = *n, LD = *lda;
  auto A = [&](int i, int j) -> double& { return a[i + j * LD]; };
  *info = 0;
  for (int k = 0; k < std::min(M, N); ++k) {
    int p = k;
    for (int i = k + 1; i < M; ++i)
      if (std::fabs(A(i, k)) > std::fabs(A(p, k))) p = i;
    ipiv[k] = p + 1;
    if (A(p, k) == 0.0) {
      if (!*info) *info = k + 1;
      continue;
    }
    if (p != k)
      for (int j = 0; j < N; ++j) std::swap(A(k, j), A(p, j));
    for (int i = k + 1; i < M; ++i) A(i, k) /= A(k, k);
    for (int j = k + 1; j < N; ++j)
      for (int i = k + 1; i < M; ++i) A(i, j) -= A(i, k) * A(k, j);
  }
}

extern "C" void dgetri_(const int* n, double* a, const int* lda, const int* ipiv, double* work, const int* lwork,
                        int* info) {
  const int N = *n, LD = *lda;
  *info = 0;
  if (*lwork == -1) {
    work[0] = N;
    return;
  }
  std::vector<double> inv((size_t)N * N);
  for (int c = 0; c < N; ++c) {
    std::vector<double> x(N, 0.0);
    x[c] = 1.0;
    for (int k = 0; k < N; ++k)
      if (ipiv[k] - 1 != k) std::swap(x[k], x[ipiv[k] - 1]);
    for (int i = 0; i < N; ++i)
      for (int k = 0; k < i; ++k) x[i] -= a[i + k * LD] * x[k];
    for (int i = N - 1; i >= 0; --i) {
      for (int k = i + 1; k < N; ++k) x[i] -= a[i + k * LD] * x[k];
      x[i] /= a[i + i * LD];
    }
    for (int i = 0; i < N; ++i) inv[i + (size_t)c * N] = x[i];
  }
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < N; ++i) a[i + j * LD] = inv[i + (size_t)j * N];
}

namespace {
struct HarnessLattice {
  int L[3] = {1, 1, 1};
  int periodic[3] = {1, 1, 1};
  int nb = 1;
  double a = 3e-10;                                  // lattice parameter (m)
  double A[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};         // lattice vectors (rows)
  std::vector<double> frac;                          // basis positions, 3 nb
  Cell supercell;
  std::vector<Vec3> pos;                             // cartesian site positions
} g_lat;

void build_geometry() {
  Mat3 m;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) m[r][c] = g_lat.L[c] * g_lat.A[3 * c + r];
  g_lat.supercell = Cell(m, Vec3b{g_lat.periodic[0] != 0, g_lat.periodic[1] != 0, g_lat.periodic[2] != 0});
  g_lat.pos.clear();
  for (int i = 0; i < g_lat.L[0]; ++i)
    for (int j = 0; j < g_lat.L[1]; ++j)
      for (int k = 0; k < g_lat.L[2]; ++k)
        for (int b = 0; b < g_lat.nb; ++b) {
          const double f[3] = {i + (g_lat.frac.empty() ? 0.0 : g_lat.frac[3 * b]),
                               j + (g_lat.frac.empty() ? 0.0 : g_lat.frac[3 * b + 1]),
                               k + (g_lat.frac.empty() ? 0.0 : g_lat.frac[3 * b + 2])};
          Vec3 r;
          for (int c = 0; c < 3; ++c) r[c] = f[0] * g_lat.A[c] + f[1] * g_lat.A[3 + c] + f[2] * g_lat.A[6 + c];
          g_lat.pos.push_back(r);
        }
}

std::string g_err;

std::string material_name_of_basis(int b) { return "M" + std::to_string(b); }
}  // namespace

// --- Lattice accessors used by the anisotropy terms (each basis site is its
// own material "M<b>") ---
Lattice::~Lattice() {}
double Lattice::parameter() const { return g_lat.a; }
const Cell& Lattice::get_supercell() { return g_lat.supercell; }
double Lattice::max_interaction_radius() const {
  const Vec3 v[3] = {g_lat.supercell.a1(), g_lat.supercell.a2(), g_lat.supercell.a3()};
  auto cross_norm = [](const Vec3& x, const Vec3& y) { return norm(cross(x, y)); };
  const int np = (g_lat.periodic[0] != 0) + (g_lat.periodic[1] != 0) + (g_lat.periodic[2] != 0);
  if (np == 3) {
    const double vol = std::fabs(dot(v[0], cross(v[1], v[2])));
    return 0.5 * std::min(vol / cross_norm(v[1], v[2]), std::min(vol / cross_norm(v[2], v[0]), vol / cross_norm(v[0], v[1])));
  }
  if (np == 2) {
    const Vec3& x = g_lat.periodic[0] ? v[0] : v[1];
    const Vec3& y = g_lat.periodic[2] ? v[2] : v[1];
    const double area = cross_norm(x, y);
    return 0.5 * std::min(area / norm(x), area / norm(y));
  }
  if (np == 1) return 0.5 * norm(g_lat.periodic[0] ? v[0] : (g_lat.periodic[1] ? v[1] : v[2]));
  return norm(v[0] + v[1] + v[2]);
}
int Lattice::num_basis_sites() const { return g_lat.nb; }
int Lattice::num_materials() const { return g_lat.nb; }
int Lattice::material_index(const std::string& name) const {
  for (int b = 0; b < g_lat.nb; ++b)
    if (material_name_of_basis(b) == name) return b;
  throw std::runtime_error("no material " + name);
}
bool Lattice::material_exists(const std::string& name) const {
  for (int b = 0; b < g_lat.nb; ++b)
    if (material_name_of_basis(b) == name) return true;
  return false;
}
int Lattice::lattice_site_material_id(int i) const { return i % g_lat.nb; }
unsigned Lattice::lattice_site_basis_index(int i) const { return (unsigned)(i % g_lat.nb); }
// reached only by Physics' "initial_state" option, which the harness never sets
const Vec3& Lattice::lattice_site_position_cart(int i) const { return g_lat.pos.at((size_t)i); }
Vec3 Lattice::displacement(const Vec3&, const Vec3&) const { throw std::runtime_error("not available"); }

// --- Hamiltonian base constructor: unit lookup and name ---
Hamiltonian::Hamiltonian(const libconfig::Setting& settings, const unsigned int size)
    : Base(settings), energy_(size), field_(size, 3) {
  input_energy_unit_name_ = jams::config_optional<std::string>(settings, "energy_units", jams::defaults::energy_unit_name);
  input_energy_unit_conversion_ = jams::internal_energy_unit_conversion.at(input_energy_unit_name_);
  input_distance_unit_conversion_ = 1.0;
  set_name(settings["module"].c_str());
}

namespace {

class TemplateExchange : public SparseInteractionHamiltonian {
 public:
  TemplateExchange(const Setting& settings, unsigned size, const orc_term& t)
      : SparseInteractionHamiltonian(settings, size) {
    const int L0 = g_lat.L[0], L1 = g_lat.L[1], L2 = g_lat.L[2];
    std::set<std::pair<int, int>> seen;
    auto site = [&](int i, int j, int k, int m) { return ((i * L1 + j) * L2 + k) * g_lat.nb + m; };
    for (int i = 0; i < L0; ++i)
      for (int j = 0; j < L1; ++j)
        for (int k = 0; k < L2; ++k)
          for (int e = 0; e < t.n_int; ++e) {
            const int m = t.bi[e];
            int d[3] = {i + t.T[3 * e], j + t.T[3 * e + 1], k + t.T[3 * e + 2]};
            bool outside = false;
            for (int l = 0; l < 3; ++l) {
              if (!g_lat.periodic[l] && (d[l] < 0 || d[l] >= g_lat.L[l])) outside = true;
              d[l] = (d[l] + g_lat.L[l]) % g_lat.L[l];
            }
            if (outside) continue;
            const int local = site(i, j, k, m);
            const int nbr = site(d[0], d[1], d[2], t.bj[e]);
            if (!seen.insert({local, nbr}).second) throw std::runtime_error("Multiple interactions");
            Mat3 J;
            for (int a = 0; a < 3; ++a)
              for (int b = 0; b < 3; ++b) J[a][b] = t.J[9 * e + 3 * a + b];
            // ExchangeHamiltonian ctor (exchange.cc:162-169): value times the
            // energy-unit factor (meV here), kept when max|J| > 0
            Mat3 Jij = 1.0 * input_energy_unit_conversion_ * J;
            if (max_abs(Jij) > 0.0) insert_interaction_tensor(local, nbr, Jij);
          }
    finalize(jams::SparseMatrixSymmetryCheck::None);
  }
};

Setting group() { return Setting(Setting::TypeGroup); }
Setting list() { return Setting(Setting::TypeList); }
Setting array() { return Setting(Setting::TypeArray); }
Setting vec3(const double* v) {
  Setting a = array();
  for (int i = 0; i < 3; ++i) a.add(Setting::number(v[i]));
  return a;
}

// The reference's CPU Heun solver with access to the solver clock (Solver's
// protected iteration_ and time_), so that the RK4 driver below can set the
// stage times as CudaRK4BaseSolver::run does while reusing the solver's
// registered Hamiltonians and Solver::compute_fields.
class HarnessSolver : public HeunLLGSolver {
 public:
  using HeunLLGSolver::HeunLLGSolver;
  void set_clock(int iteration, double time) {
    iteration_ = iteration;
    time_ = time;
  }
};

HarnessSolver* g_solver = nullptr;
std::vector<Setting> g_keep;

}  // namespace

// the reference's RK4 kernels built for the host (ref_rk4_kernels.cc)
void ref_host_llg_rk4_kernel(const double* s, double* k, const double* h, const double* noise, const double* gyro,
                             const double* mus, const double* alpha, unsigned n);
void ref_host_rk4_combine_normalise(double* s, const double* s_old, const double* k1, const double* k2,
                                    const double* k3, const double* k4, double dt, unsigned n);

extern "C" {

__attribute__((visibility("default"))) const char* ref_last_error() { return g_err.c_str(); }

__attribute__((visibility("default"))) void ref_destroy() {
  delete g_solver;
  g_solver = nullptr;
  delete globals::lattice;
  globals::lattice = nullptr;
}

// t_step_seconds: the solver's t_step setting (the reference divides by 1e-12)
__attribute__((visibility("default"))) int ref_create(const orc_model* m, double t_step_seconds) {
  try {
    ref_destroy();
    g_lat.L[0] = m->L[0];
    g_lat.L[1] = m->L[1];
    g_lat.L[2] = m->L[2];
    g_lat.nb = m->nb;
    for (int l = 0; l < 3; ++l) g_lat.periodic[l] = m->periodic[l];
    g_lat.a = 3e-10;
    for (int c = 0; c < 9; ++c) g_lat.A[c] = c % 4 == 0 ? 1.0 : 0.0;
    g_lat.frac.assign((size_t)3 * m->nb, 0.0);
    for (int t = 0; t < m->n_terms; ++t)
      if (m->terms[t].kind == ORC_TERM_DIPOLE) {
        g_lat.a = m->terms[t].lattice_parameter;
        for (int c = 0; c < 9; ++c) g_lat.A[c] = m->terms[t].lattice_vectors[c];
        for (int c = 0; c < 3 * m->nb; ++c) g_lat.frac[c] = m->terms[t].positions[c];
      }
    build_geometry();
    globals::lattice = new Lattice();
    const int n = m->L[0] * m->L[1] * m->L[2] * m->nb;
    globals::num_spins = n;
    globals::num_spins3 = 3 * n;
    globals::s.resize(n, 3);
    globals::h.resize(n, 3);
    globals::ds_dt.resize(n, 3);
    globals::alpha.resize(n);
    globals::mus.resize(n);
    globals::gyro.resize(n);
    for (int i = 0; i < n; ++i) {
      globals::mus(i) = m->mus[i % m->nb];
      globals::gyro(i) = m->gyro[i % m->nb];
      globals::alpha(i) = m->alpha[i % m->nb];
      globals::s(i, 0) = 0.0;
      globals::s(i, 1) = 0.0;
      globals::s(i, 2) = 1.0;
    }

    Setting solver_settings = group();
    solver_settings.add("module", Setting::string("llg-heun-cpu"));
    solver_settings.add("t_step", Setting::number(t_step_seconds));
    solver_settings.add("t_max", Setting::number(1.0));
    solver_settings.add("gilbert_prefactor", Setting::boolean(m->gilbert_prefactor != 0));
    g_solver = new HarnessSolver(solver_settings);

    Setting physics_settings = group();
    physics_settings.add("module", Setting::string("empty"));
    physics_settings.add("temperature", Setting::number(m->temperature));
    g_solver->register_physics_module(new EmptyPhysics(physics_settings));

    for (int t = 0; t < m->n_terms; ++t) {
      const orc_term& tm = m->terms[t];
      Setting hs = group();
      hs.add("energy_units", Setting::string("meV"));
      if (tm.kind == ORC_TERM_EXCHANGE) {
        hs.add("module", Setting::string("exchange"));
        g_solver->register_hamiltonian(new TemplateExchange(hs, n, tm));
      } else if (tm.kind == ORC_TERM_UNIAXIAL) {
        hs.add("module", Setting::string("uniaxial"));
        hs.add("order", Setting::string(tm.order == 2 ? "K1" : tm.order == 4 ? "K2" : "K3"));
        Setting& an = hs.add("anisotropies", list());
        for (int b = 0; b < m->nb; ++b) {
          Setting e = list();
          e.add(Setting::string(material_name_of_basis(b)));
          e.add(vec3(tm.axis + 3 * b));
          e.add(Setting::number(tm.K[b]));
          an.add(e);
        }
        g_solver->register_hamiltonian(new UniaxialAnisotropyHamiltonian(hs, n));
      } else if (tm.kind == ORC_TERM_CUBIC) {
        hs.add("module", Setting::string("cubic"));
        const char* key = tm.order == 1 ? "K1" : "K2";
        Setting& kl = hs.add(key, list());
        for (int b = 0; b < m->nb; ++b) {
          Setting e = list();
          e.add(Setting::number(tm.K[b]));
          e.add(vec3(tm.axis + 9 * b));
          e.add(vec3(tm.axis + 9 * b + 3));
          e.add(vec3(tm.axis + 9 * b + 6));
          kl.add(e);
        }
        g_solver->register_hamiltonian(new CubicAnisotropyHamiltonian(hs, n));
      } else if (tm.kind == ORC_TERM_APPLIED_FIELD) {
        hs.add("module", Setting::string("applied-field"));
        hs.add("field", vec3(tm.B));
        if (tm.pulse != ORC_PULSE_STATIC) {
          // the config's units: seconds and hertz (applied_field.cc:36-38,64-67)
          hs.add("type", Setting::string(tm.pulse == ORC_PULSE_SINC ? "sinc" : "sinc-cos"));
          hs.add("time_center", Setting::number(tm.time_center * 1e-12));
          hs.add("freq_bandwidth", Setting::number(tm.freq_bandwidth * 1e12));
          if (tm.pulse == ORC_PULSE_SINC_COS) hs.add("freq_center", Setting::number(tm.freq_center * 1e12));
        }
        g_solver->register_hamiltonian(new AppliedFieldHamiltonian(hs, n));
      } else if (tm.kind == ORC_TERM_ZEEMAN) {
        // per material (one per basis site): dc field, ac field and frequency
        hs.add("module", Setting::string("zeeman"));
        Setting& dc = hs.add("dc_local_field", list());
        for (int b = 0; b < m->nb; ++b) dc.add(vec3(tm.dc_field + 3 * b));
        if (tm.ac_field) {
          Setting& ac = hs.add("ac_local_field", list());
          Setting& fr = hs.add("ac_local_frequency", list());
          for (int b = 0; b < m->nb; ++b) {
            ac.add(vec3(tm.ac_field + 3 * b));
            fr.add(Setting::number(tm.ac_frequency[b]));
          }
        }
        g_solver->register_hamiltonian(new ZeemanHamiltonian(hs, n));
      } else if (tm.kind == ORC_TERM_DIPOLE) {
        hs.add("module", Setting::string("dipole-bruteforce"));
        hs.add("r_cutoff", Setting::number(tm.r_cutoff));
        g_solver->register_hamiltonian(new DipoleBruteforceHamiltonian(hs, n));
      } else {
        throw std::runtime_error("unknown term kind");
      }
    }
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

__attribute__((visibility("default"))) int ref_run(double* spins, int nsteps) {
  if (!g_solver) return -1;
  const int n = globals::num_spins;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < 3; ++j) globals::s(i, j) = spins[3 * i + j];
  for (int k = 0; k < nsteps; ++k) g_solver->run();
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < 3; ++j) spins[3 * i + j] = globals::s(i, j);
  return 0;
}

// Seeds the reference's global generator (jams::instance().random_generator(),
// pcg32), from which each HeunLLGSolver draws the seed of its own pcg32_k1024
// noise generator at construction (src/jams/solvers/cpu_llg_heun.h:35): a
// ref_create after ref_seed gives a reproducible thermal trajectory.
__attribute__((visibility("default"))) void ref_seed(uint64_t seed) { jams::instance().random_generator().seed(seed); }

// nsteps of CudaRK4BaseSolver::run (src/jams/solvers/cuda_rk4_base.cu:50-108)
// with the CUDALLGRK4Solver kernels (cuda_llg_rk4.cu:16-32), at T = 0, on the
// host: s_old = s; k1 from the fields at t0; s = s_old + dt/2 k1 at t0 + dt/2
// (cublasDcopy then cublasDaxpy, written here as a k + s with two roundings,
// as the oracle and the GPU FP64 form compute it; the library may fuse the
// multiply-add); k2;
// s = s_old + dt/2 k2; k3 at t0 + dt/2; s = s_old + dt k3; k4 at t0 + dt;
// then the combination and the normalisation of post_step (one kernel of the
// reference that evaluates both, see ref_rk4_kernels.cc).  The fields come
// from the reference's CPU Hamiltonians through Solver::compute_fields (the
// reference's GPU path sums the same terms with cuSPARSE and cuBLAS).  The
// derivative, combination and normalisation are the reference's own kernels
// (ref_rk4_kernels.cc).  The iteration and time advance as the solver's do.
__attribute__((visibility("default"))) int ref_rk4_run(double* spins, int nsteps) {
  if (!g_solver) return -1;
  try {
    if (g_solver->physics()->temperature() > 0.0) throw std::runtime_error("the RK4 driver runs at T = 0 only");
    const int n = globals::num_spins, n3 = 3 * n;
    std::vector<double> s_old(n3), k[4], zero(n3, 0.0);
    for (auto& v : k) v.assign(n3, 0.0);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < 3; ++j) globals::s(i, j) = spins[3 * i + j];
    const double dt = g_solver->time_step();
    for (int step = 0; step < nsteps; ++step) {
      const int it = g_solver->iteration();
      const double t0 = g_solver->time();
      for (int q = 0; q < n3; ++q) s_old[q] = globals::s.data()[q];
      const double stage_dt[3] = {0.5 * dt, 0.5 * dt, dt};
      for (int st = 0; st < 4; ++st) {
        g_solver->compute_fields();
        ref_host_llg_rk4_kernel(globals::s.data(), k[st].data(), globals::h.data(), zero.data(), globals::gyro.data(),
                                globals::mus.data(), globals::alpha.data(), (unsigned)n);
        if (st == 3) break;
        g_solver->set_clock(it, t0 + stage_dt[st]);
        double* s = globals::s.data();
        for (int q = 0; q < n3; ++q) s[q] = s_old[q];
        for (int q = 0; q < n3; ++q) s[q] = stage_dt[st] * k[st][q] + s[q];
      }
      ref_host_rk4_combine_normalise(globals::s.data(), s_old.data(), k[0].data(), k[1].data(), k[2].data(),
                                     k[3].data(), dt, (unsigned)n);
      g_solver->set_clock(it + 1, (it + 1) * dt);
    }
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < 3; ++j) spins[3 * i + j] = globals::s(i, j);
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

__attribute__((visibility("default"))) int ref_fields(const double* spins, double* h) {
  if (!g_solver) return -1;
  const int n = globals::num_spins;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < 3; ++j) globals::s(i, j) = spins[3 * i + j];
  g_solver->compute_fields();
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < 3; ++j) h[3 * i + j] = globals::h(i, j);
  return 0;
}

// one term's field_ after its calculate_fields at the solver time, as a
// Hamiltonian plugin leaves it (src/jams/core/hamiltonian.h:15-78)
__attribute__((visibility("default"))) int ref_term_fields(const double* spins, int term, double* h) {
  if (!g_solver || term < 0 || term >= (int)g_solver->hamiltonians().size()) return -1;
  const int n = globals::num_spins;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < 3; ++j) globals::s(i, j) = spins[3 * i + j];
  auto& hh = g_solver->hamiltonians()[term];
  hh->calculate_fields(g_solver->time());
  const double* f = hh->ptr_field();
  for (int q = 0; q < 3 * n; ++q) h[q] = f[q];
  return 0;
}

__attribute__((visibility("default"))) int ref_energies(const double* spins, double* e) {
  if (!g_solver) return -1;
  const int n = globals::num_spins;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < 3; ++j) globals::s(i, j) = spins[3 * i + j];
  int t = 0;
  // at the solver time, as the energy monitor (src/jams/monitors/energy.cc:28)
  for (auto& hh : g_solver->hamiltonians()) e[t++] = hh->calculate_total_energy(g_solver->time());
  return 0;
}

}  // extern "C"
