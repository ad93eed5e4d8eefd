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
// src/jams/hamiltonian/applied_field.cc, src/jams/core/physics.cc,
// src/jams/core/base.cc, src/jams/common.cc, and the header-only CSR builder
// and Xcsrmv_general (src/jams/containers/sparse_matrix*.h,
// src/jams/interface/sparse_blas.h).
//
// Supplied here because their own translation units pull in spglib, HDF5,
// FFTW or the whole plugin factory set:
//   - globals storage (src/jams/core/globals.h with GLOBALORIGIN),
//   - the handful of Lattice accessors the anisotropy terms call,
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
#include <jams/hamiltonian/cubic_anisotropy.h>
#include <jams/hamiltonian/sparse_interaction.h>
#include <jams/hamiltonian/uniaxial_anisotropy.h>
#include <jams/physics/empty.h>
#include <jams/solvers/cpu_llg_heun.h>

#include "llg_oracle.h"

using libconfig::Setting;

extern "C" void cblas_daxpy(int n, double a, const double* x, int incx, double* y, int incy) {
  for (int i = 0; i < n; ++i) y[i * incy] += a * x[i * incx];
}

namespace {
struct HarnessLattice {
  int L[3] = {1, 1, 1};
  int periodic[3] = {1, 1, 1};
  int nb = 1;
} g_lat;

std::string g_err;

std::string material_name_of_basis(int b) { return "M" + std::to_string(b); }
}  // namespace

// --- Lattice accessors used by the anisotropy terms (each basis site is its
// own material "M<b>") ---
Lattice::~Lattice() {}
double Lattice::parameter() const { return 3e-10; }
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
const Vec3& Lattice::lattice_site_position_cart(int) const { throw std::runtime_error("not available"); }
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

HeunLLGSolver* g_solver = nullptr;
std::vector<Setting> g_keep;

}  // namespace

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
    g_solver = new HeunLLGSolver(solver_settings);

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
        g_solver->register_hamiltonian(new AppliedFieldHamiltonian(hs, n));
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

__attribute__((visibility("default"))) int ref_energies(const double* spins, double* e) {
  if (!g_solver) return -1;
  const int n = globals::num_spins;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < 3; ++j) globals::s(i, j) = spins[3 * i + j];
  int t = 0;
  for (auto& hh : g_solver->hamiltonians()) e[t++] = hh->calculate_total_energy(0.0);
  return 0;
}

}  // extern "C"
