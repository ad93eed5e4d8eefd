// The JAMS solver module and Hamiltonian term of cuda_llg_fused_solver.h.
#include "cuda_llg_fused_solver.h"

#include <algorithm>
#include <stdexcept>

#include "jams/core/globals.h"
#include "jams/core/physics.h"
#include "jams/interface/config.h"

namespace {
std::string g_config_text;
std::string g_config_patch;

void throw_on(int rc, const llg_handle* h, const char* what) {
  if (rc != LLG_OK) throw std::runtime_error(std::string(what) + ": " + llg_last_error(h));
}
}  // namespace

void CudaFusedLLGSolver::set_config_text(const std::string& text, const std::string& patch) {
  g_config_text = text;
  g_config_patch = patch;
}

CudaFusedLLGSolver::~CudaFusedLLGSolver() {
  if (h_) llg_destroy(h_);
}

void CudaFusedLLGSolver::check(int rc) const { throw_on(rc, h_, module_.c_str()); }

void CudaFusedLLGSolver::initialize(const libconfig::Setting& settings) {
  // seconds to picoseconds and the step counts, as the reference's LLG
  // solvers read them (src/jams/solvers/cuda_llg_heun.cu:23-29)
  module_ = jams::config_required<std::string>(settings, "module");
  step_size_ = jams::config_required<double>(settings, "t_step") / 1e-12;
  const double t_max = jams::config_required<double>(settings, "t_max") / 1e-12;
  const double t_min = jams::config_optional<double>(settings, "t_min", 0.0) / 1e-12;
  max_steps_ = static_cast<int>(t_max / step_size_);
  min_steps_ = static_cast<int>(t_min / step_size_);
  const std::string precision = jams::config_optional<std::string>(settings, "precision", "fp32c");
  if (precision == "fp32c") {
    precision_ = LLG_FP32C;
  } else if (precision == "fp64") {
    precision_ = LLG_FP64;
  } else {
    throw std::runtime_error(module_ + ": precision must be \"fp32c\" or \"fp64\", not \"" + precision + "\"");
  }
  max_block_ = jams::config_optional<int>(settings, "max_block_steps", 100);
  if (max_block_ < 1) throw std::runtime_error(module_ + ": max_block_steps must be >= 1");
  if (g_config_text.empty())
    throw std::runtime_error(module_ + ": CudaFusedLLGSolver::set_config_text was not called before the solver "
                                       "was created");
  if (h_) {
    llg_destroy(h_);
    h_ = nullptr;
  }
  check(llg_create_from_config(g_config_text.c_str(), g_config_patch.c_str(), precision_, 0, &h_));
  if (llg_max_steps(h_) != max_steps_)
    throw std::runtime_error(module_ + ": the library read a different solver section (max_steps " +
                             std::to_string(llg_max_steps(h_)) + " against " + std::to_string(max_steps_) + ")");
  state_sent_ = false;
}

int CudaFusedLLGSolver::steps_to_next_stop(int iteration, int max_steps, int min_steps, int max_block,
                                           const std::vector<std::unique_ptr<Monitor>>& monitors) {
  int k = std::max(1, std::min(max_block, max_steps - iteration));
  if (iteration < min_steps) k = std::min(k, min_steps - iteration);
  // the next iteration at which a monitor updates (notify_monitors runs
  // before every run(), src/jams/core/solver.cc:110-116)
  for (int j = 1; j < k; ++j) {
    bool updates = false;
    for (const auto& m : monitors)
      if (m->is_updating(iteration + j)) {
        updates = true;
        break;
      }
    if (updates) return j;
  }
  return k;
}

void CudaFusedLLGSolver::run() {
  if (!h_) throw std::runtime_error(module_ + ": run() before initialize()");
  if (!state_sent_) {
    // the spins JAMS initialised (materials' spin settings, init_h5, ...)
    check(llg_set_state(h_, 0, globals::s.data()));
    check(llg_set_iteration(h_, iteration_));
    state_sent_ = true;
  }
  if (physics_module_) check(llg_set_temperature(h_, 0, physics_module_->temperature()));
  const int k = steps_to_next_stop(iteration_, max_steps_, min_steps_, max_block_, monitors_);
  check(llg_step(h_, k));
  iteration_ += k;
  time_ = iteration_ * step_size_;
  check(llg_get_state(h_, 0, globals::s.data()));
}

void CudaFusedLLGSolver::compute_fields() {
  if (!h_) throw std::runtime_error(module_ + ": compute_fields() before initialize()");
  check(llg_fields(h_, 0, globals::h.data()));
}

FusedTermHamiltonian::FusedTermHamiltonian(const CudaFusedLLGSolver& solver, int term, const std::string& name,
                                           unsigned size)
    : solver_(solver), term_(term) {
  set_name(name);
  energy_.resize(size);
  field_.resize(size, 3);
}

double FusedTermHamiltonian::calculate_total_energy(double /*time: the solver's*/) {
  std::vector<double> e(32);
  double m4[4];
  throw_on(llg_observables(solver_.handle(), 0, m4, e.data()), solver_.handle(), name().c_str());
  return e[term_];
}

void FusedTermHamiltonian::calculate_energies(double) {
  throw std::runtime_error(name() + ": per-spin energies are not computed by the fused LLG library");
}

void FusedTermHamiltonian::calculate_fields(double /*time: the solver's*/) {
  throw_on(llg_term_fields(solver_.handle(), 0, term_, field_.data()), solver_.handle(), name().c_str());
}

Vec3 FusedTermHamiltonian::calculate_field(int, double) {
  throw std::runtime_error(name() + ": single-spin fields are for Monte Carlo solvers, not the LLG path");
}

double FusedTermHamiltonian::calculate_energy(int, double) {
  throw std::runtime_error(name() + ": single-spin energies are for Monte Carlo solvers, not the LLG path");
}

double FusedTermHamiltonian::calculate_energy_difference(int, const Vec3&, const Vec3&, double) {
  throw std::runtime_error(name() + ": energy differences are for Monte Carlo solvers, not the LLG path");
}
