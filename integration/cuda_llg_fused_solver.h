// A JAMS solver module backed by libjams_llg.so (include/jams_llg.h): the
// drop-in for the reference's GPU LLG solvers "llg-heun-gpu" and
// "llg-rk4-gpu" (CUDAHeunLLGSolver, src/jams/solvers/cuda_llg_heun.cu:64-122;
// CUDALLGRK4Solver, src/jams/solvers/cuda_llg_rk4.cu and cuda_rk4_base.cu).
//
// It keeps the reference's plugin interface, class Solver
// (src/jams/core/solver.h:15-88): initialize(settings), run() (advances and
// bumps iteration_ and time_), name(), is_cuda_solver(), compute_fields().
// A maintainer registers it in Solver::create (src/jams/core/solver.cc:60-77)
// in place of the two GPU LLG solvers and calls
// CudaFusedLLGSolver::set_config_text with the config text (and patch string)
// where the driver reads them (src/jams/core/jams++.cc:48-84).  The library
// builds the model from that text: the materials, unit cell, lattice,
// Hamiltonian terms, solver, physics and seed JAMS itself reads.
//
// Cadence rule (src/jams/core/jams++.cc:333-347): the driver calls run()
// once per loop and notifies the monitors before each call.  run() advances
// k steps, k = the fewest of: steps to the next iteration at which any
// monitor updates (Monitor::is_updating), steps to max_steps, steps to
// min_steps (while below it, so that the convergence check sees that
// iteration), and max_block_steps (a solver setting, default 100; set it to 1
// when a physics module changes the temperature within a run, since
// update_physics_module runs once per loop).  Every run() hands the physics
// module's temperature to the library first (Solver::update_thermostat,
// src/jams/core/solver.cc:94-97) and writes the FP64 spins back to
// globals::s afterwards, so monitors see the reference's state at the
// reference's iteration numbers.
//
// Settings read from the solver section besides the reference's (t_step,
// t_max, t_min): precision = "fp32c" (default) or "fp64" (equal to the
// reference's CPU solver bit for bit); max_block_steps.
//
// Errors: every library status other than LLG_OK becomes the
// std::runtime_error the reference's CHECK macros throw
// (src/jams/cuda/cuda_common.h:43-77), with llg_last_error as the message.
#pragma once

#include <jams_llg.h>

#include <memory>
#include <string>
#include <vector>

#include "jams/core/hamiltonian.h"
#include "jams/core/monitor.h"
#include "jams/core/solver.h"

class CudaFusedLLGSolver : public Solver {
 public:
  // the config text (and patch string) the driver read; set before the
  // solver is created
  static void set_config_text(const std::string& text, const std::string& patch);

  CudaFusedLLGSolver() = default;
  explicit CudaFusedLLGSolver(const libconfig::Setting& settings) { initialize(settings); }
  ~CudaFusedLLGSolver() override;

  void initialize(const libconfig::Setting& settings) override;
  void run() override;
  std::string name() const override { return module_; }
  bool is_cuda_solver() const override { return true; }
  // globals::h = the total field at the current spins (meV), as
  // CudaSolver::compute_fields (src/jams/cuda/cuda_solver.cc:11-26)
  void compute_fields() override;

  llg_handle* handle() const { return h_; }

  // the steps run() advances from `iteration`: the cadence rule above
  static int steps_to_next_stop(int iteration, int max_steps, int min_steps, int max_block,
                                const std::vector<std::unique_ptr<Monitor>>& monitors);

 private:
  void check(int rc) const;
  llg_handle* h_ = nullptr;
  std::string module_ = "llg-heun-gpu";
  int precision_ = LLG_FP32C;
  int max_block_ = 100;
  bool state_sent_ = false;
};

// One Hamiltonian term evaluated by the library: calculate_fields fills
// field_ with that term's field at the solver's current spins and time
// (llg_term_fields), calculate_total_energy gives its energy
// (llg_observables).  The reference's Hamiltonian interface
// (src/jams/core/hamiltonian.h:15-78) also has per-spin energies, fields and
// energy differences for Monte Carlo solvers; those are not on the LLG path
// and throw.
class FusedTermHamiltonian : public Hamiltonian {
 public:
  FusedTermHamiltonian(const CudaFusedLLGSolver& solver, int term, const std::string& name, unsigned size);

  double calculate_total_energy(double time) override;
  void calculate_energies(double time) override;
  void calculate_fields(double time) override;
  Vec3 calculate_field(int i, double time) override;
  double calculate_energy(int i, double time) override;
  double calculate_energy_difference(int i, const Vec3& spin_initial, const Vec3& spin_final, double time) override;

 private:
  const CudaFusedLLGSolver& solver_;
  int term_;
};
