// Test driver for integration/cuda_llg_fused_solver.{h,cc}, built against
// the reference's headers (src/jams) with the oracle's stand-in headers and
// linked to libjams_llg.so by tests/test_adapter.py.  Test infrastructure:
// it supplies the globals storage, cblas_daxpy and the Monitor base members the adapter's
// cadence rule calls (src/jams/core/monitor.cc:65-70 restated: a monitor
// updates when the iteration is a multiple of its output_steps), then checks
//   1. the cadence rule: the iterations at which monitors update, the
//      iterations the driver loop visits at and above min_steps, and the
//      final iteration equal those of the reference's one-step-per-run()
//      loop (src/jams/core/jams++.cc:333-347), for several monitor sets;
//   2. the error convention: without a GPU, creating the solver throws
//      std::runtime_error carrying the library's message;
//   3. the link: a CPU-only library call (llg_config_describe) answers.
#define GLOBALORIGIN
#include <jams/core/globals.h>

#include <cstdio>
#include <cstring>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include "cuda_llg_fused_solver.h"

// Solver::compute_fields (in Solver's vtable) sums the terms with cblas_daxpy
extern "C" void cblas_daxpy(int n, double a, const double* x, int incx, double* y, int incy) {
  for (int i = 0; i < n; ++i) y[i * incy] += a * x[i * incx];
}

Monitor::Monitor(const libconfig::Setting& settings)
    : Base(settings), output_step_freq_(settings["output_steps"]), convergence_status_(ConvergenceStatus::kDisabled),
      convergence_tolerance_(0), convergence_stderr_(0), convergence_burn_time_(0) {}

bool Monitor::is_updating(const int& iteration) { return iteration % output_step_freq_ == 0; }

namespace {

class CountingMonitor : public Monitor {
 public:
  CountingMonitor(const libconfig::Setting& s, std::vector<int>* log) : Monitor(s), log_(log) {}
  void update(Solver& solver) override { log_->push_back(solver.iteration()); }
  void post_process() override {}

 private:
  std::vector<int>* log_;
};

libconfig::Setting monitor_settings(int every) {
  libconfig::Setting s(libconfig::Setting::TypeGroup);
  s.add("module", libconfig::Setting::string("counting"));
  s.add("output_steps", libconfig::Setting::integer(every));
  return s;
}

// the reference's loop with one step per run() (k = 1) or with the
// adapter's cadence rule; returns the monitor updates and the loop's visits
struct Trace {
  std::vector<int> updates;
  std::vector<int> visits;
};

class LoopSolver : public Solver {
 public:
  LoopSolver(int max_steps, int min_steps, int block) : block_(block) {
    max_steps_ = max_steps;
    min_steps_ = min_steps;
    step_size_ = 1.0;
  }
  void initialize(const libconfig::Setting&) override {}
  std::string name() const override { return "loop"; }
  void run() override {
    const int k = block_ ? CudaFusedLLGSolver::steps_to_next_stop(iteration_, max_steps_, min_steps_, block_, monitors_)
                         : 1;
    iteration_ += k;
  }

 private:
  int block_;
};

Trace drive(int max_steps, int min_steps, int block, const std::vector<int>& every) {
  Trace t;
  LoopSolver s(max_steps, min_steps, block);
  for (int e : every) s.register_monitor(new CountingMonitor(monitor_settings(e), &t.updates));
  while (s.is_running()) {
    s.notify_monitors();
    if (s.iteration() >= min_steps) t.visits.push_back(s.iteration());
    s.run();
  }
  t.visits.push_back(s.iteration());
  return t;
}

int failures = 0;

void expect(bool ok, const std::string& what) {
  if (!ok) {
    std::printf("FAIL %s\n", what.c_str());
    ++failures;
  }
}

}  // namespace

int main() {
  struct Case {
    int max_steps, min_steps, block;
    std::vector<int> every;
  };
  const std::vector<Case> cases = {
      {1000, 0, 100, {100}},        {1000, 0, 100, {7, 50}},   {1003, 0, 64, {250, 1000}},
      {20000, 0, 100, {}},          {500, 333, 100, {100}},    {37, 0, 100, {5, 13}},
      {10, 0, 100, {1}},            {1000, 10, 1, {3}},        {999, 0, 128, {1000}},
  };
  for (const auto& c : cases) {
    const Trace ref = drive(c.max_steps, c.min_steps, 0, c.every);
    const Trace got = drive(c.max_steps, c.min_steps, c.block, c.every);
    const std::string name = "max " + std::to_string(c.max_steps) + " min " + std::to_string(c.min_steps) +
                             " block " + std::to_string(c.block);
    expect(ref.updates == got.updates, name + ": monitor updates differ");
    expect(ref.visits.back() == got.visits.back(), name + ": final iteration differs");
    // every iteration the adapter's loop visits is one the reference visits,
    // and every monitor update and the min_steps iteration are among them
    const std::set<int> ref_visits(ref.visits.begin(), ref.visits.end());
    for (int v : got.visits) expect(ref_visits.count(v) == 1, name + ": visit " + std::to_string(v));
    if (c.min_steps > 0 && c.min_steps < c.max_steps) {
      bool seen = false;
      for (int v : got.visits) seen |= v == c.min_steps;
      expect(seen, name + ": min_steps iteration not visited");
    }
    for (size_t i = 1; i < got.visits.size(); ++i)
      expect(got.visits[i] - got.visits[i - 1] <= c.block, name + ": a run() advanced past max_block_steps");
  }

  // error convention without a GPU: the library's status becomes a
  // std::runtime_error with its message
  {
    CudaFusedLLGSolver::set_config_text("", "");
    libconfig::Setting s(libconfig::Setting::TypeGroup);
    s.add("module", libconfig::Setting::string("llg-heun-gpu"));
    s.add("t_step", libconfig::Setting::number(1e-15));
    s.add("t_max", libconfig::Setting::number(1e-12));
    bool threw = false;
    try {
      CudaFusedLLGSolver solver(s);
    } catch (const std::runtime_error& e) {
      threw = std::strstr(e.what(), "set_config_text") != nullptr;
    }
    expect(threw, "missing config text is reported");
    s.add("precision", libconfig::Setting::string("fp16"));
    CudaFusedLLGSolver::set_config_text("x", "");
    threw = false;
    try {
      CudaFusedLLGSolver solver(s);
    } catch (const std::runtime_error& e) {
      threw = std::strstr(e.what(), "precision") != nullptr;
    }
    expect(threw, "an unknown precision is reported");
  }

  // the link: a library call that needs no GPU
  {
    const char* cfg =
        "materials = ( { name = \"Fe\"; moment = 2.2; gyro = 1.0; alpha = 0.05; spin = [0.0, 0.0, 1.0]; } );\n"
        "unitcell : { parameter = 2.87e-10; basis = ( [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0] );\n"
        "  positions = ( (\"Fe\", [0.0, 0.0, 0.0]) ); };\n"
        "lattice : { size = [4, 4, 4]; periodic = [true, true, true]; };\n"
        "hamiltonians = ( { module = \"exchange\"; energy_units = \"meV\"; interactions = (\n"
        "  (\"Fe\", \"Fe\", [1.0, 0.0, 0.0], 1.0), (\"Fe\", \"Fe\", [-1.0, 0.0, 0.0], 1.0),\n"
        "  (\"Fe\", \"Fe\", [0.0, 1.0, 0.0], 1.0), (\"Fe\", \"Fe\", [0.0, -1.0, 0.0], 1.0),\n"
        "  (\"Fe\", \"Fe\", [0.0, 0.0, 1.0], 1.0), (\"Fe\", \"Fe\", [0.0, 0.0, -1.0], 1.0) ); } );\n"
        "solver : { module = \"llg-heun-gpu\"; t_step = 1.0e-15; t_max = 1.0e-12; };\n"
        "physics : { temperature = 0.0; };\n";
    std::vector<char> json(1 << 16);
    const int rc = llg_config_describe(cfg, "", json.data(), (int64_t)json.size());
    expect(rc == LLG_OK && std::strstr(json.data(), "\"nb\"") != nullptr,
           std::string("llg_config_describe: ") + (rc == LLG_OK ? "ok" : llg_last_error(nullptr)));
  }

  std::printf("%s (%d failures)\n", failures ? "FAILED" : "adapter checks passed", failures);
  return failures ? 1 : 0;
}
