"""The oracle against fixtures made by the reference's own code
(tests/golden/make_golden.py), at lengths and integrators the short golden
cases do not reach:

  sc32_heun_1000      the simple-cubic benchmark lattice (32^3, random start,
                      T = 0): the reference's HeunLLGSolver::run for 1000
                      steps; the oracle equals it bit for bit.
  tri16_dmi_rk4_1000  triangular DMI monolayer, RK4: the reference's RK4
                      kernels (cuda_llg_rk4_kernel, the RK4 combination and
                      normalisation) built for the host and driven as
                      CudaRK4BaseSolver::run; the oracle's RK4 restatement
                      agrees within 1e-12 (the reference normalises with a
                      reciprocal square root, the oracle divides by |s|).
  thermal_*           the reference's thermal Heun runs (independent seeds):
                      the stored mean and standard error are those of the runs."""
import hashlib
import os

import numpy as np
import pytest

from jams_gb300 import workloads as W
from tests.golden.cases import long_cases, thermal_cases

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
RK4_TOL = 1e-12


def test_sc32_start_is_the_fixtures():
    w, _, _ = long_cases()["sc32_heun_1000"]
    g = np.load(os.path.join(GOLDEN, "sc32_heun_1000.npz"))
    assert hashlib.sha256(W.initial_state(w, 0).tobytes()).hexdigest() == str(g["s0_sha256"])


def test_oracle_equals_reference_after_1000_heun_steps_sc32(oracle):
    w, _, _ = long_cases()["sc32_heun_1000"]
    g = np.load(os.path.join(GOLDEN, "sc32_heun_1000.npz"))
    got = oracle.OracleSim(w).run(W.initial_state(w, 0), 1000)
    assert np.array_equal(got, g["s1000"]), np.abs(got - g["s1000"]).max()


def test_oracle_rk4_agrees_with_the_reference_rk4_kernels(oracle):
    w, _, keep = long_cases()["tri16_dmi_rk4_1000"]
    g = np.load(os.path.join(GOLDEN, "tri16_dmi_rk4_1000.npz"))
    sim = oracle.OracleSim(w)
    s, done = g["s0"], 0
    for k in keep:
        s = sim.run(s, k - done, first_step=done)
        done = k
        d = np.abs(s - g["s%d" % k]).max()
        assert d <= RK4_TOL, (k, d)


@pytest.mark.parametrize("name", sorted(thermal_cases()))
def test_thermal_fixtures_hold_independent_runs(name):
    """Each thermal fixture holds the reference's runs for independent seeds,
    their mean and standard error; the stored summary is that of the runs."""
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    assert len(set(g["seeds"].tolist())) == len(g["seeds"]) >= 8
    for q in ("abs_m", "e_total", "e_term0", "e_term1"):
        runs = g[q + "_runs"]
        assert runs.size == g["seeds"].size and np.all(np.isfinite(runs))
        assert float(g[q + "_mean"]) == pytest.approx(runs.mean(), rel=1e-12)
        assert float(g[q + "_err"]) == pytest.approx(runs.std(ddof=1) / np.sqrt(runs.size), rel=1e-12)
        assert g[q + "_err"] > 0


def test_reference_rk4_kernels_run_here_when_built(oracle):
    """Where the reference build exists, its RK4 driver reproduces the
    fixture (the fixture was made by it)."""
    if not oracle.reference_available():
        pytest.skip("oracle/_ref not built (needs the reference sources)")
    w, _, _ = long_cases()["tri16_dmi_rk4_1000"]
    g = np.load(os.path.join(GOLDEN, "tri16_dmi_rk4_1000.npz"))
    got = oracle.ReferenceSim(w).rk4_run(g["s0"], 100)
    assert np.array_equal(got, g["s100"])
