"""The GPU forms against fixtures made by the reference's own code and
against the oracle, at the lengths the benchmark states.

Tolerances:
  FP64 Heun   bit-exact (max |dS| == 0) after 1000 T = 0 steps: the simple-
              cubic benchmark lattice (32^3) against the reference's own
              run, and bcc 64^3 x 2 (three shells, cubic) against the oracle
  FP64 RK4    max |dS| <= 1e-12 after 1000 steps against the reference's RK4
              kernels (they normalise with a reciprocal square root)
  FP32C       max |dS| <= 1e-5 after 1000 T = 0 steps
  thermal     <|M|> and <E> (total and exchange) of each form within 4
              combined numerical standard errors of the reference's own
              thermal run (pcg32 + std::normal_distribution noise), at 40 K
              (ordered phase) and 300 K (paramagnetic), bcc 10^3 x 2 with
              the three-shell exchange and cubic anisotropy"""
import math
import os

import numpy as np
import pytest

from jams_gb300 import stats
from jams_gb300 import workloads as W
from tests.golden.cases import THERMAL_SEED, long_cases, thermal_cases, thermal_summary

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FP32C_TOL = 1e-5
RK4_TOL = 1e-12


def test_fp64_equals_reference_after_1000_steps_sc32(llg):
    w, _, _ = long_cases()["sc32_heun_1000"]
    g = np.load(os.path.join(GOLDEN, "sc32_heun_1000.npz"))
    s = llg.Solver(w, precision=llg.FP64)
    s.set_state(W.initial_state(w, 0))
    s.step(1000)
    got = s.get_state(0)
    assert np.array_equal(got, g["s1000"]), np.abs(got - g["s1000"]).max()
    f = llg.Solver(w, precision=llg.FP32C)
    f.set_state(W.initial_state(w, 0))
    f.step(1000)
    assert np.abs(f.get_state(0) - g["s1000"]).max() <= FP32C_TOL


def test_fp64_equals_oracle_after_1000_steps_bcc64(llg, oracle):
    w = W.bcc_three_shell(L=64, T=0.0, start="random")
    s0 = W.initial_state(w, 0)
    ref = oracle.OracleSim(w, threads=os.cpu_count() or 1).run(s0, 1000)
    s = llg.Solver(w, precision=llg.FP64)
    s.set_state(s0)
    s.step(1000)
    got = s.get_state(0)
    assert np.array_equal(got, ref), np.abs(got - ref).max()
    f = llg.Solver(w, precision=llg.FP32C)
    f.set_state(s0)
    f.step(1000)
    assert np.abs(f.get_state(0) - ref).max() <= FP32C_TOL


@pytest.mark.parametrize("precision", ["FP64", "FP32C"])
def test_rk4_agrees_with_the_reference_rk4_kernels(llg, precision):
    w, _, keep = long_cases()["tri16_dmi_rk4_1000"]
    g = np.load(os.path.join(GOLDEN, "tri16_dmi_rk4_1000.npz"))
    tol = RK4_TOL if precision == "FP64" else FP32C_TOL
    s = llg.Solver(w, precision=getattr(llg, precision))
    s.set_state(g["s0"])
    done = 0
    for k in keep:
        s.step(k - done)
        done = k
        d = np.abs(s.get_state(0) - g["s%d" % k]).max()
        assert d <= tol, (k, d)


def sampled_run(llg, w, precision, burn, every, nsamp):
    s = llg.Solver(w, precision=precision)
    s.set_state(W.initial_state(w, 0))
    s.step(burn)
    abs_m, energies = [], []
    for _ in range(nsamp):
        s.step(every)
        m, e = s.observables(0)
        abs_m.append(m[3])
        energies.append(e)
    s.close()
    return thermal_summary(abs_m, energies, w.total_spins)


@pytest.mark.parametrize("precision", ["FP64", "FP32C"])
@pytest.mark.parametrize("name", sorted(thermal_cases()))
def test_equilibrium_matches_the_reference_within_error_bars(llg, name, precision):
    w, burn, every, nsamp = thermal_cases()[name]
    w.seed = THERMAL_SEED % 100003
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    got = sampled_run(llg, w, getattr(llg, precision), burn, every, nsamp)
    for q in ("abs_m", "e_total", "e_term0"):
        ref, err_ref = float(g[q + "_mean"]), float(g[q + "_nse"])
        err = math.sqrt(err_ref ** 2 + got[q + "_nse"] ** 2)
        assert abs(got[q + "_mean"] - ref) < 4 * err, (q, got[q + "_mean"], ref, err)
