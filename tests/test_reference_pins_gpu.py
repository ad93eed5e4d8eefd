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
              combined standard errors of the reference's own thermal runs
              (pcg32 + std::normal_distribution noise), at 40 K (ordered
              phase) and 300 K (paramagnetic), bcc 10^3 x 2 with the
              three-shell exchange and cubic anisotropy.  Each side's error
              is the standard error over independent runs: 8 seeds of the
              reference, 16 replicas of each GPU form in one batched handle"""
import copy
import math
import os

import numpy as np
import pytest

from jams_gb300 import stats
from jams_gb300 import workloads as W
from tests.golden.cases import THERMAL_GPU_REPLICAS, THERMAL_SEED, long_cases, over_runs, thermal_cases

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


def replica_averages(llg, w, precision, burn, every, nsamp, replicas):
    """Time averages of |M| and the energies per spin of `replicas`
    independent copies of the model's replica 0, integrated in one batched
    handle (each replica has its own Philox stream)."""
    w = copy.deepcopy(w)
    w.replicas = [copy.deepcopy(w.replicas[0]) for _ in range(replicas)]
    s = llg.Solver(w, precision=precision)
    for r in range(replicas):
        s.set_state(W.initial_state(w, r), r)
    s.step(burn)
    n = w.spins_per_replica[0]
    acc = {q: np.zeros(replicas) for q in ("abs_m", "e_total", "e_term0", "e_term1")}
    for _ in range(nsamp):
        s.step(every)
        for r in range(replicas):
            m, e = s.observables(r)
            acc["abs_m"][r] += m[3]
            acc["e_total"][r] += e.sum() / n
            acc["e_term0"][r] += e[0] / n
            acc["e_term1"][r] += e[1] / n
    s.close()
    return over_runs({q: v / nsamp for q, v in acc.items()})


@pytest.mark.parametrize("precision", ["FP64", "FP32C"])
@pytest.mark.parametrize("name", sorted(thermal_cases()))
def test_equilibrium_matches_the_reference_within_error_bars(llg, name, precision):
    w, burn, every, nsamp = thermal_cases()[name]
    w.seed = THERMAL_SEED % 100003
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    got = replica_averages(llg, w, getattr(llg, precision), burn, every, nsamp, THERMAL_GPU_REPLICAS)
    for q in ("abs_m", "e_total", "e_term0"):
        ref, err_ref = float(g[q + "_mean"]), float(g[q + "_err"])
        err = math.sqrt(err_ref ** 2 + got[q + "_err"] ** 2)
        assert abs(got[q + "_mean"] - ref) < 4 * err, (q, got[q + "_mean"], ref, err)
