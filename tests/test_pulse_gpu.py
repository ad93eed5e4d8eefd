"""Time-dependent fields on the GPU: applied-field sinc and sinc-cos pulses and
the zeeman dc / ac term, evaluated at the reference's stage times (Heun t0,
t0 + dt; RK4 t0, t0 + dt/2, t0 + dt/2, t0 + dt; t0 = iteration dt).

The time factors come from the host's C library, as the oracle's do: on one
machine the FP64 form equals the oracle bit for bit.  Against the golden
fixtures (made by the reference on another machine) it agrees within 1e-12."""
import copy
import os

import numpy as np
import pytest

from jams_gb300 import workloads as W
from tests.golden.cases import pulse_cases

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FP32C_TOL = 1e-5


def rk4(w):
    w = copy.deepcopy(w)
    w.model.integrator = W.RK4
    return w


def thermal(w, T=200.0):
    w = copy.deepcopy(w)
    for r in w.replicas:
        r.temperature = T
    return w


@pytest.mark.parametrize("name", sorted(pulse_cases().keys()))
def test_fp64_pulse_fields_follow_the_reference_golden_vectors(llg, name):
    w = pulse_cases()[name]
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    s = llg.Solver(w, precision=llg.FP64, steps_per_graph=8)
    s.set_state(g["s0"])
    np.testing.assert_allclose(s.fields(0), g["fields"], rtol=1e-14, atol=1e-14)
    done = 0
    for k in (1, 10, 100):
        s.step(k - done)
        done = k
        np.testing.assert_allclose(s.get_state(0), g["s%d" % k], rtol=0, atol=1e-12)
    np.testing.assert_allclose(s.fields(0), g["fields100"], rtol=1e-12, atol=1e-14)
    _, e = s.observables(0)
    np.testing.assert_allclose(e, g["energies100"], rtol=1e-11, atol=1e-12)
    s.synchronize()


@pytest.mark.parametrize("name", sorted(pulse_cases().keys()))
@pytest.mark.parametrize("variant", ["heun", "rk4", "heun_T"])
def test_fp64_pulse_equals_oracle(llg, oracle, name, variant):
    """Bit for bit with the oracle over step calls of several lengths (each
    call fills its own time-factor table), at T = 0 and T > 0, Heun and RK4;
    fields and energies at the solver time afterwards."""
    w = pulse_cases()[name]
    w = rk4(w) if variant == "rk4" else (thermal(w) if variant == "heun_T" else w)
    s0 = W.initial_state(w, 0)
    o = oracle.OracleSim(w)
    ref = o.run(s0, 47)
    s = llg.Solver(w, precision=llg.FP64, steps_per_graph=4)
    s.set_state(s0)
    for n in (7, 1, 13, 26):
        s.step(n)
    assert s.iteration == 47
    got = s.get_state(0)
    assert np.array_equal(got, ref), "max |dS| = %g" % np.abs(got - ref).max()
    assert np.array_equal(s.fields(0), o.fields(ref))
    _, e = s.observables(0)
    np.testing.assert_allclose(e, o.energies(ref), rtol=1e-12, atol=1e-13)


def test_fp64_pulse_table_chunks(llg, oracle):
    """One call longer than the factor table (4096 steps at two steps per
    graph) runs in chunks, each with its own table."""
    w = pulse_cases()["sc4x5x6_sinc_cos_zeeman_ac"]
    s0 = W.initial_state(w, 0)
    ref = oracle.OracleSim(w).run(s0, 4100)
    s = llg.Solver(w, precision=llg.FP64, steps_per_graph=2)
    s.set_state(s0)
    s.step(4100)
    assert np.array_equal(s.get_state(0), ref)


def _split_exchange(w):
    """The exchange as two terms, the second with a small symmetric
    off-diagonal part: the gather kernels run."""
    return W.split_exchange(w, offdiag=0.05)


@pytest.mark.parametrize("name", sorted(pulse_cases().keys()))
@pytest.mark.parametrize("path", ["tiled", "gather", "tiled_rk4", "gather_rk4"])
def test_fp32c_pulse_within_bound(llg, oracle, name, path):
    w = pulse_cases()[name]
    if path.endswith("rk4"):
        w = rk4(w)
    if path.startswith("gather"):
        w = _split_exchange(w)
    s0 = W.initial_state(w, 0)
    ref = oracle.OracleSim(w).run(s0, 200)
    s = llg.Solver(w, precision=llg.FP32C, steps_per_graph=16)
    assert (s.kernel_info()["family"] == "generic") == path.startswith("gather")
    s.set_state(s0)
    s.step(200)
    d = np.abs(s.get_state(0) - ref).max()
    assert d <= FP32C_TOL, d


@pytest.mark.parametrize("name", sorted(pulse_cases().keys()))
def test_fp32c_pulse_tilings_agree(llg, name):
    """Stored or recomputed rhs(s0) (the corrector then evaluates the field of
    s0 with the predictor's time factors), planes per CTA and rows per thread
    give the same spins bit for bit."""
    w = thermal(pulse_cases()[name], 100.0)
    outs = []
    for tx, store, occ, pair in [(2, True, 4, False), (2, False, 2, False), (6, False, 3, False),
                                 (4, True, 2, True), (8, False, 2, True)]:
        s = llg.Solver(w, precision=llg.FP32C, steps_per_graph=4)
        s.set_tuning(tx, store, occ, False, pair)
        s.set_state(W.initial_state(w, 0))
        s.step(9)
        s.step(14)
        outs.append(s.get_state(0))
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])


def test_pulse_config_run_equals_workload_run(llg):
    """A config file with a sinc-cos applied field and a zeeman ac term runs
    the same FP64 trajectory as the equivalent workload description."""
    from tests.test_config import pulse_config

    cfg = pulse_config()
    a = llg.Solver.from_config(cfg, precision=llg.FP64)
    s0 = a.get_state(0)
    w = W.sc_ferromagnet(L=4)
    w.model.terms = [w.model.terms[0],
                     W.field_term((0.5, -0.3, 2.0), pulse=W.PULSE_SINC_COS, time_center=1.0e-14 / 1e-12,
                                  freq_bandwidth=5.0e13 / 1e12, freq_center=8.0e13 / 1e12),
                     W.zeeman_term([(0.1, 0.2, -0.3)], [(0.4, 0.0, 0.3)], [30.0])]
    b = llg.Solver(w, precision=llg.FP64)
    b.set_state(s0)
    a.step(30)
    b.step(30)
    assert np.array_equal(a.get_state(0), b.get_state(0))
