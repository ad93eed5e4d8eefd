"""The restated reference GPU path (baseline/refgpu.cu, the ref-GPU column of
bench.py) computes the same Heun trajectory as the FP64 form: it is timed
doing the real work.  cuSPARSE sums each CSR row in its own order, so the
agreement is to rounding, not bit for bit."""
import numpy as np
import pytest

from jams_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def refgpu():
    from baseline import refgpu as R

    try:
        R.build()
    except RuntimeError as e:
        pytest.skip("ref-GPU baseline not built: %s" % str(e)[-200:])
    return R


@pytest.mark.parametrize("name", ["sc", "bcc3", "bcc_nn"])
def test_refgpu_trajectory_matches_fp64(llg, refgpu, name):
    w = {"sc": W.sc_ferromagnet(L=(6, 7, 8)),
         "bcc3": W.bcc_three_shell(L=6, T=0.0, start="random"),
         "bcc_nn": W.bcc_nearest_neighbour(L=5, T=0.0, start="random")}[name]
    s0 = W.initial_state(w, 0)
    ours = llg.Solver(w, precision=llg.FP64)
    ours.set_state(s0)
    ours.step(50)
    ref = refgpu.RefGpu(w)
    ref.set_state(s0)
    ms = ref.run(50)
    assert ms > 0.0
    d = np.abs(ref.get_state() - ours.get_state(0)).max()
    assert d < 1e-11, d


def test_refgpu_thermal_run_stays_normalised(llg, refgpu):
    w = W.bcc_three_shell(L=6, T=300.0, start="random")
    ref = refgpu.RefGpu(w)
    ref.set_state(W.initial_state(w, 0))
    ref.run(20)
    s = ref.get_state()
    assert np.isfinite(s).all()
    np.testing.assert_allclose(np.linalg.norm(s, axis=1), 1.0, atol=1e-12)
