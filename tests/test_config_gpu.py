"""Solvers built from JAMS config texts (llg_create_from_config) on the GPU."""
import numpy as np
import pytest

from jams_gb300 import configs as C
from jams_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_config_fp64_run_equals_oracle(llg, oracle):
    text = C.bcc_three_shell(L=6, T=300.0, steps=20, spin='"random"')
    s = llg.Solver.from_config(text, precision=llg.FP64)
    s0 = s.get_state(0)
    np.testing.assert_allclose(np.linalg.norm(s0, axis=1), 1.0, rtol=1e-15)
    assert abs(s0.mean(axis=0)).max() < 0.2  # random directions
    assert s.max_steps == 20
    w = W.bcc_three_shell(L=6, T=300.0, start="random")
    ref = oracle.OracleSim(w).run(s0, 20)
    s.step(s.max_steps)
    assert np.array_equal(s.get_state(0), ref)


def test_config_patch_sets_temperature(llg):
    text = C.sc_ferromagnet(L=8, T=0.0, steps=10)
    a = llg.Solver.from_config(text, precision=llg.FP32C)
    b = llg.Solver.from_config(text, 'physics : { temperature = 50.0; };', precision=llg.FP32C)
    assert np.array_equal(a.get_state(0), b.get_state(0))
    a.step(10)
    b.step(10)
    assert not np.array_equal(a.get_state(0), b.get_state(0))


def test_config_rk4_triangular(llg, oracle):
    text = C.triangular_dmi(L=16, T=0.0, Bz=1.0, steps=30)
    s = llg.Solver.from_config(text, precision=llg.FP64)
    s0 = s.get_state(0)
    w = W.triangular_dmi_field_sweep(L=16, n_fields=1, T=0.0)
    w.replicas[0].B = (0.0, 0.0, 1.0)
    ref = oracle.OracleSim(w).run(s0, 30)
    s.step(30)
    assert np.array_equal(s.get_state(0), ref)


def test_two_exchange_modules_run_the_tiled_kernels(llg):
    """A config with the three bcc shells split over two exchange modules:
    FP32C sums them into the three-shell stencil, so the run equals the
    one-module config's bit for bit, and the two terms' exchange energies add
    up to the one term's."""
    one = C.bcc_three_shell(L=6, T=300.0, steps=20, spin='"random"')
    shell1 = '      ("Fe", "Fe", [0.5, 0.5, 0.5], 2.0),    // shell 1: 8 at a<111>/2\n'
    assert one.count(shell1) == 1
    two = one.replace(shell1, '      ("Fe", "Fe", [0.5, 0.5, 0.5], 2.0)\n    );\n  },\n  {\n'
                              '    module = "exchange";\n    energy_units = "meV";\n    interactions = (\n')
    a = llg.Solver.from_config(one, precision=llg.FP32C)
    b = llg.Solver.from_config(two, precision=llg.FP32C)
    assert a.n_terms + 1 == b.n_terms
    assert a.kernel_info()["family"] == b.kernel_info()["family"] == "bcc3"
    assert np.array_equal(a.get_state(0), b.get_state(0))
    a.step(20)
    b.step(20)
    assert np.array_equal(a.get_state(0), b.get_state(0))
    ea, eb = a.observables(0)[1], b.observables(0)[1]
    np.testing.assert_allclose(eb[0] + eb[1], ea[0], rtol=1e-12)
    np.testing.assert_allclose(eb[2:], ea[1:], rtol=1e-12)


def test_exc_file_config_runs_like_the_inline_config(llg, tmp_path):
    """The three bcc shells read from an exc_file (JAMS format) give the
    inline config's FP64 trajectory bit for bit."""
    inline = C.bcc_three_shell(L=6, T=300.0, steps=20, spin='"random"')
    block = inline[inline.index("    interactions = ("):inline.index("    );\n", inline.index("    interactions = (")) + 7]
    exc = tmp_path / "bcc3.txt"
    exc.write_text("# type_i type_j rx ry rz J (meV)\nFe Fe 0.5 0.5 0.5 2.0\nFe Fe 1.0 0.0 0.0 1.2\n"
                   "Fe Fe 1.0 1.0 0.0 -0.1\n")
    from_file = inline.replace(block, '    exc_file = "%s";\n' % exc)
    assert from_file != inline
    a = llg.Solver.from_config(inline, precision=llg.FP64)
    b = llg.Solver.from_config(from_file, precision=llg.FP64)
    assert np.array_equal(a.get_state(0), b.get_state(0))
    a.step(20)
    b.step(20)
    assert np.array_equal(a.get_state(0), b.get_state(0))
