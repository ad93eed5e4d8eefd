"""The dipole-dipole term on the GPU (FFT convolution with this library's
own transforms and k-space product) against the oracle's direct sum: fields,
energies and trajectories, periodic and open boundaries, Heun and RK4, both
precisions, the tiled and the gather FP32 kernels."""
import copy
import os

import numpy as np
import pytest

from jams_gb300 import configs as C
from jams_gb300 import workloads as W
from tests.golden.cases import dipole_cases

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")

pytestmark = pytest.mark.gpu

FP64_FIELD_TOL = 1e-12       # relative to the largest field component
FP32C_FIELD_TOL = 2e-6
FP64_RUN_TOL = 1e-10         # max |dS| after 100 T = 0 steps (FFT rounding, not bit-exact)
FP32C_RUN_TOL = 1e-5         # max |dS| after 1000 T = 0 steps
# the dipole term's field alone, relative to its largest component: the FP32
# transforms round at ~1e-7 per pass, the tensors are stored in single
# precision
FP64_DIPOLE_TOL = 1e-11
FP32C_DIPOLE_TOL = 2e-5


def cases():
    return {
        "bcc3_periodic": W.bcc_three_shell(L=(6, 5, 7), T=0.0, start="random", dipole_cutoff=2.4),
        "sc_film_open_z": W.sc_ferromagnet(L=(8, 6, 3), periodic=(1, 1, 0), dipole_cutoff=2.2, B=(0, 0, 0.3)),
        "triangular_rk4": W.triangular_dmi_field_sweep(L=(10, 12, 1), n_fields=2, T=0.0, dipole_cutoff=3.1),
    }


def transform_cases():
    """Grids whose axes take every transform kernel: the single-precision
    register passes (power-of-two lengths 16..1024: the last grid axis as a
    real pass, the others as strided complex passes) beside the Stockham
    passes (other lengths, and every FP64 axis).  A periodic axis of L cells
    is an FFT axis of L points, an open one of 2L."""
    return {
        "bcc16_periodic": W.bcc_three_shell(L=16, T=0.0, start="random", dipole_cutoff=2.4),
        "sc_4x4x256": W.sc_ferromagnet(L=(4, 4, 256), dipole_cutoff=1.5),
        "sc_256x4x3": W.sc_ferromagnet(L=(256, 4, 3), dipole_cutoff=1.0),
        "sc_film_32x16x16_open_z": W.sc_ferromagnet(L=(32, 16, 16), periodic=(1, 1, 0), dipole_cutoff=2.2),
        "sc_128x64x8": W.sc_ferromagnet(L=(128, 64, 8), dipole_cutoff=1.5),
        "sc_4x4x256_open_z": W.sc_ferromagnet(L=(4, 4, 256), periodic=(1, 1, 0), dipole_cutoff=1.5),
        "sc_3x3x1024": W.sc_ferromagnet(L=(3, 3, 1024), dipole_cutoff=1.0),
        "sc_1024x3x3": W.sc_ferromagnet(L=(1024, 3, 3), dipole_cutoff=1.0),
    }


def start(w, r=0):
    return W.initial_state(w, r)


def oracle_dipole_field(oracle, w, s0):
    """The oracle's dipole field: its total field less the field of the same
    model without the dipole term (both in FP64)."""
    w2 = copy.deepcopy(w)
    w2.model.terms = [t for t in w2.model.terms if t.kind != W.TERM_DIPOLE]
    return oracle.OracleSim(w, 0).fields(s0) - oracle.OracleSim(w2, 0).fields(s0)


@pytest.mark.parametrize("name", sorted(transform_cases()))
@pytest.mark.parametrize("prec", ["FP64", "FP32C"])
def test_dipole_term_field_on_every_transform_length(llg, oracle, name, prec):
    w = transform_cases()[name]
    s = llg.Solver(w, precision=getattr(llg, prec))
    s0 = start(w)
    s.set_state(s0, 0)
    want = oracle_dipole_field(oracle, w, s0)
    got = s.term_fields([t.kind for t in w.model.terms].index(W.TERM_DIPOLE), 0)
    tol = FP64_DIPOLE_TOL if prec == "FP64" else FP32C_DIPOLE_TOL
    assert np.abs(want).max() > 0
    assert np.abs(got - want).max() <= tol * np.abs(want).max()


@pytest.mark.parametrize("name", sorted(cases()))
@pytest.mark.parametrize("prec", ["FP64", "FP32C"])
def test_dipole_fields_and_energies_match_oracle(llg, oracle, name, prec):
    w = cases()[name]
    s = llg.Solver(w, precision=getattr(llg, prec))
    s0 = start(w)
    s.set_state(s0, 0)
    ref = oracle.OracleSim(w, 0)
    want = ref.fields(s0)
    got = s.fields(0)
    tol = FP64_FIELD_TOL if prec == "FP64" else FP32C_FIELD_TOL
    assert np.abs(got - want).max() <= tol * np.abs(want).max()
    e_want = ref.energies(s0)
    _, e_got = s.observables(0)
    k = [t.kind for t in w.model.terms].index(W.TERM_DIPOLE)
    np.testing.assert_allclose(e_got[k], e_want[k], rtol=1e-10 if prec == "FP64" else 1e-5)


@pytest.mark.parametrize("name", sorted(cases()))
def test_fp64_dipole_run_matches_oracle(llg, oracle, name):
    w = cases()[name]
    s = llg.Solver(w, precision=llg.FP64, steps_per_graph=16)
    s0 = start(w)
    s.set_state(s0, 0)
    s.step(100)
    ref = oracle.OracleSim(w, 0).run(s0, 100)
    assert np.abs(s.get_state(0) - ref).max() <= FP64_RUN_TOL


@pytest.mark.parametrize("name", sorted(cases()))
def test_fp32c_dipole_run_within_bound(llg, oracle, name):
    w = cases()[name]
    s = llg.Solver(w, precision=llg.FP32C)
    s0 = start(w)
    s.set_state(s0, 0)
    s.step(1000)
    ref = oracle.OracleSim(w, 0).run(s0, 1000)
    assert np.abs(s.get_state(0) - ref).max() <= FP32C_RUN_TOL


@pytest.mark.parametrize("prec", ["FP64", "FP32C"])
def test_replicas_of_different_sizes_each_get_their_own_grid(llg, oracle, prec):
    """Replicas of one handle with different lattices: each has its own FFT
    grid, tensors and plans (register lengths 16 and 32 beside Stockham
    lengths 6, 10 and 12), evaluated back to back into one set of planes."""
    w = W.sc_ferromagnet(L=16, dipole_cutoff=1.5)
    w.replicas = [W.Replica(L=(16, 16, 32)), W.Replica(L=(12, 10, 6)), W.Replica(L=(16, 16, 16))]
    s = llg.Solver(w, precision=getattr(llg, prec))
    k = [t.kind for t in w.model.terms].index(W.TERM_DIPOLE)
    tol = FP64_DIPOLE_TOL if prec == "FP64" else FP32C_DIPOLE_TOL
    for r in range(len(w.replicas)):
        s.set_state(start(w, r), r)
    for r in range(len(w.replicas)):
        wr = copy.deepcopy(w)
        wr.replicas = [w.replicas[r]]
        want = oracle_dipole_field(oracle, wr, start(w, r))
        got = s.term_fields(k, r)
        assert np.abs(got - want).max() <= tol * np.abs(want).max(), r


@pytest.mark.parametrize("name, per_evaluation", [("bcc3_periodic", 7), ("sc_film_open_z", 7), ("triangular_rk4", 5),
                                                   ("bcc16_periodic", 7)])
def test_dipole_launches_are_counted(llg, name, per_evaluation):
    """Each stage evaluates the dipole field first: the forward real pass,
    one complex pass per further grid axis, the k-space product, the passes
    back and the inverse real pass (7 kernels on a 3-D grid, 5 on a
    monolayer), per replica, whichever transform kernels take the axes."""
    w = {**cases(), **transform_cases()}[name]
    s = llg.Solver(w, precision=llg.FP32C, steps_per_graph=4)
    for r in range(len(w.replicas)):
        s.set_state(start(w, r), r)
    s.step(8)
    stages = 2 if w.model.integrator == W.HEUN else 4
    tiled = s.kernel_info()["family"] != "generic"
    blocks = 2   # two 4-step graph blocks; the gather form ends each with a step-counter kernel
    want = 8 * stages * (1 + per_evaluation * len(w.replicas)) + (0 if tiled else blocks)
    assert s.last_launch_count == want


def test_dipole_tilings_agree(llg):
    """The tiled kernels add the FFT field like the other local terms: every
    tiling gives the same state, stored noise included."""
    w = W.bcc_three_shell(L=(6, 8, 10), T=300.0, start="random", dipole_cutoff=2.9)
    outs = []
    for tx, store, occ, noise in [(2, False, 2, False), (4, True, 4, False), (10, True, 3, False),
                                  (4, True, 4, True), (6, True, 2, True)]:
        s = llg.Solver(w, precision=llg.FP32C, steps_per_graph=4)
        assert s.kernel_info()["family"] == "bcc3"
        s.set_tuning(tx, store, occ, noise=noise)
        s.set_state(start(w), 0)
        s.step(9)
        outs.append(s.get_state(0))
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])


def test_dipole_from_config_equals_oracle(llg, oracle):
    text = C.bcc_three_shell(L=5, T=0.0, spin='"random"', dipole_cutoff=2.4)
    s = llg.Solver.from_config(text, precision=llg.FP64)
    w = W.bcc_three_shell(L=5, T=0.0, dipole_cutoff=2.4)
    s0 = s.get_state(0)
    s.step(20)
    ref = oracle.OracleSim(w, 0).run(s0, 20)
    assert np.abs(s.get_state(0) - ref).max() <= FP64_RUN_TOL


@pytest.mark.parametrize("prec", ["FP64", "FP32C"])
def test_axis_longer_than_a_shared_memory_line_is_an_error(llg, prec):
    """An open axis of 2500 cells is a 5000-point transform line: one line
    of a shared-memory pass (two buffers and the twiddles) does not fit a
    CTA in double precision, the precision of the tensors' transforms in
    both forms.  The refusal leaves no error behind for the next handle."""
    w = W.sc_ferromagnet(L=(4, 4, 2500), periodic=(1, 1, 0), dipole_cutoff=1.5)
    with pytest.raises(llg.LLGError, match="longer than the transform supports"):
        llg.Solver(w, precision=getattr(llg, prec))
    ok = W.sc_ferromagnet(L=(4, 4, 2400), periodic=(1, 1, 0), dipole_cutoff=1.5)   # 4800 points
    llg.Solver(ok, precision=getattr(llg, prec)).close()


def test_dipole_cutoff_beyond_inradius_is_an_error(llg):
    w = W.sc_ferromagnet(L=6, dipole_cutoff=3.5)
    with pytest.raises(llg.LLGError, match="inradius"):
        llg.Solver(w, precision=llg.FP32C)


@pytest.mark.parametrize("name", sorted(dipole_cases().keys()))
@pytest.mark.parametrize("prec", ["FP64", "FP32C"])
def test_dipole_against_reference_golden_vectors(llg, name, prec):
    """Fixtures from the reference's dipole-bruteforce Hamiltonian and CPU
    Heun solver compiled from its sources: fields and 100 Heun steps."""
    w = dipole_cases()[name]
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    s = llg.Solver(w, precision=getattr(llg, prec), steps_per_graph=16)
    s.set_state(g["s0"], 0)
    h = s.fields(0)
    tol = FP64_FIELD_TOL if prec == "FP64" else FP32C_FIELD_TOL
    assert np.abs(h - g["fields"]).max() <= tol * np.abs(g["fields"]).max()
    s.step(100)
    run_tol = FP64_RUN_TOL if prec == "FP64" else FP32C_RUN_TOL
    assert np.abs(s.get_state(0) - g["s100"]).max() <= run_tol

