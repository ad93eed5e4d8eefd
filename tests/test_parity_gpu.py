"""Parity of the sm_103a kernels (through the C ABI) with the oracle and with
the golden vectors produced by the reference's own CPU solver.

Tolerances:
  FP64 form   bit-exact (max |dS| == 0) against the reference / oracle
  FP32C form  max |dS| <= 1e-5 after 1000 T = 0 steps (benchmark bound);
              fields within 2e-6 relative to the field scale
"""
import os

import numpy as np
import pytest

from jams_gb300 import workloads as W
from tests.golden.cases import cases, pulse_cases

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FP32C_TOL = 1e-5


def solver(llg, w, precision, **kw):
    return llg.Solver(w, precision=precision, **kw)


@pytest.mark.parametrize("name", sorted(cases().keys()))
def test_fp64_equals_reference_golden_vectors(llg, name):
    w = cases()[name]
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    s = solver(llg, w, llg.FP64)
    s.set_state(g["s0"])
    assert np.array_equal(s.fields(0), g["fields"])
    done = 0
    for k in (1, 10, 100):
        s.step(k - done)
        done = k
        got = s.get_state(0)
        assert np.array_equal(got, g["s%d" % k]), "max |dS| = %g after %d steps" % (
            np.abs(got - g["s%d" % k]).max(), k)
    s.synchronize()


@pytest.mark.parametrize("name", sorted(cases().keys()))
def test_term_fields_equal_the_reference_hamiltonians_fields(llg, name):
    """llg_term_fields: each term's field as the reference's
    Hamiltonian::calculate_fields leaves it in field_ (FP64: bit for bit;
    FP32C: within 2e-6 of the field scale); the terms add up to llg_fields."""
    w = cases()[name]
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    ref = g["term_fields"]
    for prec in (llg.FP64, llg.FP32C):
        s = solver(llg, w, prec)
        s.set_state(g["s0"])
        got = np.stack([s.term_fields(t, 0) for t in range(len(w.model.terms))])
        if prec == llg.FP64:
            assert np.array_equal(got, ref)
            total = got[0].copy()
            for t in range(1, len(got)):
                total = total + got[t]
            assert np.array_equal(total, s.fields(0))
        else:
            scale = np.abs(ref).max()
            assert np.abs(got - ref).max() <= 2e-6 * scale
        s.close()


@pytest.mark.parametrize("T", [0.0, 300.0])
def test_fp64_heun_bcc_equals_oracle(llg, oracle, T):
    w = W.bcc_three_shell(L=8, T=T, start="random")
    s0 = W.initial_state(w, 0)
    ref = oracle.OracleSim(w).run(s0, 60)
    s = solver(llg, w, llg.FP64, steps_per_graph=16)
    s.set_state(s0)
    s.step(60)
    assert np.array_equal(s.get_state(0), ref)


@pytest.mark.parametrize("T", [0.0, 5.0])
def test_fp64_rk4_triangular_dmi_equals_oracle(llg, oracle, T):
    w = W.triangular_dmi_field_sweep(L=16, n_fields=1, T=T)
    w.replicas[0].B = (0.0, 0.0, 1.0)
    s0 = W.initial_state(w, 0)
    ref = oracle.OracleSim(w).run(s0, 40)
    s = solver(llg, w, llg.FP64)
    s.set_state(s0)
    s.step(40)
    assert np.array_equal(s.get_state(0), ref)


def test_fp32c_sc32_1000_steps_within_bound(llg, oracle):
    """Simple-cubic 32^3, T = 0, 1000 Heun steps (the CPU-runnable workload
    at full size): FP32C max |dS| <= 1e-5 against the FP64 oracle."""
    w = W.sc_ferromagnet(L=32, steps=1000)
    s0 = W.initial_state(w, 0)
    ref = oracle.OracleSim(w).run(s0, 1000)
    s = solver(llg, w, llg.FP32C)
    s.set_state(s0)
    s.step(1000)
    got = s.get_state(0)
    d = np.abs(got - ref).max()
    assert d <= FP32C_TOL, d
    m_ref = oracle.OracleSim(w).magnetisation(ref)
    m_got, _ = s.observables(0)
    assert np.abs(m_got - m_ref).max() < 1e-6


def test_fp32c_bcc_three_shell_1000_steps_within_bound(llg, oracle):
    w = W.bcc_three_shell(L=16, T=0.0, start="random")
    s0 = W.initial_state(w, 0)
    ref = oracle.OracleSim(w).run(s0, 1000)
    s = solver(llg, w, llg.FP32C)
    s.set_state(s0)
    s.step(1000)
    d = np.abs(s.get_state(0) - ref).max()
    assert d <= FP32C_TOL, d


@pytest.mark.parametrize("normalise", [False, True])
def test_fp32c_rk4_triangular_within_bound(llg, oracle, normalise):
    w = W.triangular_dmi_field_sweep(L=64, n_fields=1, T=0.0)
    w.replicas[0].B = (0.0, 0.0, 1.0)
    s0 = W.initial_state(w, 0)
    ref = oracle.OracleSim(w).run(s0, 1000)
    s = solver(llg, w, llg.FP32C, rk4_normalise_stages=normalise)
    s.set_state(s0)
    s.step(1000)
    d = np.abs(s.get_state(0) - ref).max()
    assert d <= FP32C_TOL, d


@pytest.mark.parametrize("name", sorted(cases().keys()))
def test_fp32c_fields(llg, name):
    w = cases()[name]
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    s = solver(llg, w, llg.FP32C)
    s.set_state(g["s0"])
    h = s.fields(0)
    scale = np.abs(g["fields"]).max()
    assert np.abs(h - g["fields"]).max() <= 2e-6 * scale


@pytest.mark.parametrize("precision", ["FP64", "FP32C"])
def test_observables_match_oracle(llg, oracle, precision):
    for name, w in cases().items():
        g = np.load(os.path.join(GOLDEN, name + ".npz"))
        s = solver(llg, w, getattr(llg, precision))
        s.set_state(g["s0"])
        m, e = s.observables(0)
        state = s.get_state(0)
        o = oracle.OracleSim(w)
        tol = 1e-12 if precision == "FP64" else 1e-6
        np.testing.assert_allclose(m, o.magnetisation(state), rtol=tol, atol=tol)
        np.testing.assert_allclose(e, o.energies(state), rtol=tol, atol=tol * np.abs(o.energies(state)).max())


@pytest.mark.parametrize("precision", ["FP64", "FP32C"])
def test_batched_replicas_equal_separate_runs(llg, precision):
    """Replicas of uneven size and temperature in one handle evolve exactly as
    they do alone (the replica index is part of the noise counter)."""
    w = W.sc_temperature_sweep(n_replicas=5, L_min=4, L_max=9, T_max=400.0, steps=50)
    p = getattr(llg, precision)
    batch = solver(llg, w, p, steps_per_graph=10)
    starts = [W.initial_state(w, r) for r in range(5)]
    for r in range(5):
        batch.set_state(starts[r], r)
    batch.step(30)
    for r in range(5):
        single = W.Workload(name="one", model=w.model, replicas=[w.replicas[r]], steps=30, seed=w.seed)
        # the replica index enters the noise counter: run the replica alone at
        # its batch position by padding with empty-temperature copies
        pad = W.Workload(name="pad", model=w.model, replicas=w.replicas[: r + 1], steps=30, seed=w.seed)
        s1 = solver(llg, pad, p, steps_per_graph=10)
        s1.set_state(starts[r], r)
        s1.step(30)
        assert np.array_equal(batch.get_state(r), s1.get_state(r))
        del single


@pytest.mark.parametrize("precision", ["FP64", "FP32C"])
def test_graph_and_direct_launches_agree(llg, precision):
    w = W.bcc_three_shell(L=6, T=200.0, start="random")
    s0 = W.initial_state(w, 0)
    p = getattr(llg, precision)
    a = solver(llg, w, p, steps_per_graph=8)
    b = solver(llg, w, p, steps_per_graph=1)
    for x in (a, b):
        x.set_state(s0)
        x.step(13)
        x.step(7)
    assert a.iteration == b.iteration == 20
    assert np.array_equal(a.get_state(0), b.get_state(0))


def test_resume_from_state_and_iteration(llg):
    """A run split at step 10 (state read back, new handle, iteration set)
    continues the noise stream exactly."""
    w = W.bcc_three_shell(L=6, T=300.0, start="random")
    s0 = W.initial_state(w, 0)
    a = solver(llg, w, llg.FP64)
    a.set_state(s0)
    a.step(20)
    b = solver(llg, w, llg.FP64)
    b.set_state(s0)
    b.step(10)
    mid = b.get_state(0)
    c = solver(llg, w, llg.FP64)
    c.set_state(mid)
    c.set_iteration(10)
    c.step(10)
    assert np.array_equal(a.get_state(0), c.get_state(0))


def test_nonfinite_spin_is_reported(llg):
    w = W.sc_ferromagnet(L=4)
    s = solver(llg, w, llg.FP32C)
    st = W.initial_state(w, 0)
    st[5] = np.nan
    s.set_state(st)
    s.step(2)
    with pytest.raises(llg.LLGError, match="NONFINITE"):
        s.synchronize()


def test_undamped_energy_drift_is_small(llg):
    """alpha = 0, T = 0: Heun conserves the energy to O(dt^2) per unit time."""
    w = W.sc_ferromagnet(L=16, alpha=0.0)
    s = solver(llg, w, llg.FP32C)
    s.set_state(W.initial_state(w, 0))
    _, e0 = s.observables(0)
    s.step(500)
    _, e1 = s.observables(0)
    assert abs(e1.sum() - e0.sum()) < 1e-3 * abs(e0.sum())


def test_topological_charge_matches_oracle(llg, oracle):
    w = W.triangular_dmi_field_sweep(L=32, n_fields=1, T=0.0)
    s0 = W.initial_state(w, 0)
    s = solver(llg, w, llg.FP64)
    s.set_state(s0)
    q = s.topological_charge(0)
    assert abs(q - oracle.topological_charge_triangular(s0, 32, 32)) < 1e-10


def test_tiled_families_selected(llg):
    """FP32C picks the tiled kernel of the matching lattice family; FP64 and
    templates outside the families use the gather kernels."""
    cases_ = [(W.sc_ferromagnet(L=8), "sc"), (W.bcc_nearest_neighbour(L=4), "bcc"),
              (W.bcc_three_shell(L=4), "bcc3"), (W.triangular_dmi_field_sweep(L=8, n_fields=1), "triangular"),
              (W.fcc_ferromagnet(L=4), "fcc"), (W.fcc_ferromagnet(L=4, J2=0.2), "fcc2")]
    for w, fam in cases_:
        assert solver(llg, w, llg.FP32C).kernel_info()["family"] == fam
        assert solver(llg, w, llg.FP64).kernel_info()["family"] == "generic"


def _split_exchange(w):
    """The same Hamiltonian with the exchange as two terms, the second with a
    small symmetric off-diagonal part: no tiled family applies (gather
    kernels)."""
    return W.split_exchange(w, offdiag=0.05)


def test_exchange_terms_are_summed_into_one_stencil(llg):
    """Two half-strength exchange terms run the tiled kernels of the
    family; their sum is exact, so the FP32C states equal the single-term
    run's bit for bit."""
    w = W.bcc_three_shell(L=8, T=300.0, start="random")
    w2 = W.split_exchange(w)
    s0 = W.initial_state(w, 0)
    out = []
    for m in (w, w2):
        s = solver(llg, m, llg.FP32C)
        assert s.kernel_info()["family"] == "bcc3"
        s.set_state(s0)
        s.step(50)
        out.append(s.get_state(0))
    assert np.array_equal(out[0], out[1])


def test_fp32c_gather_kernels_within_bound(llg, oracle):
    w = _split_exchange(W.bcc_three_shell(L=12, T=0.0, start="random"))
    s0 = W.initial_state(w, 0)
    ref = oracle.OracleSim(w).run(s0, 1000)
    s = solver(llg, w, llg.FP32C)
    assert s.kernel_info()["family"] == "generic"
    s.set_state(s0)
    s.step(1000)
    assert np.abs(s.get_state(0) - ref).max() <= FP32C_TOL


@pytest.mark.parametrize("name", ["bcc3", "sc", "tri", "fcc2"])
def test_tiling_choices_give_identical_results(llg, name):
    """Planes per CTA and stored vs recomputed rhs(s0) change the schedule,
    not the arithmetic: states are bit-identical.  Odd plane counts are
    rounded up to even (the noise of two planes comes from one draw); the
    narrow tile exists for simple cubic (elsewhere the flag is ignored); two
    rows per thread exist for all but the triangular family (the odd row
    counts leave one row of a pair outside the lattice)."""
    w = {"bcc3": W.bcc_three_shell(L=10, T=300.0, start="random"),
         "sc": W.sc_ferromagnet(L=(9, 12, 40), T=100.0),
         "tri": W.triangular_dmi_field_sweep(L=(20, 300, 1), n_fields=2, T=5.0),
         "fcc2": W.fcc_ferromagnet(L=(6, 5, 66), T=300.0, J2=0.2, start="random")}[name]
    if name == "tri":
        w.model.integrator = W.HEUN
    if name == "sc":
        w.replicas[0].L = (9, 13, 40)
    outs = []
    choices = [(1, False, 2, False, False), (1, True, 4, False, False), (3, False, 4, False, False),
               (4, True, 3, False, False), (8, True, 2, False, False), (64, False, 2, False, False),
               (2, True, 4, True, False), (6, False, 3, True, False), (64, True, 2, True, False)]
    choices = [c + (False,) for c in choices]
    if name != "tri":
        choices += [(2, False, 2, False, True, False), (4, True, 2, False, True, False),
                    (64, True, 2, False, True, False)]
        # the fused step (wide and narrow tiles, both occupancy variants)
        choices += [(2, False, 2, False, False, True), (4, False, 4, True, False, True),
                    (6, False, 4, False, False, True), (64, False, 2, True, False, True)]
    choices = [c + (False,) for c in choices]
    if name != "tri" and len(w.replicas) == 1:
        # planes loaded by TMA: stored and recomputed rhs, one and two rows
        choices += [(2, True, 4, False, False, False, True), (4, False, 2, False, False, False, True),
                    (6, True, 3, True, False, False, True), (4, True, 2, False, True, False, True),
                    (64, True, 2, False, False, False, True)]
    choices = [c + (False,) for c in choices]
    # stored noise (stored-rhs mode): one and two rows, a narrow tile, TMA
    choices += [(2, True, 4, False, False, False, False, True), (8, True, 2, False, False, False, False, True),
                (4, True, 3, True, False, False, False, True)]
    if name != "tri":
        choices += [(4, True, 2, False, True, False, False, True)]
        if len(w.replicas) == 1:
            choices += [(6, True, 4, False, False, False, True, True)]
    choices = [c + (False,) for c in choices]
    if name == "sc":
        # the half-width tile (16 cells along z): one and two rows, stored
        # or recomputed rhs, stored noise, every occupancy
        choices += [(2, False, 2, False, False, False, False, False, True),
                    (4, True, 3, False, False, False, False, False, True),
                    (6, True, 4, False, False, False, False, True, True),
                    (4, False, 2, False, True, False, False, False, True),
                    (64, True, 2, False, True, False, False, True, True)]
    for tx, store, occ, narrow, pair, fused, tma, noise, half in choices:
        s = solver(llg, w, llg.FP32C, steps_per_graph=4)
        s.set_tuning(tx, store, occ, narrow, pair, fused, tma, noise, half)
        assert s.kernel_info()["rows_per_thread"] == (2 if pair else 1)
        assert s.kernel_info()["fused"] == fused
        assert s.kernel_info()["tma"] == tma
        assert s.kernel_info()["stored_noise"] == noise
        assert (s.kernel_info()["tile_z"] == 16) == half
        for r in range(len(w.replicas)):
            s.set_state(W.initial_state(w, r), r)
        s.step(11)
        outs.append(s.get_state(-1))
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])


def _periodic(w, per):
    w.model.periodic = per
    return w


FUSED_CASES = {
    # ragged z (33 = 32 + 1) and y tiles
    "sc_ragged": lambda: W.sc_ferromagnet(L=(5, 7, 33), T=100.0),
    # open along x, and along y and z
    "sc_open_x": lambda: W.sc_ferromagnet(L=(6, 9, 35), T=100.0, periodic=(0, 1, 1)),
    "sc_open_yz": lambda: W.sc_ferromagnet(L=(7, 5, 9), T=50.0, periodic=(1, 0, 0)),
    # periodic axes shorter than the tile and its halo (the halo wraps more than once)
    "bcc_tiny": lambda: W.bcc_nearest_neighbour(L=(4, 3, 3), T=500.0, start="random"),
    "bcc3_open_z": lambda: _periodic(W.bcc_three_shell(L=(6, 9, 35), T=300.0, start="random"), (1, 1, 0)),
    "bcc3_odd_x": lambda: W.bcc_three_shell(L=(9, 8, 40), T=300.0, start="random"),
    "fcc_ragged": lambda: W.fcc_ferromagnet(L=(3, 5, 66), T=300.0, start="random"),
    "fcc2_open_y": lambda: _periodic(W.fcc_ferromagnet(L=(4, 6, 33), T=300.0, J2=0.2, start="random"), (1, 0, 1)),
    # a time-dependent applied field and zeeman ac field (stage times)
    "bcc_pulse": lambda: pulse_cases()["bcc4_sinc_zeeman_dc_ac"],
}


@pytest.mark.parametrize("name", sorted(FUSED_CASES))
def test_fused_step_equals_the_two_pass_step(llg, name):
    """The fused Heun step (predictor of tile + halo in shared memory, then
    the corrector in the same sweep) gives the stage kernels' states bit for
    bit: the same operations per spin, the same Philox noise for the halo
    cells, at open and periodic boundaries, ragged tiles and lattices smaller
    than a tile."""
    w = FUSED_CASES[name]()
    ref = solver(llg, w, llg.FP32C, steps_per_graph=4)
    assert ref.kernel_info()["family"] != "generic"
    ref.set_tuning(4, True, 2)
    for r in range(len(w.replicas)):
        ref.set_state(W.initial_state(w, r), r)
    ref.step(9)
    want = ref.get_state(-1)
    for tx, occ, narrow in ((2, 2, False), (4, 4, True), (64, 2, False)):
        s = solver(llg, w, llg.FP32C, steps_per_graph=4)
        s.set_tuning(tx, False, occ, narrow, False, True)
        assert s.kernel_info()["fused"]
        for r in range(len(w.replicas)):
            s.set_state(W.initial_state(w, r), r)
        s.step(9)
        got = s.get_state(-1)
        assert np.array_equal(got, want), (tx, occ, narrow, np.abs(got - want).max())
        s.step(1)
        assert s.last_launch_count == 1   # one kernel per step, which also advances the step counter
        s.close()


# TMA rows: the contiguous row (z cells x basis sites) a multiple of 16 bytes
TMA_CASES = {
    "sc_ragged": lambda: W.sc_ferromagnet(L=(5, 7, 36), T=100.0),
    "sc_open_x": lambda: W.sc_ferromagnet(L=(6, 9, 40), T=100.0, periodic=(0, 1, 1)),
    "sc_open_yz": lambda: W.sc_ferromagnet(L=(7, 5, 12), T=50.0, periodic=(1, 0, 0)),
    "bcc_tiny": lambda: W.bcc_nearest_neighbour(L=(4, 3, 4), T=500.0, start="random"),
    "bcc3_open_z": lambda: _periodic(W.bcc_three_shell(L=(6, 9, 34), T=300.0, start="random"), (1, 1, 0)),
    "bcc3_odd_x": lambda: W.bcc_three_shell(L=(9, 8, 40), T=300.0, start="random"),
    "fcc_ragged": lambda: W.fcc_ferromagnet(L=(3, 5, 66), T=300.0, start="random"),
    "fcc2_open_y": lambda: _periodic(W.fcc_ferromagnet(L=(4, 6, 33), T=300.0, J2=0.2, start="random"), (1, 0, 1)),
    "bcc_pulse": lambda: pulse_cases()["bcc4_sinc_zeeman_dc_ac"],
}


@pytest.mark.parametrize("name", sorted(TMA_CASES))
def test_tma_plane_loads_equal_register_staging(llg, name):
    """The stage kernels with planes loaded by TMA box loads (zeros outside
    open boundaries, periodic images read from global memory) give the
    register-staged kernels' states bit for bit, Heun and RK4."""
    w = TMA_CASES[name]()
    for integ in (W.HEUN, W.RK4):
        w.model.integrator = integ
        outs = []
        for tma in (False, True):
            for tx, store, occ in ((2, True, 4), (4, False, 2), (64, True, 2)):
                s = solver(llg, w, llg.FP32C, steps_per_graph=4)
                s.set_tuning(tx, store, occ, False, False, False, tma)
                s.set_state(W.initial_state(w, 0), 0)
                s.step(9)
                outs.append(s.get_state(0))
                s.close()
        for o in outs[1:]:
            assert np.array_equal(o, outs[0]), np.abs(o - outs[0]).max()


def test_tma_is_refused_where_unsupported(llg):
    sweep = W.sc_temperature_sweep(n_replicas=2, L_min=8, L_max=8)
    s = solver(llg, sweep, llg.FP32C)
    with pytest.raises(llg.LLGError, match="one replica"):
        s.set_tuning(4, True, 2, False, False, False, True)
    tri = W.triangular_dmi_field_sweep(L=(20, 30, 1), n_fields=1, T=5.0)
    t = solver(llg, tri, llg.FP32C)
    with pytest.raises(llg.LLGError, match="TMA"):
        t.set_tuning(4, True, 2, False, False, False, True)
    odd = solver(llg, W.sc_ferromagnet(L=(6, 5, 9)), llg.FP32C)   # rows of 9 floats: 36 bytes
    with pytest.raises(llg.LLGError, match="multiple of 16"):
        odd.set_tuning(4, True, 2, False, False, False, True)


def test_fused_step_is_refused_where_unsupported(llg):
    tri = W.triangular_dmi_field_sweep(L=(20, 30, 1), n_fields=1, T=5.0)
    s = solver(llg, tri, llg.FP32C)
    with pytest.raises(llg.LLGError, match="fused step"):
        s.set_tuning(4, False, 2, False, False, True)
    sc = solver(llg, W.sc_ferromagnet(L=16), llg.FP32C)
    with pytest.raises(llg.LLGError, match="fused step"):
        sc.set_tuning(4, True, 2, False, False, True)


@pytest.mark.parametrize("pair", [False, True])
def test_stored_noise_with_replicas_at_zero_kelvin(llg, pair):
    """Stored noise on a handle whose replicas sit above and at 0 K: the
    predictor writes the thermal field of the warm replicas only, and the
    host keeps the cold replicas' planes at zero, also after a replica is
    cooled to 0 K between steps.  Both forms give the same states."""
    w = W.bcc_three_shell(L=8, T=300.0, start="random")
    w.replicas = [W.Replica(L=(8, 8, 8), temperature=300.0), W.Replica(L=(8, 8, 8), temperature=0.0),
                  W.Replica(L=(6, 8, 10), temperature=150.0)]
    outs = []
    for noise in (False, True):
        s = solver(llg, w, llg.FP32C, steps_per_graph=4)
        s.set_tuning(4, True, 2, pair=pair, noise=noise)
        assert s.kernel_info()["stored_noise"] == noise
        for r in range(len(w.replicas)):
            s.set_state(W.initial_state(w, r), r)
        s.step(6)
        s.set_temperature(0, 0.0)
        s.step(5)
        s.set_temperature(1, 80.0)
        s.step(3)
        outs.append([s.get_state(r) for r in range(len(w.replicas))])
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


def test_half_width_tile_on_replicas_of_uneven_sizes(llg):
    """The half-width simple-cubic tile on a batch of replicas whose z
    extents are not multiples of 16 or 32, open and periodic: the same
    states as the 32-cell tile."""
    w = W.sc_ferromagnet(L=16, T=200.0)
    w.replicas = [W.Replica(L=(17, 19, 23), temperature=200.0), W.Replica(L=(16, 16, 16), temperature=0.0),
                  W.Replica(L=(9, 40, 41), temperature=600.0)]
    outs = []
    for half in (False, True):
        for pair in (False, True):
            s = solver(llg, w, llg.FP32C, steps_per_graph=4)
            s.set_tuning(4, True, 2, pair=pair, half_z=half)
            for r in range(len(w.replicas)):
                s.set_state(W.initial_state(w, r), r)
            s.step(9)
            outs.append(s.get_state(-1))
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])
    w.model.periodic = (1, 0, 0)
    outs = []
    for half in (False, True):
        s = solver(llg, w, llg.FP32C, steps_per_graph=4)
        s.set_tuning(2, False, 4, half_z=half)
        for r in range(len(w.replicas)):
            s.set_state(W.initial_state(w, r), r)
        s.step(7)
        outs.append(s.get_state(-1))
    assert np.array_equal(outs[0], outs[1])


def test_half_width_tile_is_refused_where_unsupported(llg):
    s = solver(llg, W.bcc_nearest_neighbour(L=8, T=300.0), llg.FP32C)
    with pytest.raises(llg.LLGError, match="half-width tile"):
        s.set_tuning(4, True, 2, half_z=True)
    s = solver(llg, W.sc_ferromagnet(L=(8, 8, 40), T=10.0), llg.FP32C)
    for kw in ({"narrow": True}, {"fused": True, "store_rhs": False}, {"tma": True}):
        with pytest.raises(llg.LLGError, match="half-width tile"):
            args = dict(store_rhs=True, occupancy=2)
            args.update(kw)
            s.set_tuning(4, half_z=True, **args)


def test_stored_noise_needs_stored_rhs_mode(llg):
    s = solver(llg, W.bcc_nearest_neighbour(L=8, T=300.0), llg.FP32C)
    with pytest.raises(llg.LLGError, match="stored noise"):
        s.set_tuning(4, False, 2, noise=True)
    with pytest.raises(llg.LLGError, match="stored noise"):
        s.set_tuning(4, False, 2, fused=True, noise=True)
    s.set_tuning(4, True, 2, noise=True)
    assert s.kernel_info()["stored_noise"]


def test_two_rows_per_thread_is_refused_where_unsupported(llg):
    tri = W.triangular_dmi_field_sweep(L=(20, 30, 1), n_fields=1, T=5.0)
    s = solver(llg, tri, llg.FP32C)
    with pytest.raises(llg.LLGError, match="two rows per thread"):
        s.set_tuning(4, False, 2, False, True)
    sc = solver(llg, W.sc_ferromagnet(L=16), llg.FP32C)
    with pytest.raises(llg.LLGError, match="two rows per thread"):
        sc.set_tuning(4, False, 2, True, True)
    sc.set_tuning(4, True, 4, False, True)   # occupancy 4 runs as 2
    assert sc.kernel_info()["occupancy"] == 2


def test_autotune_keeps_state_and_iteration(llg):
    w = W.bcc_three_shell(L=8, T=300.0, start="random")
    s0 = W.initial_state(w, 0)
    a = solver(llg, w, llg.FP32C)
    a.set_state(s0)
    a.step(5)
    before = a.get_state(0)
    info = a.autotune(trial_steps=3)
    assert info["family"] == "bcc3" and info["planes_per_cta"] >= 1
    assert a.iteration == 5
    assert np.array_equal(a.get_state(0), before)
    a.step(7)
    b = solver(llg, w, llg.FP32C)
    b.set_state(s0)
    b.step(12)
    assert np.array_equal(a.get_state(0), b.get_state(0))


@pytest.mark.parametrize("J2", [None, 0.2])
def test_fcc_families_match_oracle(llg, oracle, J2):
    """fcc (4-site cell, 12 + 6 neighbours): FP64 bit for bit and FP32C within
    bound against the oracle after 1000 T = 0 steps."""
    w = W.fcc_ferromagnet(L=(5, 6, 7), T=0.0, J2=J2, start="random")
    s0 = W.initial_state(w, 0)
    ref = oracle.OracleSim(w).run(s0, 1000)
    s = solver(llg, w, llg.FP32C)
    assert s.kernel_info()["family"] == ("fcc" if J2 is None else "fcc2")
    s.set_state(s0)
    s.step(1000)
    assert np.abs(s.get_state(0) - ref).max() <= FP32C_TOL
    d = solver(llg, w, llg.FP64)
    d.set_state(s0)
    d.step(1000)
    assert np.array_equal(d.get_state(0), ref)



@pytest.mark.parametrize("prec", ["FP64", "FP32C"])
def test_magnetisation_by_material_and_position(llg, prec):
    """The reference monitor's groupings (magnetisation.cc:20-104): per basis
    position, per material (here two materials on the fcc cell's four sites),
    and none; normalised by sum mu_s or in Bohr magnetons."""
    w = W.fcc_ferromagnet(L=(3, 4, 5), T=0.0, start="random")
    w.model.mus = np.array([2.0, 1.5, 1.5, 2.0]) * W.K_BOHR_MAGNETON_IU
    s = solver(llg, w, getattr(llg, prec))
    s0 = W.initial_state(w, 0)
    s.set_state(s0)
    s.step(3)
    st = s.get_state(0)
    nb = w.model.nb
    mus = np.tile(w.model.mus, len(st) // nb)
    ms = st * mus[:, None]

    def want(groups, normalize):
        out = []
        for g in range(max(groups) + 1):
            sel = np.isin(np.arange(len(st)) % nb, [b for b in range(nb) if groups[b] == g])
            v = ms[sel].sum(axis=0)
            f = 1.0 / mus[sel].sum() if normalize else 1.0 / W.K_BOHR_MAGNETON_IU
            out.append(np.concatenate([v * f, [np.linalg.norm(v) * f]]))
        return np.array(out)

    for groups in ([0, 1, 2, 3], [0, 1, 1, 0], [0, 0, 0, 0]):
        for normalize in (True, False):
            got = s.magnetisation_groups(groups, normalize=normalize)
            np.testing.assert_allclose(got, want(groups, normalize), rtol=1e-12, atol=1e-12)
    m4, _ = s.observables(0)
    np.testing.assert_allclose(s.magnetisation_groups([0, 0, 0, 0])[0], m4, rtol=1e-13, atol=1e-15)
    import ctypes

    g = np.array([0, 1, 2, 5], dtype=np.int32)
    out = np.empty(12)
    rc = s.L.llg_magnetisation_groups(s.h, 0, g.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), 3, 1,
                                      out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert rc < 0 and "outside" in s.L.llg_last_error(s.h).decode()
