"""The bounds-checked build (compiled with LLG_BOUNDS_CHECK, in place of a
memory checker). Every gathered neighbour,
fetched plane, ring slot and written spin index is checked against its array.
A miss would set a status bit that llg_synchronize reports as LLG_ERR_BOUNDS,
and the access would be skipped. Across the kernel forms it must run clean
and give the same spins, fields and energies as the normal build, bit for bit."""

import numpy as np
import pytest

from jams_gb300 import workloads as W
from tests.golden.cases import pulse_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def checked(llg):
    from jams_gb300 import build

    build.build(checked=True)
    return True


def _generic(w):
    # two exchange terms, one with an off-diagonal part: the gather kernels
    return W.split_exchange(w, offdiag=0.05)


def _open_sc():
    w = W.sc_ferromagnet(L=(7, 5, 9), T=50.0)
    w.model.periodic = (0, 1, 0)
    return w


def _tri_rk4():
    return W.triangular_dmi_field_sweep(L=(13, 21, 1), n_fields=2, T=5.0)


CASES = {
    "bcc3_tiled": (lambda: W.bcc_three_shell(L=(5, 6, 7), T=300.0, start="random"), "FP32C", None),
    "bcc3_pair_rows": (lambda: W.bcc_three_shell(L=(5, 6, 7), T=300.0, start="random"), "FP32C", (4, True, 2, False,
                                                                                                  True)),
    "sc_open_narrow": (_open_sc, "FP32C", (2, False, 4, True, False)),
    "tri_rk4": (_tri_rk4, "FP32C", None),
    "fcc2": (lambda: W.fcc_ferromagnet(L=(3, 4, 5), T=300.0, J2=0.2, start="random"), "FP32C", None),
    "bcc3_generic": (lambda: _generic(W.bcc_three_shell(L=5, T=300.0, start="random")), "FP32C", None),
    "bcc3_fp64": (lambda: W.bcc_three_shell(L=5, T=300.0, start="random"), "FP64", None),
    "sc_film_dipole": (lambda: W.sc_ferromagnet(L=(6, 5, 3), periodic=(1, 1, 0), dipole_cutoff=2.2), "FP32C", None),
    "pulse_zeeman": (lambda: pulse_cases()["bcc4_sinc_zeeman_dc_ac"], "FP64", None),
    # the fused Heun step: wide and narrow tiles, open and wrapping halos
    "bcc3_fused": (lambda: W.bcc_three_shell(L=(5, 6, 35), T=300.0, start="random"), "FP32C",
                   (2, False, 2, False, False, True)),
    "sc_open_fused_narrow": (_open_sc, "FP32C", (4, False, 4, True, False, True)),
    "fcc_fused": (lambda: W.fcc_ferromagnet(L=(3, 4, 5), T=300.0, start="random"), "FP32C",
                  (2, False, 2, False, False, True)),
    # planes loaded by TMA: stored rhs, two rows per thread, open axes
    "bcc3_tma": (lambda: W.bcc_three_shell(L=(5, 6, 36), T=300.0, start="random"), "FP32C",
                 (2, True, 4, False, False, False, True)),
    "bcc3_tma_pair": (lambda: W.bcc_three_shell(L=(5, 6, 36), T=300.0, start="random"), "FP32C",
                      (4, True, 2, False, True, False, True)),
    "sc_open_tma": (lambda: W.sc_ferromagnet(L=(7, 5, 12), T=50.0, periodic=(0, 1, 0)), "FP32C",
                    (2, True, 4, True, False, False, True)),
    # the half-width simple-cubic tile: ragged z and y edges, open z, two rows
    "sc_half_open": (lambda: W.sc_ferromagnet(L=(6, 11, 21), T=50.0, periodic=(1, 1, 0)), "FP32C",
                     (4, True, 2, False, True, False, False, True, True)),
    "sc_half": (lambda: W.sc_ferromagnet(L=(5, 9, 35), T=50.0), "FP32C",
                (2, False, 3, False, False, False, False, False, True)),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_checked_build_runs_clean_and_equal(llg, checked, name):
    make, prec, tuning = CASES[name]
    w = make()
    p = getattr(llg, prec)
    sims = []
    for chk in (True, False):   # the checked build first: it skips and reports any access out of range
        s = llg.Solver(w, precision=p, steps_per_graph=4, checked=chk)
        if tuning:
            s.set_tuning(*tuning)
        for r in range(len(w.replicas)):
            s.set_state(W.initial_state(w, r), r)
        s.step(7)
        s.step(5)
        s.synchronize()   # raises LLG_ERR_BOUNDS if any index was out of range
        sims.append(s)
    b, a = sims
    assert np.array_equal(a.get_state(-1), b.get_state(-1))
    assert np.array_equal(a.fields(0), b.fields(0))
    assert np.array_equal(a.observables(0)[1], b.observables(0)[1])
    b.synchronize()
