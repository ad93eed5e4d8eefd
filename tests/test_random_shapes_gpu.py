"""Randomised lattice shapes: every stencil family on random extents (down
to a single cell along an axis) with random open / periodic axes.  The FP64
form equals the oracle bit for bit; the FP32C form stays within its bound;
tiling variants agree bit for bit.  Seeded, so a failure reproduces."""
import numpy as np
import pytest

from jams_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FAMILIES = ["sc", "bcc", "bcc3", "fcc2", "tri"]


def make(name, L, periodic, seed):
    if name == "sc":
        w = W.sc_ferromagnet(L=L, seed=seed)
    elif name == "bcc":
        w = W.bcc_nearest_neighbour(L=L, T=0.0, start="random", seed=seed)
    elif name == "bcc3":
        w = W.bcc_three_shell(L=L, T=0.0, start="random", seed=seed)
    elif name == "fcc2":
        w = W.fcc_ferromagnet(L=L, T=0.0, J2=0.2, start="random", seed=seed)
    else:
        w = W.triangular_dmi_field_sweep(L=(L[0], L[1], 1), n_fields=1, T=0.0, seed=seed)
        w.model.integrator = W.HEUN
        periodic = (periodic[0], periodic[1], 1)
    w.model.periodic = tuple(periodic)
    return w


def cases(n=40):
    rng = np.random.default_rng(20261204)
    out = []
    for k in range(n):
        name = FAMILIES[k % len(FAMILIES)]
        L = tuple(int(v) for v in rng.integers(1, 12, size=3))
        periodic = tuple(int(v) for v in rng.integers(0, 2, size=3))
        out.append((name, L, periodic, k))
    return out


@pytest.mark.parametrize("name,L,periodic,seed", cases())
def test_random_shape(llg, oracle, name, L, periodic, seed):
    w = make(name, L, periodic, seed)
    try:
        ref_sim = oracle.OracleSim(w)
    except RuntimeError as e:   # e.g. a pair reached twice on a tiny periodic lattice
        with pytest.raises(llg.LLGError):
            llg.Solver(w, precision=llg.FP64)
        pytest.skip("rejected by both: %s" % e)
    s0 = W.initial_state(w, 0)
    ref = ref_sim.run(s0, 12)
    a = llg.Solver(w, precision=llg.FP64, steps_per_graph=4)
    a.set_state(s0)
    a.step(12)
    assert np.array_equal(a.get_state(0), ref)
    outs = []
    for tx, store, occ in [(2, True, 4), (6, False, 2)]:
        b = llg.Solver(w, precision=llg.FP32C, steps_per_graph=4)
        b.set_tuning(tx, store, occ)
        b.set_state(s0)
        b.step(12)
        outs.append(b.get_state(0))
    assert np.abs(outs[0] - ref).max() <= 1e-5
    assert np.array_equal(outs[0], outs[1])
