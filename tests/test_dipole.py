"""CPU tests of the dipole-dipole term: the oracle's restatement of the sum
the reference's FFT term convolves (dipole_fft.cc, dipole_bruteforce.cc)
against known answers and an independent all-pairs sum, and the config
front end's dipole modules."""
import math

import numpy as np
import pytest

from jams_gb300 import configs as C
from jams_gb300 import workloads as W

MU0_IU = 4.0 * math.pi * 1e-7 / 6.24150907e21   # src/jams/helpers/consts.h:38


def random_spins(n, seed):
    s = np.random.default_rng(seed).normal(size=(n, 3))
    return s / np.linalg.norm(s, axis=1)[:, None]


def dipole_only(w):
    w.model.terms = [t for t in w.model.terms if t.kind == W.TERM_DIPOLE]
    return w


def all_pairs_field(w, s, rc):
    """Direct sum over every pair closer than rc (minimum image along the
    periodic axes), written independently of the oracle."""
    m = w.model
    L = np.array(w.replicas[0].L)
    per = np.array(m.periodic, dtype=bool)
    cells = np.stack(np.meshgrid(*[np.arange(n) for n in L], indexing="ij"), -1).reshape(-1, 3)
    pos = (cells[:, None, :] + m.basis_frac[None, :, :]).reshape(-1, 3)
    A = np.asarray(m.cell, dtype=np.float64).T           # rows a1, a2, a3
    a = next(t for t in m.terms if t.kind == W.TERM_DIPOLE).lattice_parameter
    w0 = MU0_IU / (4.0 * math.pi * a ** 3)
    mus = np.tile(m.mus, len(cells))
    h = np.zeros_like(s)
    for i in range(len(pos)):
        x = pos - pos[i]
        x[:, per] -= L[per] * np.floor(x[:, per] / L[per] + 0.5)
        r = x @ A
        r2 = (r * r).sum(1)
        keep = (r2 > 0) & (r2 <= rc * rc)
        rr, r2k, sj = r[keep], r2[keep], s[keep]
        t = (3.0 * rr * (sj * rr).sum(1)[:, None] - r2k[:, None] * sj) / (np.sqrt(r2k) ** 5)[:, None]
        h[i] = mus[i] * w0 * (mus[keep][:, None] * t).sum(0)
    return h


def test_uniform_cubic_lattice_has_no_dipole_field(oracle):
    """A uniformly magnetised simple-cubic lattice summed over a cubic-
    symmetric (spherical) cutoff: the dipole field vanishes."""
    w = dipole_only(W.sc_ferromagnet(L=8, dipole_cutoff=3.5))
    s = np.tile([0.3, 0.4, math.sqrt(0.75)], (512, 1))
    h = oracle.OracleSim(w, 0).fields(s)
    assert np.abs(h).max() < 1e-15


def test_two_spins_known_answer(oracle):
    """Two moments a lattice parameter apart along x, both along x:
    h = mu^2 mu0 / (4 pi a^3) * 2 (along x) on each."""
    w = dipole_only(W.sc_ferromagnet(L=(2, 1, 1), periodic=(0, 0, 0), dipole_cutoff=1.5))
    s = np.array([[1.0, 0.0, 0.0], [1.0, 0.0, 0.0]])
    sim = oracle.OracleSim(w, 0)
    h = sim.fields(s)
    mu = w.model.mus[0]
    expect = mu * mu * MU0_IU / (4.0 * math.pi * 3.0e-10 ** 3) * 2.0
    np.testing.assert_allclose(h[:, 0], expect, rtol=1e-14)
    assert np.abs(h[:, 1:]).max() == 0.0
    e = sim.energies(s)
    np.testing.assert_allclose(e[0], -0.5 * 2 * expect, rtol=1e-14)


@pytest.mark.parametrize("case", ["bcc_periodic", "sc_film", "triangular"])
def test_oracle_equals_all_pairs_sum(oracle, case):
    if case == "bcc_periodic":
        w, rc = W.bcc_three_shell(L=(5, 6, 7), dipole_cutoff=2.4, start="random"), 2.4
    elif case == "sc_film":
        w, rc = W.sc_ferromagnet(L=(6, 5, 3), periodic=(1, 1, 0), dipole_cutoff=2.2), 2.2
    else:
        w, rc = W.triangular_dmi_field_sweep(L=(8, 9, 1), n_fields=1, dipole_cutoff=3.1), 3.1
    w = dipole_only(w)
    n = int(np.prod(w.replicas[0].L)) * w.model.nb
    s = random_spins(n, 7)
    h = oracle.OracleSim(w, 0).fields(s)
    ref = all_pairs_field(w, s, rc + 1e-4)
    assert np.abs(h - ref).max() <= 1e-13 * np.abs(ref).max()


def test_cutoff_beyond_inradius_is_rejected(oracle):
    w = W.sc_ferromagnet(L=6, dipole_cutoff=3.5)
    with pytest.raises(RuntimeError, match="inradius"):
        oracle.OracleSim(w, 0)


def test_config_dipole_module(llg):
    d = llg.describe_config(C.bcc_three_shell(L=8, dipole_cutoff=2.5))
    t = d["terms"][-1]
    assert t["module"] == "dipole-fft" and t["kind"] == W.TERM_DIPOLE
    assert t["dipole"] == [2.5, 1e-4, 2.87e-10]
    assert t["lattice_vectors"] == [1, 0, 0, 0, 1, 0, 0, 0, 1]
    assert t["positions"] == [0, 0, 0, 0.5, 0.5, 0.5]
    with pytest.raises(llg.LLGError, match="r_cutoff"):
        llg.describe_config(C.bcc_three_shell(L=8).replace(
            '{ module = "cubic";', '{ module = "dipole-fft"; },\n  { module = "cubic";'))
