"""CPU tests of the oracle: pinned to golden vectors made by the reference
itself, to the Philox4x32-10 known-answer vectors, and to analytic results."""
import math
import os

import numpy as np
import pytest

from jams_gb300 import workloads as W
from tests.golden.cases import cases, dipole_cases, pulse_cases

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("name", sorted(cases().keys()))
def test_oracle_matches_reference_golden_vectors(oracle, name):
    """Fields, energies and 1/10/100-step Heun trajectories of the oracle equal
    the reference's own CPU solver (HeunLLGSolver::run) bit for bit."""
    w = cases()[name]
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    sim = oracle.OracleSim(w)
    s0 = g["s0"]
    assert np.array_equal(sim.fields(s0), g["fields"])
    np.testing.assert_allclose(sim.energies(s0), g["energies"], rtol=1e-13, atol=1e-12)
    s = s0
    done = 0
    for k in (1, 10, 100):
        s = sim.run(s, k - done, first_step=done)
        done = k
        assert np.array_equal(s, g["s%d" % k]), "max |dS| = %g after %d steps" % (np.abs(s - g["s%d" % k]).max(), k)


@pytest.mark.parametrize("name", sorted(pulse_cases().keys()))
def test_oracle_matches_reference_pulse_golden_vectors(oracle, name):
    """Time-dependent applied fields (sinc, sinc-cos pulses) and zeeman dc / ac
    fields at the stage times t0 and t0 + dt of every Heun step: fields,
    energies and trajectories equal the reference's own applied_field.cc and
    zeeman.cc, and so do the fields and energies at the solver time 100 dt."""
    w = pulse_cases()[name]
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    sim = oracle.OracleSim(w)
    s0 = g["s0"]
    assert np.array_equal(sim.fields(s0), g["fields"])
    np.testing.assert_allclose(sim.energies(s0), g["energies"], rtol=1e-13, atol=1e-12)
    s = s0
    done = 0
    for k in (1, 10, 100):
        s = sim.run(s, k - done, first_step=done)
        done = k
        assert np.array_equal(s, g["s%d" % k]), "max |dS| = %g after %d steps" % (np.abs(s - g["s%d" % k]).max(), k)
    assert np.array_equal(sim.fields(s), g["fields100"])
    np.testing.assert_allclose(sim.energies(s), g["energies100"], rtol=1e-13, atol=1e-12)
    assert not np.array_equal(g["fields100"], g["fields"])


def test_oracle_pulse_shapes(oracle):
    """The applied field of one spin follows B sinc(pi f_bw (t - t_c)) and
    B sinc(...) cos(2 pi f_c (t - t_c)); the zeeman field dc + ac cos(2 pi f t)."""
    B = np.array([0.3, -0.2, 1.5])
    tc, fbw, fc, fz = 0.02, 60.0, 90.0, 25.0
    for pulse in (W.PULSE_SINC, W.PULSE_SINC_COS):
        w = W.sc_ferromagnet(L=1, J=0.0, dz=0.0)
        w.model.terms = [W.field_term(B, pulse=pulse, time_center=tc, freq_bandwidth=fbw, freq_center=fc),
                         W.zeeman_term([(0.1, 0.0, 0.2)], [(0.0, 0.4, 0.0)], [fz])]
        sim = oracle.OracleSim(w)
        s = np.array([[0.0, 0.0, 1.0]])
        mus = w.model.mus[0]
        for t in (0.0, 0.013, 0.02, 0.05):
            x = math.pi * fbw * (t - tc)
            f = 1.0 if x == 0.0 else math.sin(x) / x
            if pulse == W.PULSE_SINC_COS:
                f *= math.cos(2 * math.pi * fc * (t - tc))
            want = mus * B * f + mus * (np.array([0.1, 0.0, 0.2]) + np.array([0.0, 0.4, 0.0]) *
                                        math.cos(2 * math.pi * fz * t))
            np.testing.assert_allclose(sim.fields(s, t)[0], want, rtol=1e-12, atol=1e-15)


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(__file__), "..", "oracle", "_ref",
                                                    "libjams_ref.so")),
                    reason="reference build (oracle/_ref) exists only where the reference sources are")
def test_oracle_matches_reference_build_longer_run(oracle):
    w = W.bcc_three_shell(L=6, T=0.0, start="random")
    s0 = W.initial_state(w, 0)
    a = oracle.OracleSim(w).run(s0, 300)
    b = oracle.ReferenceSim(w).run(s0, 300)
    assert np.array_equal(a, b)


def test_philox_known_answers(oracle):
    """Philox4x32-10 known-answer vectors published with Random123 (counter 0,
    key 0 and counter/key all ones), checked through the noise path's raw
    generator: the first normal is a fixed function of the first word pair."""
    import ctypes

    L = oracle.lib()
    # expose the raw generator through the normal transform: rebuild the
    # expected normals from the published words with the same transform
    words_zero = (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)
    z = oracle.noise_normals(0, 0, 0, 0)
    expect = _normals_from_words(words_zero)
    assert np.array_equal(z, expect)
    words_ones = (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)
    z = oracle.noise_normals(0xFFFFFFFFFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFFFFFFFFFF, 0xFFFFFFFF)
    assert np.array_equal(z, _normals_from_words(words_ones))
    del L, ctypes


def _normals_from_words(c):
    """Box-Muller of the oracle, evaluated with numpy float32 (same IEEE
    single-precision operations; fma done in float64 then rounded, which is
    exact for these operand sizes)."""
    f32 = np.float32

    def fma(a, b, cc):
        return f32(np.float64(a) * np.float64(b) + np.float64(cc))

    def nlog(u):
        b = np.array([u], dtype=np.float32).view(np.uint32)[0]
        e = int(b >> 23) - 127
        mb = (int(b) & 0x007FFFFF) | 0x3F800000
        if mb > 0x3FB504F3:
            mb -= 0x00800000
            e += 1
        m = np.array([mb], dtype=np.uint32).view(np.float32)[0]
        f = f32(f32(m - f32(1)) / f32(m + f32(1)))
        f2 = f32(f * f)
        p = f32(float.fromhex("0x1.c71c72p-4"))
        for cst in ("0x1.24924ap-3", "0x1.99999ap-3", "0x1.555556p-2"):
            p = fma(p, f2, f32(float.fromhex(cst)))
        p = fma(p, f2, f32(1))
        lnm = f32(f32(2) * f32(f * p))
        return fma(f32(e), f32(float.fromhex("0x1.62e430p-1")), lnm)

    def sincos(k):
        q = k >> 22
        j = k & 0x3FFFFF
        if j >= (1 << 21):
            q += 1
            j -= 1 << 22
        r = f32(f32(j) * f32(2.0 ** -22))
        r2 = f32(r * r)
        sp = f32(float.fromhex("0x1.507834p-13"))
        for cst in ("-0x1.32d2ccp-8", "0x1.466bc6p-4", "-0x1.4abbcep-1", "0x1.921fb6p+0"):
            sp = fma(sp, r2, f32(float.fromhex(cst)))
        sn = f32(sp * r)
        cp = f32(float.fromhex("0x1.e1f506p-11"))
        for cst in ("-0x1.55d3c8p-6", "0x1.03c1f0p-2", "-0x1.3bd3ccp+0"):
            cp = fma(cp, r2, f32(float.fromhex(cst)))
        cs = fma(cp, r2, f32(1))
        return [(sn, cs), (cs, -sn), (-sn, -cs), (-cs, sn)][q & 3]

    u1 = f32(f32((c[0] >> 8) + 1) * f32(2.0 ** -24))
    u2 = f32(f32((c[2] >> 8) + 1) * f32(2.0 ** -24))
    r1 = f32(np.sqrt(f32(f32(-2) * nlog(u1))))
    r2 = f32(np.sqrt(f32(f32(-2) * nlog(u2))))
    s1, c1 = sincos(c[1] >> 8)
    s2, c2 = sincos(c[3] >> 8)
    return np.array([f32(r1 * c1), f32(r1 * s1), f32(r2 * c2)], dtype=np.float32)


def test_noise_moments(oracle):
    """The normals are N(0,1): mean, variance, kurtosis and tail mass over
    300k draws within 5 standard errors."""
    n = 100_000
    z = np.array([oracle.noise_normals(7, 3, 11, i) for i in range(n)], dtype=np.float64).reshape(-1)
    m = z.size
    assert abs(z.mean()) < 5 / math.sqrt(m)
    assert abs(z.var() - 1.0) < 5 * math.sqrt(2.0 / m)
    k = ((z - z.mean()) ** 4).mean() / z.var() ** 2
    assert abs(k - 3.0) < 5 * math.sqrt(24.0 / m)
    tail = (np.abs(z) > 2.0).mean()
    assert abs(tail - 0.0455003) < 5 * math.sqrt(0.0455 * 0.9545 / m)


def test_uniform_ferromagnet_exchange_field(oracle):
    """Exchange field of a uniform state is sum_j J_ij S (SC: 6 J; bcc: 8 J1 +
    6 J2 + 12 J3)."""
    for w, zj in ((W.sc_ferromagnet(L=4), 6 * 1.0), (W.bcc_three_shell(L=4), 8 * 2.0 + 6 * 1.2 + 12 * -0.1)):
        w.model.terms = w.model.terms[:1]
        sim = oracle.OracleSim(w)
        s = np.zeros((sim.n, 3))
        s[:, 0] = 1.0
        h = sim.fields(s)
        np.testing.assert_allclose(h[:, 0], zj, rtol=1e-14)
        np.testing.assert_allclose(h[:, 1:], 0.0, atol=1e-15)


def test_anisotropy_fields_at_known_angles(oracle):
    """Uniaxial K1: h = 2 K (S.z) z; cubic K1 at S = (1,1,1)/sqrt3:
    h = 2K * (2/3) / sqrt3 * (1,1,1)."""
    w = W.sc_ferromagnet(L=2, dz=0.3)
    w.model.terms = [w.model.terms[1]]
    sim = oracle.OracleSim(w)
    th = 0.7
    s = np.tile([math.sin(th), 0.0, math.cos(th)], (sim.n, 1))
    np.testing.assert_allclose(sim.fields(s)[:, 2], 2 * 0.3 * math.cos(th), rtol=1e-14)
    w = W.bcc_three_shell(L=2)
    w.model.terms = [w.model.terms[1]]
    sim = oracle.OracleSim(w)
    s = np.full((sim.n, 3), 1 / math.sqrt(3))
    np.testing.assert_allclose(sim.fields(s), 2 * 0.005 * (2 / 3) / math.sqrt(3), rtol=1e-13)


def test_single_spin_precession_frequency(oracle):
    """Undamped single spin in B = 1 T z precesses at omega = gamma B: after
    n steps the azimuth advances by gamma B n dt (Heun error O(dt^2))."""
    w = W.sc_ferromagnet(L=1, J=0.0, dz=0.0, alpha=0.0)
    w.model.terms = [w.model.terms[2]]
    sim = oracle.OracleSim(w)
    s0 = np.array([[1.0, 0.0, 0.0]])
    n = 1000
    s = sim.run(s0, n)
    phi = math.atan2(s[0, 1], s[0, 0])
    expect = w.model.gyro[0] * 1.0 * n * w.model.dt  # dS/dt = -gamma S x B: counter-clockwise
    assert abs(math.remainder(phi - expect, 2 * math.pi)) < 1e-6
    assert abs(s[0, 2]) < 1e-14


def test_damped_relaxation_to_field(oracle):
    """With damping a spin relaxes towards +B."""
    w = W.sc_ferromagnet(L=1, J=0.0, dz=0.0, alpha=0.5, B=(0, 0, 10.0))
    w.model.terms = [w.model.terms[2]]
    sim = oracle.OracleSim(w)
    s = sim.run(np.array([[1.0, 0.0, 0.0]]), 20000)
    assert s[0, 2] > 0.999


def test_multiple_interactions_error(oracle):
    """A template that reaches the same site twice is rejected, as the
    reference's neighbour list does (interactions.cc:371-380)."""
    w = W.sc_ferromagnet(L=(2, 4, 4))
    with pytest.raises(RuntimeError, match="Multiple interactions"):
        oracle.OracleSim(w)


def test_topological_charge_of_uniform_and_skyrmion(oracle):
    L = 32
    s = np.zeros((L * L, 3))
    s[:, 2] = 1.0
    assert abs(oracle.topological_charge_triangular(s, L, L)) < 1e-14
    # Belavin-Polyakov-like texture on the triangular lattice: |Q| close to 1
    a1 = np.array([1.0, 0.0])
    a2 = np.array([0.5, math.sqrt(3) / 2])
    c = (L / 2) * (a1 + a2)
    for i in range(L):
        for j in range(L):
            r = i * a1 + j * a2 - c
            rr = math.hypot(*r)
            th = math.pi * math.exp(-rr / 4.0)
            ph = math.atan2(r[1], r[0])
            s[i * L + j] = [math.sin(th) * math.cos(ph), math.sin(th) * math.sin(ph), math.cos(th)]
    q = oracle.topological_charge_triangular(s, L, L)
    assert abs(abs(q) - 1.0) < 0.05


@pytest.mark.parametrize("name", sorted(dipole_cases().keys()))
def test_oracle_dipole_matches_reference_golden_vectors(oracle, name):
    """The dipole fixtures come from the reference's dipole-bruteforce
    Hamiltonian (dipole_bruteforce.cc) compiled from its sources; the oracle's
    direct sum differs from it only in summation order."""
    w = dipole_cases()[name]
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    sim = oracle.OracleSim(w)
    h = sim.fields(g["s0"])
    assert np.abs(h - g["fields"]).max() <= 1e-14 * np.abs(g["fields"]).max()
    np.testing.assert_allclose(sim.energies(g["s0"]), g["energies"], rtol=1e-13, atol=1e-16)
    s = g["s0"]
    done = 0
    for k in (1, 10, 100):
        s = sim.run(s, k - done, first_step=done)
        done = k
        assert np.abs(s - g["s%d" % k]).max() <= 1e-13, k

