"""Finite-temperature checks of both arithmetic forms on the GPU.

1. Free spins in a field: the time average of S.B/|B| equals the Langevin
   function L(mu_s B / k_B T) (classical Boltzmann distribution), which
   tests the noise amplitude sqrt(2 alpha k_B T / (gamma mu_s dt)).
2. bcc three-shell Hamiltonian with cubic anisotropy at 300 K (the
   benchmark's, on a smaller lattice; paramagnetic at this temperature):
   <|M|> and <E> of the FP32C form agree with the FP64 form within their
   statistical error bars (the spread of independent replicas' averages)."""
import math

import numpy as np
import pytest

from jams_gb300 import stats
from jams_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def sample(s, burn, n, every):
    s.step(burn)
    m_abs, energy = [], []
    for _ in range(n):
        s.step(every)
        m, e = s.observables(0)
        m_abs.append(m[3])
        energy.append(e.sum())
    return np.array(m_abs), np.array(energy)


@pytest.mark.parametrize("gilbert", [True, False])
@pytest.mark.parametrize("precision", ["FP64", "FP32C"])
def test_free_spins_follow_the_langevin_function(llg, precision, gilbert):
    """With gilbert_prefactor the reference's LLG (gamma / (1 + alpha^2),
    noise variance / (1 + alpha^2)) samples the Boltzmann distribution at T;
    without it the Landau-Lifshitz form with the noise in both terms samples
    it at (1 + alpha^2) T.  Both are the reference's conventions
    (src/jams/solvers/cpu_llg_heun.cc:36-43, src/jams/core/lattice.cc:91-97)."""
    T, B, alpha = 10.0, 10.0, 0.5
    w = W.sc_ferromagnet(L=32, J=0.0, dz=0.0, B=(0.0, 0.0, B), alpha=alpha, T=T)
    w.model.terms = [w.model.terms[2]]  # Zeeman only
    w.start = "+z"
    if gilbert:
        w.model.gilbert_prefactor = True
        w.model.gyro = w.model.gyro / (1.0 + alpha * alpha)
    s = llg.Solver(w, precision=getattr(llg, precision))
    s.set_state(W.initial_state(w, 0))
    mz = []
    s.step(6000)
    for _ in range(300):
        s.step(50)
        m, _ = s.observables(0)
        mz.append(m[2])
    mz = np.array(mz)
    t_eff = T if gilbert else T * (1.0 + alpha * alpha)
    expect = stats.langevin(w.model.mus[0] * B / (W.K_BOLTZMANN_IU * t_eff))
    err = stats.num_std_err(mz)
    # time-step bias of the Heun scheme is small here (gamma B dt = 1.8e-3)
    assert abs(mz.mean() - expect) < 4 * err + 2e-3, (mz.mean(), expect, err)


def test_fp32c_equilibrium_matches_fp64_within_error_bars(llg):
    """Eight independent replicas of each form (their noise is keyed by the
    replica), each time-averaged after burn-in; the error bar is the spread
    of the replica averages.  One run's spectral error underestimates it:
    |M| of order 1 / sqrt(N) in the paramagnet drifts over thousands of
    steps."""
    reps = 8

    def batch(seed):
        w = W.bcc_three_shell(L=12, T=300.0, start="+z", seed=seed)
        w.replicas = [W.Replica(L=(12, 12, 12), temperature=300.0) for _ in range(reps)]
        return w

    w64, w32 = batch(11), batch(12)
    a = llg.Solver(w64, precision=llg.FP64)
    b = llg.Solver(w32, precision=llg.FP32C)
    means = []
    for s, w in ((a, w64), (b, w32)):
        for r in range(reps):
            s.set_state(W.initial_state(w, r), r)
        s.step(4000)
        m_abs = np.zeros((200, reps))
        energy = np.zeros((200, reps))
        for k in range(200):
            s.step(20)
            for r in range(reps):
                m, e = s.observables(r)
                m_abs[k, r] = m[3]
                energy[k, r] = e.sum()
        means.append((m_abs.mean(axis=0), energy.mean(axis=0)))
    for xa, xb in zip(means[0], means[1]):
        err = math.sqrt(xa.var(ddof=1) / reps + xb.var(ddof=1) / reps)
        assert abs(xa.mean() - xb.mean()) < 4 * err, (xa.mean(), xb.mean(), err)
    # 300 K is above this Hamiltonian's ordering temperature (mean field:
    # sum_j J_ij / 3 k_B = 85 K): |M| is of order 1/sqrt(N)
    assert means[0][0].mean() < 5.0 / math.sqrt(w64.total_spins / reps)
