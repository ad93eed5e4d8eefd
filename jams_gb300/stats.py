"""Error bars of time series of observables, as the reference computes them.

spectral_density_zero restates Stats::spectral_density_zero
(src/jams/helpers/stats.cc:16-50, after Monahan, "Numerical Methods of
Statistics"): the periodogram of the series, windowed over the first
ceil(sqrt(n)) frequencies above zero; the numerical standard error of the
mean of an autocorrelated series is sqrt(S(0) / n).  geweke restates
Stats::geweke (stats.cc:52-75): mean of the first 10 % against the last
50 %, and the NSE of the last 90 %.
"""
from __future__ import annotations

import math

import numpy as np


def spectral_density_zero(x) -> float:
    x = np.asarray(x, dtype=np.float64)
    n = x.size
    nd = int(math.ceil(math.sqrt(n)))
    X = np.fft.rfft(x)
    p = np.abs(X) ** 2
    s0 = 0.5 * p[1]
    for k in range(nd):
        if k + 1 < p.size:
            s0 += p[k + 1]
    return (2.0 / n) * s0 / float(2 * nd + 1)


def num_std_err(x) -> float:
    """NSE of the mean: sqrt(S(0) / n)."""
    x = np.asarray(x, dtype=np.float64)
    return math.sqrt(spectral_density_zero(x) / x.size)


def geweke(x):
    """(diagnostic, NSE of the last 90 %); infinite for fewer than 100 points."""
    x = np.asarray(x, dtype=np.float64)
    n = x.size
    na, nb = int(0.1 * n), int(0.5 * n)
    if na < 10:
        return math.inf, math.inf
    a, b = x[:na], x[nb:]
    diag = (a.mean() - b.mean()) / math.sqrt(spectral_density_zero(a) / na + spectral_density_zero(b) / b.size)
    return diag, math.sqrt(spectral_density_zero(x[na:]) / (n - na))


def langevin(x: float) -> float:
    """Classical Langevin function coth(x) - 1/x: <S.B>/|B| of a free spin."""
    if abs(x) < 1e-4:
        return x / 3.0
    return 1.0 / math.tanh(x) - 1.0 / x
