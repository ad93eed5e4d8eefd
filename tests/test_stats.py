"""CPU tests of the error-bar estimators."""
import math

import numpy as np

from jams_gb300 import stats


def test_nse_of_white_noise_is_sigma_over_root_n():
    rng = np.random.default_rng(3)
    x = rng.normal(0.0, 2.0, 40000)
    assert abs(stats.num_std_err(x) / (2.0 / math.sqrt(x.size)) - 1.0) < 0.15


def test_nse_of_ar1_process_includes_autocorrelation():
    """AR(1) with coefficient phi: the variance of the mean is
    sigma_e^2 / (1 - phi)^2 / n."""
    rng = np.random.default_rng(4)
    phi, n = 0.9, 200000
    e = rng.normal(size=n)
    x = np.empty(n)
    x[0] = 0.0
    for k in range(1, n):
        x[k] = phi * x[k - 1] + e[k]
    expect = 1.0 / (1.0 - phi) / math.sqrt(n)
    assert abs(stats.num_std_err(x) / expect - 1.0) < 0.25


def test_geweke_flags_a_drift():
    rng = np.random.default_rng(5)
    x = rng.normal(size=5000)
    d0, _ = stats.geweke(x)
    assert abs(d0) < 4
    d1, _ = stats.geweke(x + np.linspace(0, 3, x.size))
    assert abs(d1) > 4


def test_langevin_function():
    assert abs(stats.langevin(1e-6) - 1e-6 / 3) < 1e-15
    assert abs(stats.langevin(1.0) - (1 / math.tanh(1.0) - 1.0)) < 1e-15
