"""Error-bar analysis of correlated series (simpimc_gb300/stats.py) on series with known answers:
i.i.d. normals (kappa = 1) and AR(1) processes x_t = phi x_{t-1} + e_t, whose autocorrelation is
phi^t and whose integrated time is (1 + phi) / (1 - phi)."""
import math

import numpy as np

from simpimc_gb300 import stats


def ar1(phi, n, seed):
    rng = np.random.default_rng(seed)
    e = rng.standard_normal(n)
    x = np.empty(n)
    x[0] = e[0] / math.sqrt(1 - phi * phi)
    for t in range(1, n):
        x[t] = phi * x[t - 1] + e[t]
    return x


def test_autocorrelation_of_ar1_is_phi_to_the_lag():
    x = ar1(0.8, 200000, 1)
    for t in (1, 2, 5):
        assert abs(stats.autocorrelation(x, t) - 0.8 ** t) < 0.02


def test_kappa_and_error_of_known_processes():
    x = np.random.default_rng(2).standard_normal(100000)
    m, err, k = stats.stats(x)
    assert abs(k - 1.0) < 0.05
    assert abs(err - 1.0 / math.sqrt(x.size)) < 0.05 / math.sqrt(x.size)
    phi = 0.9
    x = ar1(phi, 400000, 3)
    m, err, k = stats.stats(x)
    k_true = (1 + phi) / (1 - phi)
    assert abs(k - k_true) < 0.1 * k_true
    # against the exact error sqrt(var kappa / N) of the process, var = 1 / (1 - phi^2)
    exact = math.sqrt(k_true / (1 - phi * phi) / x.size)
    assert abs(err - exact) < 0.1 * exact
    # blocking takes the largest level estimate, so it errs on the high side
    assert exact * 0.9 < stats.blocking_error(x) < exact * 1.3


def test_unweighted_average_of_runs():
    m, e, k = stats.unweighted_avg([1.0, 3.0], [0.3, 0.4], [2.0, 4.0])
    assert m == 2.0 and abs(e - 0.25) < 1e-15 and k == 3.0
