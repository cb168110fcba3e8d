"""Error bars of correlated Monte Carlo series (the reference's scripts/Stats.cpp, corrected).

The reference estimates the autocorrelation time kappa = 1 + 2 sum_t C(t), summing the
normalised autocorrelation C(t) until it first drops to zero or below, and the error of the mean
as sqrt(var / (N / kappa)) (Stats.cpp:43-80). Its C(t) pairs x[i] with x[N - t - i] instead of
x[i + t] (Stats.cpp:48), which is not an autocorrelation; here C(t) pairs x[i] with x[i + t].
Flyvbjerg-Petersen blocking is provided as an independent estimate of the same error.
"""
from __future__ import annotations

import math

import numpy as np

__all__ = ["autocorrelation", "kappa", "stats", "unweighted_avg", "blocking_error"]


def autocorrelation(x, t: int, mean: float | None = None, var: float | None = None) -> float:
    """C(t) = sum_{i < N-t} (x_i - mean)(x_{i+t} - mean) / (var (N - t)) (Stats.cpp:43-51)."""
    x = np.asarray(x, dtype=np.float64)
    n = x.size
    mean = float(x.mean()) if mean is None else mean
    var = float(np.mean(x * x) - mean * mean) if var is None else var
    if var == 0.0 or t >= n:
        return 0.0
    return float(np.dot(x[: n - t] - mean, x[t:] - mean) / (var * (n - t)))


def kappa(x) -> float:
    """Autocorrelation time 1 + 2 sum_{t >= 1} C(t), summed while C(t) > 0 (Stats.cpp:53-64)."""
    x = np.asarray(x, dtype=np.float64)
    mean = float(x.mean())
    var = float(np.mean(x * x) - mean * mean)
    tot = 0.0
    for t in range(1, x.size):
        c = autocorrelation(x, t, mean, var)
        if c <= 0.0:
            break
        tot += c
    return 1.0 + 2.0 * tot


def stats(x):
    """(mean, error of the mean, kappa) of a correlated series (Stats.cpp:74-83)."""
    x = np.asarray(x, dtype=np.float64)
    mean = float(x.mean())
    var = float(np.mean(x * x) - mean * mean)
    k = kappa(x)
    n_eff = x.size / k
    return mean, math.sqrt(max(var, 0.0) / n_eff), k


def unweighted_avg(means, errors, kappas):
    """Combination of independent runs (Stats.cpp:66-72): mean of the means, root-mean-square of
    the errors divided by the number of runs, mean kappa."""
    means, errors, kappas = (np.asarray(v, dtype=np.float64) for v in (means, errors, kappas))
    return float(means.mean()), float(math.sqrt(np.sum(errors * errors)) / errors.size), float(kappas.mean())


def blocking_error(x) -> float:
    """Standard error of the mean by Flyvbjerg-Petersen blocking: the largest naive error over the
    halving levels that keep at least 16 blocks."""
    x = np.asarray(x, dtype=np.float64)
    best = 0.0
    while x.size >= 16:
        best = max(best, float(np.std(x, ddof=1) / math.sqrt(x.size)))
        n = x.size // 2
        x = 0.5 * (x[0:2 * n:2] + x[1:2 * n:2])
    return best
