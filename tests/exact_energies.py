"""Exact energies of systems the library can run, for statistical checks of whole runs.

exact_sho_energy: one Cartesian degree of freedom in the harmonic trap under the reference's
discretised action (kinetic_class.h, trap_class.h), E = -d ln Z_M / d beta from the circulant
normal modes of the M-slice ring.

free_particle_energy_1d: one free particle on a periodic line of length L at inverse temperature
beta: Z = sum_k exp(-lambda beta k^2), k = 2 pi j / L, so E = <lambda k^2>. The Gaussian link
propagator summed over images is the exact free propagator, so this holds for any M.
"""
import math

import numpy as np


def exact_sho_energy(beta, M, omega, lam=0.5):
    tau = beta / M
    a = 1.0 / (4 * lam * tau)
    c = 0.5 * tau * omega ** 2 * (1 + tau ** 2 * omega ** 2 / 12)
    cb = 0.5 * omega ** 2 * (1 + 3 * tau ** 2 * omega ** 2 / 12)
    s2 = np.sin(np.pi * np.arange(M) / M) ** 2
    mu = 4 * a * s2 + c
    dmu = -4 * s2 / (4 * lam * tau ** 2) + cb
    return 1.0 / (2 * tau) + np.sum(dmu / mu) / (2 * M)


def free_particle_energy_1d(beta, L, lam=0.5, j_max=200):
    j = np.arange(-j_max, j_max + 1)
    e = lam * (2.0 * math.pi * j / L) ** 2
    w = np.exp(-beta * e)
    return float(np.sum(e * w) / np.sum(w))


def blocked_error(x, n_blocks=20):
    x = np.asarray(x)
    nb = len(x) // n_blocks
    means = x[: nb * n_blocks].reshape(n_blocks, nb).mean(axis=1)
    return means.std(ddof=1) / math.sqrt(n_blocks)
