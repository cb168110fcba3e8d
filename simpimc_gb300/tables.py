"""Pair-action table files for BarePairAction (Coulomb with an optional Ewald long-range split).

The reference reads these tables from HDF5 files written by its `pagen` generator (an empty
submodule in the reference repository). This module writes the same datasets
(src/actions/pair_action/bare_pair_action_class.h:39-76) in the plain-text container that
`simpimc_gb300/src/framework/table_io.h` reads:

* ``v/diag/{n_r, r, v_r}``                 pair potential q_a q_b / r on a logarithmic grid;
* ``v/diag/{n_r_long, r_long, v_long_r}``  long-range part q_a q_b erf(alpha r) / r;
* ``v/diag/v_long_r_0``                    its r -> 0 limit, 2 alpha / sqrt(pi) (self term);
* ``v/diag/{n_k, k, v_long_k}``            4 pi q_a q_b exp(-k^2 / 4 alpha^2) / (V k^2) for every
  distinct |k| of the box lattice below k_cut (matched by magnitude at load time);
* ``v/diag/v_long_k_0``                    -pi q_a q_b / (alpha^2 V) (neutralising background).

This is the standard Ewald breakup. With the half-space k-vector sum of CalcVLong it gives
sum_{k in half space} v_long_k |rho_k|^2 = (2 pi / V) sum_{k != 0} exp(-k^2/4a^2) |rho_k|^2 / k^2.
The splitting parameter defaults to alpha = sqrt(k_cut / L), which balances the real-space
error erfc(alpha L/2) against the reciprocal-space error exp(-k_cut^2 / 4 alpha^2).
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np

__all__ = ["write_table", "coulomb_table", "lattice_k_magnitudes", "ewald_alpha"]


def write_table(path, datasets: dict) -> None:
    """Write ``{dataset path: scalar or 1-D array}`` in the table container format."""
    lines = ["# pair-action table: '<dataset> <count>' then the values"]
    for key, val in datasets.items():
        arr = np.atleast_1d(np.asarray(val, dtype=np.float64))
        lines.append(f"{key} {arr.size}")
        for i in range(0, arr.size, 4):
            lines.append(" ".join(repr(float(x)) for x in arr[i:i + 4]))
    Path(path).write_text("\n".join(lines) + "\n")


def lattice_k_magnitudes(L: float, k_cut: float, n_d: int = 3) -> np.ndarray:
    """Distinct |k| of k = 2 pi n / L with 0 < |k| < k_cut (the k-vector set of KSpace::Setup)."""
    box = 2.0 * math.pi / L
    nmax = int(math.ceil(1.1 * k_cut / box))
    rng = np.arange(-nmax, nmax + 1)
    grids = np.meshgrid(*([rng] * n_d), indexing="ij")
    n2 = sum(g.astype(np.int64) ** 2 for g in grids).ravel()
    n2 = np.unique(n2[(n2 > 0)])
    mags = box * np.sqrt(n2.astype(np.float64))
    return mags[mags < k_cut]


def ewald_alpha(L: float, k_cut: float) -> float:
    return math.sqrt(k_cut / L)


def coulomb_table(path, *, z_ab: float = 1.0, L: float = 0.0, k_cut: float = 0.0, n_d: int = 3,
                  r_min: float = 1.0e-4, r_max: float | None = None, n_r: int = 2000,
                  n_r_long: int = 2048, alpha: float | None = None) -> dict:
    """Write a BarePairAction table for the pair potential z_ab / r and return its datasets.

    With ``L > 0`` and ``k_cut > 0`` the long-range Ewald datasets are included as well.
    """
    if r_max is None:
        r_max = math.sqrt(n_d) * L / 2.0 if L > 0 else 100.0
    r = np.geomspace(r_min, r_max, n_r)
    ds = {"v/diag/n_r": n_r, "v/diag/r": r, "v/diag/v_r": z_ab / r}
    if L > 0 and k_cut > 0:
        a = ewald_alpha(L, k_cut) if alpha is None else alpha
        vol = L ** n_d
        rl = np.linspace(r_min, math.sqrt(n_d) * L / 2.0, n_r_long)
        vl = np.array([z_ab * math.erf(a * x) / x for x in rl])
        k = lattice_k_magnitudes(L, k_cut, n_d)
        vk = z_ab * 4.0 * math.pi * np.exp(-k * k / (4.0 * a * a)) / (vol * k * k)
        ds.update({
            "v/diag/n_r_long": n_r_long,
            "v/diag/r_long": rl,
            "v/diag/v_long_r": vl,
            "v/diag/v_long_r_0": z_ab * 2.0 * a / math.sqrt(math.pi),
            "v/diag/n_k": k.size,
            "v/diag/k": k,
            "v/diag/v_long_k": vk,
            "v/diag/v_long_k_0": -z_ab * math.pi / (a * a * vol),
        })
    write_table(path, ds)
    return ds
