"""Pair-action table files for BarePairAction and IlkkaPairAction (Coulomb, optional Ewald split).

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

__all__ = ["write_table", "read_table", "coulomb_table", "ilkka_table", "david_table", "lattice_k_magnitudes", "ewald_alpha"]


def write_table(path, datasets: dict) -> None:
    """Write ``{dataset path: scalar, 1-D array or string}`` in the table container format."""
    lines = ["# pair-action table: '<dataset> <count>' then the values"]
    for key, val in datasets.items():
        if isinstance(val, str):
            if "\n" in val:
                raise ValueError(f"string dataset {key!r} spans lines")
            lines.append(f"{key} str")
            lines.append(val)
            continue
        arr = np.atleast_1d(np.asarray(val, dtype=np.float64))
        lines.append(f"{key} {arr.size}")
        for i in range(0, arr.size, 4):
            lines.append(" ".join(repr(float(x)) for x in arr[i:i + 4]))
    Path(path).write_text("\n".join(lines) + "\n")


def read_table(path) -> dict:
    """Read a container file: ``{dataset path: 1-D float64 array or string}``."""
    out: dict = {}
    key, want, vals = None, None, []
    lines = Path(path).read_text().splitlines()
    i = 0
    while i < len(lines):
        toks = lines[i].split("#", 1)[0].split()
        i += 1
        if key is None and len(toks) == 2 and toks[1] == "str":
            out[toks[0]] = lines[i] if i < len(lines) else ""
            i += 1
            continue
        for tok in toks:
            if key is None:
                key = tok
            elif want is None:
                want, vals = int(tok), []
            else:
                vals.append(float(tok))
            if key is not None and want is not None and len(vals) == want:
                out[key] = np.asarray(vals, dtype=np.float64)
                key, want, vals = None, None, []
    if key is not None:
        raise ValueError(f"{path}: dataset {key!r} is incomplete")
    return out


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


def _ilkka_grid(x_max: float, n: int) -> np.ndarray:
    """Non-uniform grid on [0, x_max], denser at small distances: x_max t^1.5 for uniform t."""
    t = np.linspace(0.0, 1.0, n)
    return x_max * t ** 1.5


def ilkka_table(path, *, tau: float, lam: float = 0.5, z_ab: float = 1.0, L: float = 0.0, k_cut: float = 0.0,
                n_d: int = 3, n_xy: int = 64, xy_max: float | None = None, alpha: float | None = None) -> dict:
    """Write an IlkkaPairAction table (src/actions/pair_action/ilkka_pair_action_class.h:253-432).

    The reference's tables come from a pair-density squarer that is not part of its repository, so
    this one is synthetic but smooth and of the right shape. The off-diagonal action is the
    end-point average of a Gaussian-smeared Coulomb potential at the two 'extremal' distances,

        u(x, y) = tau [phi(x) + phi(y)] / 2,   phi(r) = z erf(r / a) / r,   a = sqrt(4 lambda tau),

    with x = q + s/2, y = q - s/2, q = (|r| + |r'|) / 2, s = |r - r'|: it equals tau phi(r) on the
    diagonal r = r'. du(x, y) is its tau derivative (a depends on tau). The grids in x and y are
    equal and non-uniform, and u(x, y) = u(y, x), so the matrix storage order (value (i, j) at
    i n_y + j here) cannot change the spline. With ``L > 0`` and ``k_cut > 0`` the long-range parts
    are the Ewald split of BarePairAction's table scaled for the action (u = tau v) and its tau
    derivative (du = v); ``v/diag`` holds the potential datasets as for BarePairAction.
    """
    a = math.sqrt(4.0 * lam * tau)
    if xy_max is None:
        xy_max = math.sqrt(n_d) * L if L > 0 else 20.0
    g = _ilkka_grid(xy_max, n_xy)
    erf = np.vectorize(math.erf)

    def phi(r):
        r = np.asarray(r, dtype=np.float64)
        out = np.empty_like(r)
        small = r < 1e-8
        out[small] = z_ab * 2.0 / (a * math.sqrt(math.pi))
        rr = r[~small]
        out[~small] = z_ab * erf(rr / a) / rr
        return out

    def dphi_da(r):
        r = np.asarray(r, dtype=np.float64)
        return -z_ab * 2.0 / math.sqrt(math.pi) * np.exp(-(r / a) ** 2) / (a * a)

    X, Y = np.meshgrid(g, g, indexing="ij")
    u = tau * 0.5 * (phi(X) + phi(Y))
    # d/dtau [tau Phi(a(tau))] = Phi + tau dPhi/da da/dtau, da/dtau = a / (2 tau)
    du = 0.5 * (phi(X) + phi(Y)) + 0.5 * a * 0.5 * (dphi_da(X) + dphi_da(Y))
    ds = {
        "u/off_diag/n_x": n_xy, "u/off_diag/n_y": n_xy, "u/off_diag/x": g, "u/off_diag/y": g, "u/off_diag/u_xy": u.ravel(),
        "du/off_diag/n_x": n_xy, "du/off_diag/n_y": n_xy, "du/off_diag/x": g, "du/off_diag/y": g, "du/off_diag/du_xy": du.ravel(),
    }
    v = coulomb_table(path, z_ab=z_ab, L=L, k_cut=k_cut, n_d=n_d, alpha=alpha)  # v/diag datasets (file rewritten below)
    ds.update(v)
    if L > 0 and k_cut > 0:
        ds.update({
            "u/diag/n_r_long": v["v/diag/n_r_long"], "u/diag/r_long": v["v/diag/r_long"],
            "u/diag/u_long_r": tau * v["v/diag/v_long_r"], "u/diag/u_long_r_0": tau * v["v/diag/v_long_r_0"],
            "u/diag/n_k": v["v/diag/n_k"], "u/diag/k": v["v/diag/k"],
            "u/diag/u_long_k": tau * v["v/diag/v_long_k"], "u/diag/u_long_k_0": tau * v["v/diag/v_long_k_0"],
            "du/diag/n_r_long": v["v/diag/n_r_long"], "du/diag/r_long": v["v/diag/r_long"],
            "du/diag/du_long_r": v["v/diag/v_long_r"], "du/diag/du_long_r_0": v["v/diag/v_long_r_0"],
            "du/diag/n_k": v["v/diag/n_k"], "du/diag/k": v["v/diag/k"],
            "du/diag/du_long_k": v["v/diag/v_long_k"], "du/diag/du_long_k_0": v["v/diag/v_long_k_0"],
        })
    write_table(path, ds)
    return ds


def david_table(path, *, tau: float, n_order: int = 2, lam: float = 0.5, z_ab: float = 1.0, L: float = 0.0,
                k_cut: float = 0.0, n_d: int = 3, n_grid: int = 200, r_max: float | None = None,
                alpha: float | None = None, n_tau: int = 1) -> dict:
    """Write a DavidPairAction table (src/actions/pair_action/david_pair_action_class.h:190-358).

    The squarer that writes these tables is not part of the reference, so the table is synthetic:
    a smeared Coulomb potential V(r) = z erf(r / a) / r (a = sqrt(4 lambda tau)), the diagonal action
    u_00(r) = tau V(r) + tau^2 w(r) with w(r) = z exp(-r^2 / a^2) / (2 a), and off-diagonal
    coefficients u_kj(q) = tau^k c_kj V(q) / a^(2k) (k = 1..n_order, j = 0..k, c_kj = (-1)^(k+j)
    / (4^k (j + 1))) of the expansion sum_kj u_kj z^(2j) s^(2(k-j)). The beta derivatives are the
    tau derivatives at fixed a, with the potential taken out of the diagonal one as in the
    reference's files (du_00 - V). Datasets, with ``n = n_order``:

    * ``u_kj_n/grid/{start, end, n_grid_points, type, grid_points}``: a general grid, type "GENERAL"
      (the reference also reads LOG, LINEAR and LOGLIN grid types, whose knots the points give);
    * ``u_kj_n/taus``, ``potential/data``;
    * ``u_kj_n/data`` and ``du_kj_dbeta_n/data``: n_val x n_grid x n_tau values, value index
      fastest (Armadillo's cube order), n_val = sum_{i=0..n} (i + 1). Table l is made for the time
      step tau 2^l (the bisection's level l with max_level = n_tau - 1), with the potential of tau;
    * with ``L > 0`` and ``k_cut > 0``: ``long_range/{k_cut, n_k, k_points, u_k}`` (V u_k is the
      k-space Ewald potential, listed with k = 0 for its constant) and ``squarer/v_image``.
    """
    a = math.sqrt(4.0 * lam * tau)
    if r_max is None:
        r_max = math.sqrt(n_d) * L / 2.0 if L > 0 else 20.0
    t = np.linspace(0.0, 1.0, n_grid)
    r = 1.0e-3 + (r_max - 1.0e-3) * t ** 2
    erf = np.vectorize(math.erf)
    V = z_ab * erf(r / a) / r
    w = z_ab * np.exp(-(r / a) ** 2) / (2.0 * a)
    n_val = sum(i + 1 for i in range(n_order + 1))
    us, dus, taus = [], [], []
    for lvl in range(n_tau):
        tl = tau * 2 ** lvl
        al = math.sqrt(4.0 * lam * tl)
        wl = z_ab * np.exp(-(r / al) ** 2) / (2.0 * al)
        u = np.zeros((n_val, n_grid))
        du = np.zeros((n_val, n_grid))
        u[0] = tl * V + tl * tl * wl
        du[0] = 2.0 * tl * wl  # d u_00 / d tau - V
        for k in range(1, n_order + 1):
            for j in range(k + 1):
                c = (-1.0) ** (k + j) / (4.0 ** k * (j + 1))
                idx = k * (k + 1) // 2 + j
                u[idx] = tl ** k * c * V / al ** (2 * k)
                du[idx] = k * tl ** (k - 1) * c * V / al ** (2 * k)
        us.append(u.T.ravel())  # value index fastest
        dus.append(du.T.ravel())
        taus.append(tl)
    pre = f"u_kj_{n_order}"
    ds = {
        f"{pre}/grid/start": r[0], f"{pre}/grid/end": r[-1], f"{pre}/grid/n_grid_points": n_grid, f"{pre}/grid/type": "GENERAL",
        f"{pre}/grid/grid_points": r,
        f"{pre}/taus": tau if n_tau == 1 else np.array(taus), "potential/data": V,
        f"{pre}/data": np.concatenate(us),  # then grid, then tau
        f"du_kj_dbeta_{n_order}/data": np.concatenate(dus),
    }
    if L > 0 and k_cut > 0:
        al = ewald_alpha(L, k_cut) if alpha is None else alpha
        vol = L ** n_d
        k = lattice_k_magnitudes(L, k_cut, n_d)
        uk = z_ab * 4.0 * math.pi * np.exp(-k * k / (4.0 * al * al)) / (k * k)  # divided by V at load
        ds.update({
            "long_range/k_cut": k_cut, "long_range/n_k": k.size + 1,
            "long_range/k_points": np.concatenate([[0.0], k]),
            "long_range/u_k": np.concatenate([[-z_ab * math.pi / (al * al)], uk]),
            "squarer/v_image": z_ab * 2.0 * al / math.sqrt(math.pi),
        })
    write_table(path, ds)
    return ds
