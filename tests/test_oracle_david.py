"""CPU pins of the oracle's DavidPairAction (david_pair_action_class.h:7-361) against an independent
restatement on scipy's natural cubic splines: the endpoint and off-diagonal expansion of CalcU and
CalcdUdBeta with the reference's clamps (GetLimits), the k-space long-range action, DActionDBeta,
Potential, and the base class's central-difference gradient."""
import math

import numpy as np
import pytest

import oracle
from simpimc_gb300.configs import electron_gas, trapped_coulomb
from simpimc_gb300.tables import david_table

scipy_interp = pytest.importorskip("scipy.interpolate")


class Multi:
    """Component splines of a David table (component 0 the potential), argument clamped to the grid.
    Every component is zero at the last grid point: the reference fills its spline data below that
    point only (david_pair_action_class.h:262-271) and leaves the zero-initialised value there."""

    def __init__(self, ds, key, n_order, level=0):
        g = np.asarray(ds[f"u_kj_{n_order}/grid/grid_points"])
        n_val = sum(i + 1 for i in range(n_order + 1))
        block = len(g) * n_val  # one table per tau: value index fastest, then grid, then tau
        data = np.asarray(ds[key])[level * block:(level + 1) * block].reshape(len(g), n_val)
        cols = [np.asarray(ds["potential/data"], dtype=float).copy()] + [data[:, v].copy() for v in range(n_val)]
        for c in cols:
            c[-1] = 0.0
        self.lo, self.hi = g[0], g[-1]
        self.s = [scipy_interp.CubicSpline(g, c, bc_type="natural") for c in cols]
        self.n_order = n_order

    def __call__(self, comp, x):
        return float(self.s[comp](min(max(x, self.lo), self.hi)))

    def offdiag(self, q, z, s):
        tot = 0.0
        for k in range(1, self.n_order + 1):
            for j in range(k + 1):
                tot += self(k * (k + 1) // 2 + j + 1, q) * z ** (2 * j) * s ** (2 * (k - j))
        return tot


def link(m, r, rp, s, diag_comp, add_v):
    q, z = 0.5 * (r + rp), r - rp
    rc, rpc = min(max(r, m.lo), m.hi), min(max(rp, m.lo), m.hi)
    u = 0.5 * (m(diag_comp, rc) + m(diag_comp, rpc))
    if add_v:
        u += 0.5 * (m(0, rc) + m(0, rpc))
    if s > 0.0 and q < m.hi:
        u += m.offdiag(q, z, s)
    return u


def dists(a0, c0, a1, c1, L):
    il = 1.0 / L if L > 0 else 0.0
    r = a0 - c0
    rp = a1 - c1
    r = r - np.rint(r * il) * L
    rp = rp + np.rint((r - rp) * il) * L
    s = r - rp
    s = s - np.rint(s * il) * L
    return np.linalg.norm(r), np.linalg.norm(rp), np.linalg.norm(s)


@pytest.fixture(scope="module")
def trap(tmp_path_factory):
    d = tmp_path_factory.mktemp("david_trap")
    xml, path = trapped_coulomb(d, n_part=5, n_bead=16, n_level=2, seed=3, pair="DavidPairAction", n_order=2)
    ds = david_table(d / "check.pat", tau=2.0 / 16, n_order=2, lam=0.5, z_ab=1.0, L=0.0)
    c = oracle.OracleSim(xml, base_dir=d)
    c.set_path(path)
    yield c, path, ds
    c.close()


def test_oracle_david_action_and_dbeta(trap):
    c, path, ds = trap
    u = Multi(ds, "u_kj_2/data", 2)
    du = Multi(ds, "du_kj_dbeta_2/data", 2)
    N, M, _ = path.shape
    for p, b0, b1 in [(0, 0, 4), (3, 13, 17)]:
        want = 0.0
        for b in range(b0, b1):
            for q in range(N):
                if q != p:
                    want += link(u, *dists(path[q, b % M], path[p, b % M], path[q, (b + 1) % M], path[p, (b + 1) % M], 0.0), 1, False)
        got = c.get_action(2, b0, b1, [(0, p)], 0, 0)
        assert abs(got - want) <= 1e-12 * max(1.0, abs(want)), (got, want)
    want_du = want_v = 0.0
    for p in range(N - 1):
        for q in range(p + 1, N):
            for b in range(M):
                r, rp, s = dists(path[q, b], path[p, b], path[q, (b + 1) % M], path[p, (b + 1) % M], 0.0)
                want_du += link(du, r, rp, s, 1, True)
                want_v += 0.5 * (u(0, r) + u(0, rp))
    assert abs(c.dactiondbeta(2) - want_du) <= 1e-11 * abs(want_du)
    assert abs(c.potential(2) - want_v) <= 1e-11 * abs(want_v)


def test_oracle_david_gradient_is_central_difference(trap):
    c, path, ds = trap
    u = Multi(ds, "u_kj_2/data", 2)
    N, M, _ = path.shape
    p, b, eps = 2, 7, 1e-4

    def action_of(x):
        pth = path.copy()
        pth[p, b] = x
        tot = 0.0
        for bo in ((b + 1) % M, (b - 1) % M):
            for q in range(N):
                if q != p:
                    tot += link(u, *dists(pth[q, b], pth[p, b], pth[q, bo], pth[p, bo], 0.0), 1, False)
        return tot

    want = np.zeros(3)
    for d in range(3):
        e = np.zeros(3)
        e[d] = eps
        want[d] = (action_of(path[p, b] + e) - action_of(path[p, b] - e)) / (2 * eps)
    got = c.get_action_gradient(2, b, b + 1, [(0, p)], 0, 0)
    np.testing.assert_allclose(got, want, rtol=1e-7, atol=1e-9)


def test_oracle_david_ewald_action(tmp_path):
    xml, path = electron_gas(tmp_path, n_part=6, n_bead=8, n_level=2, rs=2.0, k_cut_units=3.0, seed=8, pair="DavidPairAction",
                             n_order=1)
    L = (4.0 * math.pi * 6 / 3.0) ** (1.0 / 3.0) * 2.0
    k_cut = 3.0 * 2.0 * math.pi / L
    path = np.random.default_rng(4).uniform(-L / 2, L / 2, size=path.shape)
    ds = david_table(tmp_path / "check.pat", tau=8.0 / 8, n_order=1, lam=0.5, z_ab=1.0, L=L, k_cut=k_cut)
    u = Multi(ds, "u_kj_1/data", 1)
    c = oracle.OracleSim(xml, base_dir=tmp_path)
    c.set_path(path)
    kv = c.kvecs()
    kmag = np.linalg.norm(kv, axis=1)
    kt, ut = np.asarray(ds["long_range/k_points"]), np.asarray(ds["long_range/u_k"]) / L ** 3
    uk = np.array([ut[np.argmin(np.abs(kt - m))] for m in kmag]) * (8.0 / 8)
    up = path[:3]
    M = path.shape[1]
    rho = np.exp(1j * np.einsum("kd,pbd->pbk", kv, up)).sum(axis=0)
    p, b0, b1 = 1, 2, 6
    want = 0.0
    for b in range(b0, b1):
        for q in range(3):
            if q != p:
                want += link(u, *dists(up[q, b % M], up[p, b % M], up[q, (b + 1) % M], up[p, (b + 1) % M], L), 1, False)
    want += sum(float(np.sum(uk * np.abs(rho[b % M]) ** 2)) for b in range(b0, b1))
    got = c.get_action(2, b0, b1, [(0, p)], 0, 0)
    assert abs(got - want) <= 1e-10 * max(1.0, abs(want)), (got, want)
    c.close()


def test_oracle_david_level_tables(tmp_path):
    """max_level 2: level l sums links of stride 2^l with the table of index l (u_kj(level)), and the
    action above max_level is zero (pair_action_class.h:267-291, david_pair_action_class.h:63-102)."""
    xml, path = trapped_coulomb(tmp_path, n_part=5, n_bead=16, n_level=3, seed=5, pair="DavidPairAction", n_order=2,
                                pair_max_level=2)
    ds = david_table(tmp_path / "check.pat", tau=2.0 / 16, n_order=2, lam=0.5, z_ab=1.0, L=0.0, n_tau=3)
    c = oracle.OracleSim(xml, base_dir=tmp_path)
    c.set_path(path)
    N, M, _ = path.shape
    seen = []
    for level in range(3):
        u = Multi(ds, "u_kj_2/data", 2, level)
        skip = 1 << level
        for p, b0, b1 in [(1, 0, 8), (4, 12, 20)]:
            want = 0.0
            for b in range(b0, b1, skip):
                for q in range(N):
                    if q != p:
                        want += link(u, *dists(path[q, b % M], path[p, b % M], path[q, (b + skip) % M],
                                               path[p, (b + skip) % M], 0.0), 1, False)
            got = c.get_action(2, b0, b1, [(0, p)], level, 0)
            assert abs(got - want) <= 1e-12 * max(1.0, abs(want)), (level, got, want)
            seen.append(got)
    assert len(set(seen)) == len(seen)
    assert c.get_action(2, 0, 8, [(0, 1)], 3, 0) == 0.0
    c.close()


def test_oracle_david_refuses_missing_level_tables(tmp_path):
    """A table with fewer taus than max_level + 1 is an input error (david_pair_action_class.h:234-246)."""
    xml, _ = trapped_coulomb(tmp_path, n_part=5, n_bead=16, n_level=3, seed=5, pair="DavidPairAction", n_order=2,
                             pair_max_level=2)
    david_table(tmp_path / "david_open_16_2.0_2_2.pat", tau=2.0 / 16, n_order=2, lam=0.5, z_ab=1.0, L=0.0, n_tau=2)
    with pytest.raises(RuntimeError, match="fewer taus"):
        oracle.OracleSim(xml, base_dir=tmp_path)


def test_david_table_levels_layout(tmp_path):
    """n_tau tables for tau 2^l, value index fastest, then grid, then tau; the first block equals the
    one-table file's (the levels share the grid and the potential)."""
    one = david_table(tmp_path / "one.pat", tau=0.125, n_order=2, n_grid=50)
    three = david_table(tmp_path / "three.pat", tau=0.125, n_order=2, n_grid=50, n_tau=3)
    assert np.allclose(three["u_kj_2/taus"], [0.125, 0.25, 0.5])
    n_val = 6
    for key in ("u_kj_2/data", "du_kj_dbeta_2/data"):
        assert len(three[key]) == 3 * 50 * n_val
        assert np.array_equal(three[key][:50 * n_val], one[key])
        assert not np.array_equal(three[key][50 * n_val:100 * n_val], one[key])
    assert np.array_equal(three["potential/data"], one["potential/data"])
