"""CPU pins of the oracle's IlkkaPairAction (ilkka_pair_action_class.h:7-433) against an independent
restatement built on scipy's natural cubic splines.

The 2-D table spline of the reference (einspline NUBspline_2d_d with natural conditions) is the
tensor product of natural cubic splines. Here it is evaluated as scipy natural splines along x
within every grid row, then a natural spline along y through those values; the oracle's own
construction is separate C++ code. The checks cover GetAction (short range, and the Ewald part
against densities summed in numpy), the analytic gradient against central differences of the same
scipy action, DActionDBeta and Potential.
"""
import math

import numpy as np
import pytest

import oracle
from simpimc_gb300.configs import electron_gas, trapped_coulomb
from simpimc_gb300.tables import ilkka_table

scipy_interp = pytest.importorskip("scipy.interpolate")


class Spline2:
    """Natural bicubic spline through f[i, j] = f(x_i, y_j), extended by the edge cubics."""

    def __init__(self, x, y, f):
        self.x, self.y = np.asarray(x), np.asarray(y)
        self.rows = [scipy_interp.CubicSpline(self.x, f[:, j], bc_type="natural", extrapolate=True) for j in range(len(self.y))]

    def __call__(self, xx, yy):
        col = np.array([r(xx) for r in self.rows])
        return float(scipy_interp.CubicSpline(self.y, col, bc_type="natural", extrapolate=True)(yy))


class Spline1:
    """Natural cubic spline with the reference's clamp of the argument to the grid (SetLimits)."""

    def __init__(self, x, y):
        self.lo, self.hi = x[0], x[-1]
        self.s = scipy_interp.CubicSpline(x, y, bc_type="natural")

    def __call__(self, r):
        return float(self.s(min(max(r, self.lo), self.hi)))


def tables(ds):
    n = int(ds["u/off_diag/n_x"])
    g = ds["u/off_diag/x"]
    u = Spline2(g, g, np.asarray(ds["u/off_diag/u_xy"]).reshape(n, n))
    du = Spline2(g, g, np.asarray(ds["du/off_diag/du_xy"]).reshape(n, n))
    return u, du


def dr_drp_drrp(a0, c0, a1, c1, L):
    """Path::DrDrpDrrp (path_class.h:137-150): r second minus first particle, r' nearest r."""
    il = 1.0 / L if L > 0 else 0.0
    r = a0 - c0
    rp = a1 - c1
    r = r - np.rint(r * il) * L
    rp = rp + np.rint((r - rp) * il) * L
    s = r - rp
    s = s - np.rint(s * il) * L
    return np.linalg.norm(r), np.linalg.norm(rp), np.linalg.norm(s)


def link_u(u, ulr, r, rp, s):
    q = 0.5 * (r + rp)
    val = u(q + 0.5 * s, q - 0.5 * s)
    if ulr is not None:
        val -= 0.5 * ulr(r) + 0.5 * ulr(rp)
    return val


@pytest.fixture(scope="module")
def trap(tmp_path_factory):
    d = tmp_path_factory.mktemp("ilkka_trap")
    xml, path = trapped_coulomb(d, n_part=5, n_bead=16, n_level=2, seed=3, pair="IlkkaPairAction")
    ds = ilkka_table(d / "check.pat", tau=2.0 / 16, lam=0.5, z_ab=1.0, L=0.0)
    c = oracle.OracleSim(xml, base_dir=d)
    c.set_path(path)
    yield c, path, ds
    c.close()


def test_oracle_ilkka_action_matches_scipy(trap):
    c, path, ds = trap
    u, du = tables(ds)
    a = 2  # Kinetic, Trap, Coulomb
    N, M, _ = path.shape
    for p, b0, b1 in [(0, 0, 4), (3, 13, 17), (4, 5, 9)]:
        want = 0.0
        for b in range(b0, b1):
            for q in range(N):
                if q == p:
                    continue
                # pairs (p, q): r = r_q - r_p
                r, rp, s = dr_drp_drrp(path[q, b % M], path[p, b % M], path[q, (b + 1) % M], path[p, (b + 1) % M], 0.0)
                want += link_u(u, None, r, rp, s)
        got = c.get_action(a, b0, b1, [(0, p)], 0, 0)
        assert abs(got - want) <= 1e-12 * max(1.0, abs(want)), (p, b0, got, want)


def test_oracle_ilkka_gradient_matches_differences(trap):
    c, path, ds = trap
    u, du = tables(ds)
    N, M, _ = path.shape
    p, b = 2, 7

    def action_of(x):
        pth = path.copy()
        pth[p, b] = x
        tot = 0.0
        for bo in ((b + 1) % M, (b - 1) % M):
            for q in range(N):
                if q == p:
                    continue
                r, rp, s = dr_drp_drrp(pth[q, b], pth[p, b], pth[q, bo], pth[p, bo], 0.0)
                tot += link_u(u, None, r, rp, s)
        return tot

    h = 1e-5
    fd = np.zeros(3)
    for d in range(3):
        e = np.zeros(3)
        e[d] = h
        fd[d] = (action_of(path[p, b] + e) - action_of(path[p, b] - e)) / (2 * h)
    g = c.get_action_gradient(2, b, b + 1, [(0, p)], 0, 0)
    np.testing.assert_allclose(g, fd, rtol=1e-6, atol=1e-8)


def test_oracle_ilkka_dbeta_and_potential(trap):
    c, path, ds = trap
    u, du = tables(ds)
    v = Spline1(ds["v/diag/r"], ds["v/diag/v_r"])
    N, M, _ = path.shape
    want_du = want_v = 0.0
    for p in range(N - 1):
        for q in range(p + 1, N):
            for b in range(M):
                r, rp, s = dr_drp_drrp(path[q, b], path[p, b], path[q, (b + 1) % M], path[p, (b + 1) % M], 0.0)
                want_du += link_u(du, None, r, rp, s)
                want_v += 0.5 * v(r) + 0.5 * v(rp)
    assert abs(c.dactiondbeta(2) - want_du) <= 1e-11 * abs(want_du)
    assert abs(c.potential(2) - want_v) <= 1e-11 * abs(want_v)


def test_oracle_ilkka_ewald_action(tmp_path):
    xml, path = electron_gas(tmp_path, n_part=6, n_bead=8, n_level=2, rs=2.0, k_cut_units=3.0, seed=8, pair="IlkkaPairAction")
    L = (4.0 * math.pi * 6 / 3.0) ** (1.0 / 3.0) * 2.0
    k_cut = 3.0 * 2.0 * math.pi / L
    rng = np.random.default_rng(4)
    path = rng.uniform(-L / 2, L / 2, size=path.shape)
    ds = ilkka_table(tmp_path / "check.pat", tau=8.0 / 8, lam=0.5, z_ab=1.0, L=L, k_cut=k_cut)
    u, _ = tables(ds)
    ulr = Spline1(ds["u/diag/r_long"], ds["u/diag/u_long_r"])
    c = oracle.OracleSim(xml, base_dir=tmp_path)
    c.set_path(path)
    kv = c.kvecs()
    kmag = np.linalg.norm(kv, axis=1)
    ktab, utab = np.asarray(ds["u/diag/k"]), np.asarray(ds["u/diag/u_long_k"])
    uk = np.array([utab[np.argmin(np.abs(ktab - m))] if np.min(np.abs(ktab - m)) < 1e-8 else 0.0 for m in kmag])
    up = path[:3]  # species eU: particles 0..2
    M = path.shape[1]
    rho = np.exp(1j * np.einsum("kd,pbd->pbk", kv, up)).sum(axis=0)  # [M][K]
    p, b0, b1 = 1, 2, 6
    want = 0.0
    for b in range(b0, b1):
        for q in range(3):
            if q == p:
                continue
            r, rp, s = dr_drp_drrp(up[q, b % M], up[p, b % M], up[q, (b + 1) % M], up[p, (b + 1) % M], L)
            want += link_u(u, ulr, r, rp, s)
    want += sum(float(np.sum(uk * np.abs(rho[b % M]) ** 2)) for b in range(b0, b1))
    got = c.get_action(2, b0, b1, [(0, p)], 0, 0)  # KineticU, KineticD, then CoulombUU
    assert abs(got - want) <= 1e-10 * max(1.0, abs(want)), (got, want)
    c.close()


def test_oracle_ilkka_levels_use_stride(tmp_path):
    """max_level 1: the level-1 action sums links of stride 2 with the one table; level 2 is zero
    (pair_action_class.h:267-291; ilkka_pair_action_class.h:77-101 takes no level)."""
    xml, path = trapped_coulomb(tmp_path, n_part=5, n_bead=16, n_level=3, seed=7, pair="IlkkaPairAction", pair_max_level=1)
    ds = ilkka_table(tmp_path / "check.pat", tau=2.0 / 16, lam=0.5, z_ab=1.0, L=0.0)
    u, _ = tables(ds)
    c = oracle.OracleSim(xml, base_dir=tmp_path)
    c.set_path(path)
    N, M, _ = path.shape
    for level in (0, 1):
        skip = 1 << level
        for p, b0, b1 in [(2, 0, 8), (4, 10, 18)]:
            want = 0.0
            for b in range(b0, b1, skip):
                for q in range(N):
                    if q != p:
                        want += link_u(u, None, *dr_drp_drrp(path[q, b % M], path[p, b % M], path[q, (b + skip) % M],
                                                             path[p, (b + skip) % M], 0.0))
            got = c.get_action(2, b0, b1, [(0, p)], level, 0)
            assert abs(got - want) <= 1e-12 * max(1.0, abs(want)), (level, p, got, want)
    assert c.get_action(2, 0, 8, [(0, 2)], 2, 0) == 0.0
    c.close()
