"""CPU pins of the oracle's permuting bisection (perm_bisect_class.h:7-133,
perm_bisect_iterative_class.h:7-231, perm_bisect_table_class.h:7-240) and of the path permutation
in the kinetic action, the Sign and the Permutation observables.

Known answer: N non-interacting bosons in the harmonic trap. With the primitive kinetic action and
the trap's per-bead cofactor a (trap_class.h:19), the weight of a path permutation is the product
over its cycles of the partition function of one ring of (cycle length) x M beads, and per Cartesian
direction a ring of n beads gives prod_j (2 - 2 cos(2 pi j / n) + c)^(-1/2) = (2 cosh(n theta) - 2)^(-1/2)
with c = 4 lambda tau a = 2 cosh(theta) - 2 (the common per-link normalisation cancels). So the
probability of each cycle structure is exact at finite M, and the sampled frequencies must match
within their blocked error bars.
"""
import math

import numpy as np
import pytest

import oracle
from simpimc_gb300.configs import trapped_bosons

BETA, M, OMEGA, LAM = 2.0, 16, 1.0, 0.5


def ring_weight(k):
    tau = BETA / M
    a = 0.5 * tau * OMEGA**2 * (1 + tau**2 * OMEGA**2 / 12)
    theta = math.acosh(1 + 4 * LAM * tau * a / 2)
    return (2 * math.cosh(k * M * theta) - 2) ** -1.5


def exact_sectors(n):
    """Probability of each cycle structure (sorted cycle lengths) of n bosons."""
    def classes(n, maxpart):
        if n == 0:
            yield ()
            return
        for k in range(min(n, maxpart), 0, -1):
            for rest in classes(n - k, k):
                yield (k,) + rest
    w = {}
    for c in classes(n, n):
        # number of permutations with cycle type c: n! / prod(k^m_k m_k!)
        count = math.factorial(n)
        for k in set(c):
            m = c.count(k)
            count //= k**m * math.factorial(m)
        w[tuple(sorted(c))] = count * math.prod(ring_weight(k) for k in c)
    tot = sum(w.values())
    return {k: v / tot for k, v in w.items()}


def cycle_type(pi):
    seen, out = set(), []
    for p in range(len(pi)):
        if p in seen:
            continue
        q, n = p, 0
        while True:
            seen.add(q)
            q = int(pi[q])
            n += 1
            if q == p:
                break
        out.append(n)
    return tuple(sorted(out))


def sample(sim, n, sweeps):
    series = []
    for _ in range(sweeps):
        sim.move_attempts(0, n)
        sim.move_attempts(1, n)
        series.append(cycle_type(sim.get_perm(0, n)))
    return series


def check_frequencies(series, exact, n_blocks=40, z_max=4.5):
    for key, p in exact.items():
        x = np.array([1.0 if s == key else 0.0 for s in series])
        blocks = x[: len(x) // n_blocks * n_blocks].reshape(n_blocks, -1).mean(axis=1)
        err = blocks.std(ddof=1) / math.sqrt(n_blocks)
        z = (x.mean() - p) / max(err, 1e-12)
        assert abs(z) < z_max, (key, x.mean(), p, err)


@pytest.mark.parametrize("perm,n_perm_part", [("PermBisectIterative", 0), ("PermBisectTable", 3)])
def test_oracle_permutation_sectors_exact(tmp_path, perm, n_perm_part):
    n = 3
    xml, path = trapped_bosons(tmp_path, n_part=n, beta=BETA, n_bead=M, n_level=2, perm=perm, n_perm_part=n_perm_part, seed=7)
    c = oracle.OracleSim(xml, base_dir=tmp_path)
    c.set_path(path)
    series = sample(c, n, 60000)
    check_frequencies(series, exact_sectors(n))
    att, acc = c.perm_stats(1, n)
    assert att.sum() > 0 and acc.sum() > 0
    c.close()


def test_oracle_fermion_sign_exact(tmp_path):
    n = 2
    xml, path = trapped_bosons(tmp_path, n_part=n, beta=BETA, n_bead=M, n_level=2, fermi=True, seed=11)
    c = oracle.OracleSim(xml, base_dir=tmp_path)
    c.set_path(path)
    signs = []
    for _ in range(60000):
        c.move_attempts(0, n)
        c.move_attempts(1, n)
        c.observable_accumulate(2)  # Sign
        signs.append(1.0 if cycle_type(c.get_perm(0, n)) == (1, 1) else -1.0)
    block = c.observable_block(2)
    s = np.array(signs)
    assert block[0] == pytest.approx(s.mean(), abs=1e-12)
    ex = exact_sectors(n)
    want = ex[(1, 1)] - ex[(2,)]
    b = s[: len(s) // 40 * 40].reshape(40, -1).mean(axis=1)
    err = b.std(ddof=1) / math.sqrt(40)
    assert abs(s.mean() - want) < 4.5 * err, (s.mean(), want, err)
    c.close()


def test_oracle_kinetic_follows_the_closure(tmp_path):
    """Kinetic dS/dbeta, virial term, segment action and gradient with a permuted closure, against
    a direct evaluation along the permuted rings."""
    n = 4
    xml, path = trapped_bosons(tmp_path, n_part=n, beta=BETA, n_bead=M, n_level=2, seed=3)
    c = oracle.OracleSim(xml, base_dir=tmp_path)
    c.set_path(path)
    pi = np.array([2, 0, 1, 3])
    c.set_perm(0, pi)
    tau = BETA / M
    i4 = 1.0 / (4 * LAM * tau)

    def bead(p, t):  # bead t steps after (p, 0) along the permuted links
        while t >= M:
            p, t = pi[p], t - M
        return path[p, t]

    want = n * M * 3 / (2 * tau)
    for p in range(n):
        for b in range(M):
            want -= np.sum((bead(p, b) - bead(p, b + 1)) ** 2) * i4 / tau
    assert c.dactiondbeta(0) == pytest.approx(want, rel=1e-12)
    # segment crossing the closure, level 0 and level 1
    for level in (0, 1):
        skip = 1 << level
        want = sum(np.sum((bead(1, t) - bead(1, t + skip)) ** 2) * i4 / skip for t in range(M - 4, M + 4, skip))
        assert c.get_action(0, M - 4, M + 4, [(0, 1)], level, 0) == pytest.approx(want, rel=1e-12)
    # gradient at bead 0 of particle 0: previous bead is (pi^-1(0), M - 1)
    inv = np.argsort(pi)
    g = 2 * i4 * ((path[0, 0] - path[inv[0], M - 1]) + (path[0, 0] - path[0, 1]))
    np.testing.assert_allclose(c.get_action_gradient(0, 0, 1, [(0, 0)], 0, 0), g, rtol=1e-12, atol=1e-12)
    # virial window: sum over starts of (window displacement) . (first link)
    W = M
    tot = n * M * 3 / (2 * tau) / W
    for p in range(n):
        for b in range(M):
            d1 = bead(p, b + 1) - bead(p, b)
            dl = bead(p, b + W) - bead(p, b)
            tot -= np.dot(dl, d1) * i4 / (W * tau)
    assert c.virial_energy(0, W) == pytest.approx(tot, rel=1e-10)
    c.close()


def test_oracle_permutation_observable_sectors(tmp_path):
    """Sector numbers follow the ascending-composition order of the partitions of N."""
    n = 5
    xml, path = trapped_bosons(tmp_path, n_part=n, beta=BETA, n_bead=M, n_level=2, seed=5)
    c = oracle.OracleSim(xml, base_dir=tmp_path)
    c.set_path(path)

    def partitions(n, lo=1):
        if n == 0:
            yield ()
            return
        for k in range(lo, n + 1):
            for rest in partitions(n - k, k):
                yield (k,) + rest
    order = sorted(partitions(n))  # ascending compositions in lexicographic order
    for pi in ([0, 1, 2, 3, 4], [1, 0, 2, 3, 4], [1, 2, 0, 4, 3], [1, 2, 3, 4, 0]):
        c.set_perm(0, pi)
        c.observable_accumulate(1)
        blk = c.observable_block(1)
        ct = cycle_type(pi)
        hist = np.zeros(n)
        for k in ct:
            hist[k - 1] += 1
        np.testing.assert_allclose(blk[:n], hist / hist.sum())
        assert blk[n] == order.index(ct) and blk[n + 1] == 1
    c.close()
