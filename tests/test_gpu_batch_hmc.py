"""Batched hybrid Monte Carlo ("batched + adjoint") against the FP64 oracle's HMC move.

Every chain of the batch has, besides its Bisect move, the library's whole-path HMC move (Gaussian
momenta, leapfrog on S(R) + |P|^2/2 with the exact gradient of the kinetic, trap and bare Coulomb
action, Metropolis on dH). The batch computes it in FP32 with double-float energy sums; the oracle
restates it in FP64 with the same counter-based draws. The tests replay both: identical accept counts
and positions within 1e-4 (FP32 positions, as the batched bisection tests), bisection sweeps
interleaved, and the graph-replayed measurement cycle with HMC attempts equal to the same calls
made one by one.
"""
import numpy as np
import pytest

from simpimc_gb300 import ChainBatch
from simpimc_gb300.configs import trapped_coulomb

pytestmark = pytest.mark.gpu

SHAPES = [(5, 16, 2), (17, 32, 3), (33, 64, 3), (64, 32, 2), (40, 128, 3)]


def _items(tmp_path, hmc=(0.03, 10)):
    out = []
    for c, (n, m, lvl) in enumerate(SHAPES):
        xml, p = trapped_coulomb(tmp_path, n_part=n, n_bead=m, n_level=lvl, seed=300 + c, hmc=hmc)
        out.append((xml, np.asarray(p, dtype=np.float32).astype(np.float64)))
    return out


def _batch(tmp_path, items):
    b = ChainBatch([x for x, _ in items], base_dir=tmp_path)
    for c, (_, p) in enumerate(items):
        b.set_path(c, p)
    return b


def test_batch_hmc_replays_oracle(tmp_path, gpu_lib, oracle_mod):
    items = _items(tmp_path)
    b = _batch(tmp_path, items)
    # smooth the N(0, 1) starting paths with bisection sweeps, then alternate HMC and bisection
    schedule = [("sweeps", 10), ("hmc", 6), ("bisect", 40), ("hmc", 6)]
    for kind, n in schedule:
        if kind == "sweeps":
            b.sweeps(n)
        elif kind == "hmc":
            b.hmc_attempts(n)
        else:
            b.attempts(n)
    hatt, hacc = b.hmc_counters()
    batt, bacc = b.counters()
    assert np.all(hatt == 12)
    assert 0 < int(hacc.sum()) < 12 * len(SHAPES)  # the move accepts and rejects
    for c, (xml, p) in enumerate(items):
        o = oracle_mod.OracleSim(xml, base_dir=tmp_path, chain=c)
        o.set_path(p)
        n, m, lvl = SHAPES[c]
        per_sweep = n * ((m + (1 << lvl) - 1) >> lvl)
        for kind, k in schedule:
            if kind == "sweeps":
                o.move_attempts(0, k * per_sweep)
            elif kind == "hmc":
                o.move_attempts(1, k)
            else:
                o.move_attempts(0, k)
        assert int(hacc[c]) == o.move_stats(1)[2], (c, int(hacc[c]), o.move_stats(1))
        assert int(bacc[c]) == o.move_stats(0)[2], (c, int(bacc[c]), o.move_stats(0))
        dp = np.max(np.abs(b.get_path(c) - o.get_path()))
        assert dp < 1e-4, (c, dp)
        o.close()
    b.close()


def test_batch_hmc_cycle_graph_equals_calls(tmp_path, gpu_lib):
    items = _items(tmp_path)
    g = _batch(tmp_path, items)
    s = _batch(tmp_path, items)
    g.set_hmc_per_cycle(2)
    g.run(3, 1)
    for _ in range(3):
        s.sweeps(1)
        s.hmc_attempts(2)
        s.measure()
    for c in range(len(items)):
        assert np.array_equal(g.get_path(c), s.get_path(c)), c
        eg, ng = g.energy(c)
        es, ns = s.energy(c)
        assert ng == ns == 3 and np.array_equal(eg, es)
    assert np.array_equal(g.hmc_counters()[1], s.hmc_counters()[1])
    g.close()
    s.close()


def test_batch_hmc_needs_the_move(tmp_path, gpu_lib):
    from simpimc_gb300 import PimcError
    items = _items(tmp_path, hmc=None)
    b = _batch(tmp_path, items)
    with pytest.raises(PimcError):
        b.hmc_attempts(1)
    b.close()
