"""Batched hybrid Monte Carlo ("batched + adjoint") against the FP64 oracle's HMC move.

Every chain of the batch has, besides its Bisect move, the library's whole-path HMC move (Gaussian
momenta, leapfrog on S(R) + |P|^2/2 with the exact gradient of the kinetic, trap and bare Coulomb
action, Metropolis on dH). The batch computes it in FP32 with double-float energy sums; the oracle
restates it in FP64 with the same counter-based draws. The tests replay both: identical accept counts
and positions within 1e-4 (FP32 positions, as the batched bisection tests), bisection sweeps
interleaved, and the graph-replayed measurement cycle with HMC attempts equal to the same calls
made one by one. A chain runs on a cluster of k thread blocks split by slices; the trajectory is the
same FP32 sequence for every k, so paths and accept counts are identical across k = 1, 2, 4, 8.
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


@pytest.mark.parametrize("k", [1, 8])
def test_batch_hmc_replays_oracle(tmp_path, gpu_lib, oracle_mod, k):
    items = _items(tmp_path)
    b = _batch(tmp_path, items)
    b.hmc_cluster = k
    assert b.hmc_cluster == k
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


@pytest.mark.parametrize("heavy", [0, 2])
def test_batch_hmc_cycle_graph_equals_calls(tmp_path, gpu_lib, heavy):
    """The cycle's graph (with `heavy` > 0: the heaviest chains on one stream beside the others on a
    second) gives the same bits as the same calls made one by one."""
    items = _items(tmp_path)
    g = _batch(tmp_path, items)
    s = _batch(tmp_path, items)
    g.overlap = heavy
    assert g.overlap == heavy
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


def test_batch_hmc_cluster_size_leaves_trajectory_unchanged(tmp_path, gpu_lib):
    items = _items(tmp_path)
    runs = []
    for k in (1, 2, 4, 8):
        b = _batch(tmp_path, items)
        b.hmc_cluster = k
        b.sweeps(5)
        b.hmc_attempts(4)
        b.attempts(20)
        b.hmc_attempts(4)
        runs.append(([b.get_path(c) for c in range(len(items))], b.hmc_counters()[1].copy()))
        b.close()
    for paths, acc in runs[1:]:
        assert np.array_equal(acc, runs[0][1])
        for c in range(len(items)):
            assert np.array_equal(paths[c], runs[0][0][c]), c


def test_batch_hmc_cluster_size_must_divide_n_bead(tmp_path, gpu_lib):
    from simpimc_gb300 import PimcError
    xml_a, pa = trapped_coulomb(tmp_path, n_part=6, n_bead=12, n_level=2, seed=1, hmc=(0.03, 4))
    xml_b, pb = trapped_coulomb(tmp_path, n_part=5, n_bead=16, n_level=2, seed=2, hmc=(0.03, 4))
    b = ChainBatch([xml_a, xml_b], base_dir=tmp_path)
    b.set_path(0, pa)
    b.set_path(1, pb)
    for bad in (3, 16):
        with pytest.raises(PimcError, match="1, 2, 4 or 8"):
            b.hmc_cluster = bad
    with pytest.raises(PimcError, match="divide"):
        b.hmc_cluster = 8  # 12 slices do not split over 8 blocks
    b.hmc_cluster = 4
    b.hmc_attempts(3)
    assert np.all(b.hmc_counters()[0] == 3)
    b.close()


def test_batch_hmc_needs_the_move(tmp_path, gpu_lib):
    from simpimc_gb300 import PimcError
    items = _items(tmp_path, hmc=None)
    b = _batch(tmp_path, items)
    with pytest.raises(PimcError):
        b.hmc_attempts(1)
    b.close()


def test_autotune_with_hmc_keeps_state(tmp_path, gpu_lib):
    """The autotuner's trials (tiles, split chains, cluster sizes, overlapped cycles) leave the
    paths, every counter and the energy series as they were."""
    items = _items(tmp_path)
    b = _batch(tmp_path, items)
    b.set_hmc_per_cycle(1)
    b.run(2, 1)
    before = [b.get_path(c) for c in range(len(items))]
    cnt0, hcnt0 = b.counters(), b.hmc_counters()
    e0 = [b.energy(c) for c in range(len(items))]
    b.autotune(1)
    assert b.hmc_cluster in (1, 2, 4, 8) and 0 <= b.overlap < len(items)
    cnt1, hcnt1 = b.counters(), b.hmc_counters()
    for x, y in zip(cnt0 + hcnt0, cnt1 + hcnt1):
        assert np.array_equal(x, y)
    for c in range(len(items)):
        assert np.array_equal(before[c], b.get_path(c))
        e1 = b.energy(c)
        assert e1[1] == e0[c][1] == 2 and np.array_equal(e1[0], e0[c][0])
    b.close()
