"""Batched independent chains (FP32 positions and action terms, double-float sums) against the
FP64 oracle and the single-chain FP64 GPU path.

Tolerances:
  * energy components of one configuration (the chain's FP32 positions fed to the oracle as
    doubles): |batch - oracle| <= 1e-5 * max(1, |oracle|);
  * Markov-chain replay: chain i draws from the same stream as an oracle created with chain = i,
    so accept counts match exactly and positions stay within 1e-4 after a few hundred attempts
    (FP32 rounding of the proposals accumulates; a decision can only differ within ~1e-6 of
    the threshold, which these seeds never hit);
  * graph replay and kernel launches of the same work give identical bits.
"""
import numpy as np
import pytest

from simpimc_gb300 import ChainBatch, Simulation
from simpimc_gb300.configs import batched_trap_chains, trapped_coulomb

pytestmark = pytest.mark.gpu

SHAPES = [  # (n_part, n_bead, n_level)
    (2, 8, 1), (5, 16, 2), (16, 32, 3), (33, 32, 3), (40, 64, 4), (17, 128, 5), (64, 32, 3), (9, 8, 3),
    (2, 16, 3),  # one partner: item and pair indices divide by 1
]


def f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


@pytest.fixture(scope="module")
def chains(tmp_path_factory, gpu_lib, oracle_mod):
    d = tmp_path_factory.mktemp("batch")
    items = []
    for c, (n, m, lvl) in enumerate(SHAPES):
        xml, path = trapped_coulomb(d, n_part=n, n_bead=m, n_level=lvl, seed=300 + c, write_table=(c == 0))
        items.append((xml, f32(path)))
    return d, items


def make_batch(d, items):
    b = ChainBatch([x for x, _ in items], base_dir=d)
    for c, (_, p) in enumerate(items):
        b.set_path(c, p)
    return b


def test_energy_matches_oracle(chains, oracle_mod):
    d, items = chains
    b = make_batch(d, items)
    b.measure()
    for c, (xml, path) in enumerate(items):
        o = oracle_mod.OracleSim(xml, base_dir=d, chain=c)
        o.set_path(path)
        M = path.shape[1]
        ref = np.array([o.dactiondbeta(a) / M for a in range(3)])
        series, n = b.energy(c)
        assert n == 1
        got = series[0]
        assert np.all(np.abs(got[1:] - ref) <= 1e-5 * np.maximum(1.0, np.abs(ref))), (c, got, ref)
        assert abs(got[0] - ref.sum()) <= 1e-5 * max(1.0, abs(ref.sum())), (c, got[0], ref.sum())
        o.close()
    b.close()


def test_replay_matches_oracle(chains, oracle_mod):
    d, items = chains
    b = make_batch(d, items)
    n_att = 300
    b.attempts(n_att)
    att, acc = b.counters()
    assert np.all(att == n_att)
    for c, (xml, path) in enumerate(items):
        o = oracle_mod.OracleSim(xml, base_dir=d, chain=c)
        o.set_path(path)
        o.move_attempts(0, n_att)
        st = o.move_stats(0)
        assert int(acc[c]) == int(st[2]), (c, int(acc[c]), st)
        n, m, lvl = b.shapes[c]
        if (1 << lvl) < m:  # a whole-ring segment drops the kinetic action and is always rejected here
            assert 0 < int(acc[c]) < n_att, (c, int(acc[c]))
        assert np.max(np.abs(b.get_path(c) - o.get_path())) < 1e-4, c
        o.close()
    b.close()


@pytest.mark.parametrize("wave", [2, 4, 8])
def test_concurrent_attempts_replay_oracle(chains, oracle_mod, wave):
    """Attempts run several at a time, out of order where they commute (a scoreboard over the next
    16 draws), give the sequential chain: the oracle's accept counts and positions."""
    d, items = chains
    b = make_batch(d, items)
    b.set_tiles(2, 16, wave)
    n_att = 300
    b.attempts(n_att)
    att, acc = b.counters()
    assert np.all(att == n_att)
    for c, (xml, path) in enumerate(items):
        o = oracle_mod.OracleSim(xml, base_dir=d, chain=c)
        o.set_path(path)
        o.move_attempts(0, n_att)
        assert int(acc[c]) == int(o.move_stats(0)[2]), (c, wave, int(acc[c]), o.move_stats(0))
        assert np.max(np.abs(b.get_path(c) - o.get_path())) < 1e-4, (c, wave)
        o.close()
    b.close()


def test_same_chain_as_fp64_gpu_path(chains):
    """Chain i of the batch and a single-chain FP64 context with chain = i make the same moves."""
    d, items = chains
    b = make_batch(d, items)
    c = 3
    xml, path = items[c]
    s = Simulation(xml, base_dir=d, chain=c)
    s.set_path(path)
    b.attempts(200)
    s.move_attempts(0, 200)
    _, acc = b.counters()
    assert int(acc[c]) == s.move_counters(0)[3]
    assert np.max(np.abs(b.get_path(c) - s.get_path())) < 1e-4
    s.close()
    b.close()


def test_graph_run_equals_launches(chains):
    d, items = chains
    b1 = make_batch(d, items)
    b2 = make_batch(d, items)
    b1.run(3, 2)
    for _ in range(3):
        b2.sweeps(2)
        b2.measure()
    a1, c1 = b1.counters()
    a2, c2 = b2.counters()
    assert np.array_equal(a1, a2) and np.array_equal(c1, c2)
    for c, (_, path) in enumerate(items):
        n, m, lvl = b1.shapes[c]
        B = 1 << lvl
        assert int(a1[c]) == 6 * n * ((m + B - 1) // B)
        assert np.array_equal(b1.get_path(c), b2.get_path(c))
        e1, n1 = b1.energy(c)
        e2, n2 = b2.energy(c)
        assert n1 == n2 == 3 and np.array_equal(e1, e2)
    b1.close()
    b2.close()


def test_autotune_keeps_state(chains):
    d, items = chains
    b = make_batch(d, items)
    b.attempts(50)
    before = [b.get_path(c) for c in range(len(items))]
    att0, acc0 = b.counters()
    ipl, mw, wave, sec = b.autotune(1)
    assert ipl >= 1 and 1 <= mw <= 16 and 1 <= wave <= 8 and sec > 0
    att1, acc1 = b.counters()
    assert np.array_equal(att0, att1) and np.array_equal(acc0, acc1)
    for c in range(len(items)):
        assert np.array_equal(before[c], b.get_path(c))
    b.close()


def test_tile_shape_does_not_change_the_chain(chains):
    d, items = chains
    ref = None
    for ipl, mw, wave in ((1, 16, 1), (4, 4, 1), (32, 1, 1), (2, 16, 2), (4, 16, 4), (8, 8, 4), (2, 16, 8), (4, 8, 8)):
        b = make_batch(d, items)
        b.set_tiles(ipl, mw, wave)
        b.attempts(150)
        _, acc = b.counters()
        paths = [b.get_path(c) for c in range(len(items))]
        if ref is None:
            ref = (acc, paths)
        else:
            assert np.array_equal(acc, ref[0])
            for c in range(len(items)):
                assert np.max(np.abs(paths[c] - ref[1][c])) < 1e-5
        b.close()


def test_uneven_batch_runs(tmp_path, gpu_lib):
    items = batched_trap_chains(tmp_path, n_chains=24, seed0=77)
    b = ChainBatch([x for x, _ in items], base_dir=tmp_path)
    for c, (_, p) in enumerate(items):
        b.set_path(c, p)
    b.run(2, 1)
    att, acc = b.counters()
    for c in range(len(items)):
        n, m, lvl = b.shapes[c]
        assert int(att[c]) == 2 * n * ((m + (1 << lvl) - 1) >> lvl)
        e, k = b.energy(c)
        assert k == 2 and np.all(np.isfinite(e))
    assert np.all(acc > 0)
    b.close()



def test_rounds_count_the_scheduler(chains):
    """pimc_batch_rounds: one round per attempt at wave 1; at wave 8 every round runs at least one
    attempt and the chains with room for concurrent attempts run several per round."""
    d, items = chains
    b = make_batch(d, items)
    b.set_tiles(2, 16, 1)
    b.attempts(40)
    r1 = b.rounds()
    assert np.array_equal(r1, np.full(len(items), 40, dtype=np.uint64))
    b.set_tiles(2, 16, 8)
    b.attempts(200)
    r2 = b.rounds() - r1
    att, _ = b.counters()
    assert np.all(att == 240) and np.all(r2 >= 1) and np.all(r2 <= 200)
    long_chains = [c for c, (n, m, lvl) in enumerate(SHAPES) if m >= 4 * (1 << lvl) and n >= 16]
    assert long_chains and all(int(r2[c]) < 170 for c in long_chains), [(c, int(r2[c])) for c in long_chains]
    b.close()


@pytest.mark.parametrize("n_split", [1, 4, 9])
def test_split_chains_match_one_block_per_chain(chains, n_split):
    """The most expensive chains on two-block clusters (both blocks hold the path; a round runs up
    to eight commuting attempts, commits written into both copies) make the same moves as the
    one-block launch: identical accept counts and paths, bit for bit; odd and even chain counts."""
    d, items = chains
    ref = make_batch(d, items)
    ref.set_tiles(2, 16, 8)
    ref.attempts(150)
    ref.sweeps(2)
    b = make_batch(d, items)
    b.set_tiles(2, 16, 8)
    b.split = n_split
    assert b.split == n_split
    b.attempts(150)
    b.sweeps(2)
    a0, c0 = ref.counters()
    a1, c1 = b.counters()
    assert np.array_equal(a0, a1) and np.array_equal(c0, c1)
    for c in range(len(items)):
        assert np.array_equal(ref.get_path(c), b.get_path(c)), c
    ref.close()
    b.close()
