"""GPU parity at the benchmark workloads' full sizes, against the FP64 oracle.

The sweep kernel splits its work by the workload's size: the (slice residue, k-chunk) cells of each
block follow K and 2^l, the automatic attempts-in-flight setting follows 2^l K, and the batched
kernel stages a chain's path in shared memory only when it fits. The small parity tests therefore
do not run the code paths the benchmark runs. These tests do, at the benchmark sizes:

- the 66-electron gas (N = 66 as 33 + 33, r_s = 2, beta = 8, M = 128, |k| < 12 (2 pi / L), 3561
  half-space k-vectors, bisection level 4, automatic attempts in flight): one full sweep (528
  attempts) replayed by the oracle. Accept counts identical, positions and per-slice densities within
  1e-9, dS/dbeta of every action within 1e-10 relative (the FP64 tolerances of the parity tests);
- the four heaviest chains (M = 128, largest N) of the 256-chain batch, run inside the whole batch
  with the autotuned tile (their paths staged in shared memory): 320 attempts per chain replayed by
  the oracle. Accept counts identical, positions within 1e-4 (FP32 positions);
- the 1024-electron gas (r_s = 1, beta = 4, M = 512, |k| < 23 (2 pi / L), 25366 half-space k-vectors, level 4),
  with the oracle in its lean-density mode (the reference's per-bead densities would take 426 GB):
  256 attempts of the double-float sweep replayed exactly (accept counts identical, positions within
  1e-9, densities within 1e-8 absolute), then the FP32 mode's path, estimators and S(k) on the first
  200 |k| shells against the FP64 oracle on that same path, each within 1e-5 relative (the FP32
  tolerance); the observed errors are printed.
"""
import numpy as np
import pytest

from simpimc_gb300 import ChainBatch, Simulation
from simpimc_gb300.configs import batched_trap_chains, electron_gas

pytestmark = pytest.mark.gpu


def rel_close(g, c, rel):
    g = np.asarray(g)
    c = np.asarray(c)
    return np.all(np.abs(g - c) <= rel * np.maximum(1.0, np.abs(c)))


def _replay_schedule(o, reps):
    for _ in range(reps):
        o.move_attempts(0, 1)
        o.move_attempts(1, 1)


def test_egas66_full_sweep_replay(tmp_path, gpu_lib, oracle_mod):
    xml, path = electron_gas(tmp_path, n_part=66, rs=2.0, beta=8.0, n_bead=128, k_cut_units=12.0, n_level=4, seed=20261203)
    path = path + 0.3 * np.random.default_rng(66).standard_normal(path.shape)
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    assert g.n_k == c.n_k == 3561
    g.set_path(path)
    c.set_path(path)
    reps = 33 * (128 // 16)  # one sweep: N_s ceil(M / 2^l) attempts of each species, alternating
    g.sweep([0, 1], [1, 1], reps)
    _replay_schedule(c, reps)
    for m in range(2):
        assert g.move_stats(m) == c.move_stats(m), (m, g.move_stats(m), c.move_stats(m))
    assert g.move_stats(0)[2] > 20  # the chain moved
    assert np.max(np.abs(g.get_path(1) - c.get_path(1))) < 1e-9
    for s in range(2):
        assert np.max(np.abs(g.rho_k(s) - c.rho_k(s))) < 1e-9, s
    for a in range(g.n_actions):
        assert rel_close(g.dactiondbeta(a), c.dactiondbeta(a), 1e-10), a
    g.close()
    c.close()


def test_batch_heaviest_chains_replay(tmp_path, gpu_lib, oracle_mod):
    items = batched_trap_chains(tmp_path, n_chains=256, seed0=1000, n_level=3)
    items = [(x, np.asarray(p, dtype=np.float32).astype(np.float64)) for x, p in items]
    b = ChainBatch([x for x, _ in items], base_dir=tmp_path)
    for i, (_, p) in enumerate(items):
        b.set_path(i, p)
    b.autotune(1)  # the tile the benchmark runs; the chains' state is restored afterwards
    for i, (_, p) in enumerate(items):
        assert np.array_equal(b.get_path(i), p)
    n_att = 320
    b.attempts(n_att)
    att, acc = b.counters()
    heavy = sorted((i for i, s in enumerate(b.shapes) if s[1] == 128), key=lambda i: -b.shapes[i][0])[:4]
    assert min(b.shapes[i][0] for i in heavy) >= 120, [b.shapes[i] for i in heavy]
    for i in heavy:
        xml, p = items[i]
        o = oracle_mod.OracleSim(xml, base_dir=tmp_path, chain=i)
        o.set_path(p)
        o.move_attempts(0, n_att)
        assert int(att[i]) == n_att
        assert int(acc[i]) == o.move_stats(0)[2], (i, b.shapes[i], int(acc[i]), o.move_stats(0))
        assert np.max(np.abs(b.get_path(i) - o.get_path())) < 1e-4, i
        o.close()
    b.close()


def _shell_means(kmag, sk, n_shells):
    mags = np.round(kmag, 9)
    shells = np.unique(mags)[:n_shells]
    return np.array([sk[mags == m].mean() for m in shells])


def test_egas1024_replay_and_fp32_estimators(tmp_path, gpu_lib, oracle_mod):
    xml, path = electron_gas(tmp_path, n_part=1024, rs=1.0, beta=4.0, n_bead=512, k_cut_units=23.0, n_level=4, seed=777,
                             structure_factor=True)
    path = path + 0.15 * np.random.default_rng(1024).standard_normal(path.shape)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path, lean_densities=True)
    assert c.n_k == 25366
    reps = 128

    # double-float sweep against the FP64 oracle, attempt for attempt
    g = Simulation(xml, base_dir=tmp_path)
    g.set_path(path)
    c.set_path(path)
    g.sweep([0, 1], [1, 1], reps)
    _replay_schedule(c, reps)
    for m in range(2):
        assert g.move_stats(m) == c.move_stats(m), (m, g.move_stats(m), c.move_stats(m))
    assert np.max(np.abs(g.get_path(1) - c.get_path(1))) < 1e-9
    for s in range(2):
        assert np.max(np.abs(g.rho_k(s) - c.rho_k(s))) < 1e-8, s
    g.close()

    # FP32 mode: its path after the same attempts, its estimators against the oracle on that path
    g = Simulation(xml, base_dir=tmp_path)
    g.set_precision(32)
    g.set_path(path)
    g.sweep([0, 1], [1, 1], reps)
    final = g.get_path(1)
    c.set_path(final)
    g.observable_accumulate(0)
    g.observable_accumulate(2)
    c.observable_accumulate(0)
    c.observable_accumulate(2)
    eg, ec = g.observable_block(0), c.observable_block(0)
    sg, sc = g.observable_block(2), c.observable_block(2)
    kmag = np.linalg.norm(g.kvecs(), axis=1)
    shg, shc = _shell_means(kmag, sg, 200), _shell_means(kmag, sc, 200)
    e_err = float(np.max(np.abs(eg - ec) / np.maximum(1.0, np.abs(ec))))
    s_err = float(np.max(np.abs(shg - shc) / np.maximum(1.0, np.abs(shc))))
    print(f"FP32 mode vs FP64 oracle, N=1024 M=512 K=25366: energy terms max rel err {e_err:.3e}, "
          f"S(k) 200 shells max rel err {s_err:.3e}")
    assert eg.shape == ec.shape and len(shg) == 200
    assert e_err < 1e-5, (eg, ec)
    assert s_err < 1e-5
    g.close()
    c.close()
