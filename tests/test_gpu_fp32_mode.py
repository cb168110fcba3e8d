"""FP32 sweep mode (FP32 per-slice densities, bead phases and Ewald differences with compensated
sums; double-float positions, pair links and acceptance) against the FP64 oracle.

Tolerances: the draws are shared, so accept counts match the oracle exactly and positions to
1e-9 (no decision lies within the FP32 error of its threshold for these seeds); densities after
the run within 2e-5 absolute per component (FP32 phases and sums of up to 33 unit phases);
estimator values within 1e-5 relative (FP32-accurate densities fed to the FP64 estimators).
"""
import numpy as np
import pytest

from simpimc_gb300 import Simulation
from simpimc_gb300.configs import electron_gas

pytestmark = pytest.mark.gpu


def test_fp32_mode_replays_oracle(tmp_path, gpu_lib, oracle_mod):
    xml, path = electron_gas(tmp_path, n_part=14, n_bead=16, n_level=2, rs=2.0, k_cut_units=4.0, seed=9)
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_precision(32)
    g.set_path(path)
    c.set_path(path)
    g.sweep([0, 1], [7, 7], n_rep=20)
    for _ in range(20):
        c.move_attempts(0, 7)
        c.move_attempts(1, 7)
    for m in range(2):
        assert g.move_stats(m) == c.move_stats(m)
    assert np.max(np.abs(g.get_path(1) - c.get_path(1))) < 1e-9
    for s in range(2):
        assert np.max(np.abs(g.rho_k(s) - c.rho_k(s))) < 2e-5
    for a in range(g.n_actions):
        gd, cd = g.dactiondbeta(a), c.dactiondbeta(a)
        assert abs(gd - cd) <= 1e-5 * max(1.0, abs(cd)), (a, gd, cd)
    g.close()
    c.close()


def test_precision_switch_keeps_the_chain(tmp_path, gpu_lib, oracle_mod):
    """Switching precision between sweep calls continues the same Markov chain."""
    xml, path = electron_gas(tmp_path, n_part=10, n_bead=16, n_level=2, rs=2.0, k_cut_units=4.0, seed=15)
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_path(path)
    c.set_path(path)
    for bits in (32, 64, 32):
        g.set_precision(bits)
        g.sweep([0, 1], [5, 5], n_rep=6)
        for _ in range(6):
            c.move_attempts(0, 5)
            c.move_attempts(1, 5)
    for m in range(2):
        assert g.move_stats(m) == c.move_stats(m)
    assert np.max(np.abs(g.get_path(1) - c.get_path(1))) < 1e-9
    g.close()
    c.close()


def test_sweep_chains_fp32_replay_oracle(tmp_path, gpu_lib, oracle_mod):
    """Electron-gas chains in FP32 mode in one pimc_sweep_chains launch: the permutation kernel's
    plain bisection with FP32 densities and Ewald terms. Each chain replays the FP64 oracle (same
    tolerances as above)."""
    import math

    from simpimc_gb300 import sweep_chains
    sims, refs = [], []
    for c in range(3):
        d = tmp_path / f"egas{c}"
        xml, path = electron_gas(d, n_part=14, n_bead=16, n_level=2, rs=2.0, k_cut_units=4.0, seed=31 + c)
        L = ((4.0 * math.pi * 14 / 3.0) ** (1.0 / 3.0)) * 2.0
        path = path + 0.3 * np.random.default_rng(70 + c).standard_normal(path.shape)
        path -= np.rint(path / L) * L
        g = Simulation(xml, base_dir=d, chain=c)
        o = oracle_mod.OracleSim(xml, base_dir=d, chain=c)
        g.set_precision(32)
        g.set_path(path)
        o.set_path(path)
        sims.append(g)
        refs.append(o)
    sweep_chains(sims, [0, 1], [7, 7], 12)
    for g, o in zip(sims, refs):
        for _ in range(12):
            o.move_attempts(0, 7)
            o.move_attempts(1, 7)
        for m in range(2):
            assert g.move_stats(m) == o.move_stats(m), m
        assert np.max(np.abs(g.get_path(1) - o.get_path(1))) < 1e-9
        for s in range(2):
            assert np.max(np.abs(g.rho_k(s) - o.rho_k(s))) < 2e-5
        for a in range(g.n_actions):
            gd, cd = g.dactiondbeta(a), o.dactiondbeta(a)
            assert abs(gd - cd) <= 1e-5 * max(1.0, abs(cd)), (a, gd, cd)
        g.close()
        o.close()


def test_fp32_exchanges_with_ewald_replay_oracle(tmp_path, gpu_lib, oracle_mod):
    """Exchanges of the up spins of an electron gas in FP32 mode (permutation kernel, FP32 densities
    of the relabelled paths): accept counts, path permutation and positions as the FP64 oracle's,
    densities within 2e-5."""
    import math
    xml, path = electron_gas(tmp_path, n_part=8, n_bead=16, n_level=2, rs=1.0, beta=4.0, k_cut_units=3.3, seed=4,
                             perm="PermBisectIterative")
    L = (4.0 * math.pi * 8 / 3.0) ** (1.0 / 3.0) * 1.0
    rng = np.random.default_rng(2)
    centre = rng.uniform(-L / 2, L / 2, size=(8, 1, 3))
    path = centre + 0.2 * rng.standard_normal(path.shape)
    path -= np.rint(path / L) * L
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_precision(32)
    g.set_path(path)
    c.set_path(path)
    pm = 2  # BisectU, BisectD, PermU
    for m, chunk in [(pm, 30), (0, 10), (pm, 200), (1, 10), (pm, 200)]:
        g.move_attempts(m, chunk)
        c.move_attempts(m, chunk)
        assert g.move_stats(m) == c.move_stats(m), (m, chunk)
        assert np.max(np.abs(g.get_path(1) - c.get_path(1))) < 1e-9
    np.testing.assert_array_equal(g.get_perm(0), c.get_perm(0, 4))
    for s in range(2):
        assert np.max(np.abs(g.rho_k(s) - c.rho_k(s))) < 2e-5
    g.close()
    c.close()
