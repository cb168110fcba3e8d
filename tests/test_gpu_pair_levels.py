"""GPU parity of pair actions with max_level > 0 against the FP64 oracle.

A pair action contributes to the bisection's level-l test when l <= max_level (pair_action_class.h:
267-302): links of stride 2^l, with DavidPairAction reading its table of index l (u_kj(level),
david_pair_action_class.h:63-102, 234-316), IlkkaPairAction its one table, the bare action zero
(its level_tau, bare_pair_action_class.h:146-150), and the Ewald part tau 2^l v_k (bare) or u_k
(tables) over the level's slices. Such moves run on the permutation kernel's plain variant, which
forms every level's terms; the bare short-range action stays on the sweep kernel. Ewald parts above
level 0 are refused. Tolerances: action values 1e-10 relative; trajectories identical accept counts
and positions within 1e-9.
"""
import numpy as np
import pytest

from simpimc_gb300 import PimcError, Simulation, sweep_chains
from simpimc_gb300.configs import electron_gas, trapped_coulomb

pytestmark = pytest.mark.gpu


def close(g, c, rel=1e-10):
    g = np.asarray(g, dtype=float)
    c = np.asarray(c, dtype=float)
    return np.all(np.abs(g - c) <= rel * np.maximum(1.0, np.abs(c)))


@pytest.mark.parametrize("pair", ["DavidPairAction", "IlkkaPairAction", "BarePairAction"])
def test_trap_bisection_replay_pair_levels(tmp_path, gpu_lib, oracle_mod, pair):
    xml, path = trapped_coulomb(tmp_path, n_part=8, n_bead=32, n_level=3, seed=23, pair=pair, n_order=2, pair_max_level=2)
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_path(path)
    c.set_path(path)
    for chunk in (1, 37, 400):
        g.move_attempts(0, chunk)
        c.move_attempts(0, chunk)
        assert g.move_stats(0) == c.move_stats(0), chunk
        assert np.max(np.abs(g.get_path(1) - c.get_path(1))) < 1e-9
    g.sweep([0], [50], n_rep=3)
    c.move_attempts(0, 150)
    assert g.move_stats(0) == c.move_stats(0)
    assert np.max(np.abs(g.get_path(1) - c.get_path(1))) < 1e-9
    for a in range(g.n_actions):
        assert close(g.dactiondbeta(a), c.dactiondbeta(a), 1e-9), a
    g.close()
    c.close()


def test_david_level_table_actions(tmp_path, gpu_lib, oracle_mod):
    xml, path = trapped_coulomb(tmp_path, n_part=8, n_bead=32, n_level=3, seed=11, pair="DavidPairAction", n_order=2,
                                pair_max_level=2)
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_path(path)
    c.set_path(path)
    new = path.copy()
    new[3, 5:12] += 0.3 * np.random.default_rng(4).standard_normal((7, 3))
    g.set_path(new, 1)
    c.set_path(new, 1)
    vals = []
    for level in range(4):
        for mode in (0, 1):
            gv = g.get_action(2, 4, 12, [(0, 3)], level, mode)
            cv = c.get_action(2, 4, 12, [(0, 3)], level, mode)
            assert close(gv, cv), (level, mode, gv, cv)
            vals.append(gv)
        gg = g.get_action_gradient(2, 8, 8 + (1 << min(level, 2)), [(0, 3)], level, 1)
        cg = c.get_action_gradient(2, 8, 8 + (1 << min(level, 2)), [(0, 3)], level, 1)
        assert close(gg, cg, 1e-8), (level, gg, cg)
    assert vals[-1] == 0.0 and vals[-2] == 0.0  # level 3 > max_level
    assert len(set(vals[:6])) == 6
    g.close()
    c.close()


@pytest.mark.parametrize("pair", ["BarePairAction", "IlkkaPairAction", "DavidPairAction"])
def test_egas_long_range_above_level_zero_refused(tmp_path, gpu_lib, pair):
    """An Ewald part with max_level > 0 is refused by every route into the moves: the reference latches
    its densities at the first level that reaches the action (pair_action_class.h:293-298)."""
    xml, path = electron_gas(tmp_path, n_part=14, n_bead=32, n_level=2, rs=2.0, k_cut_units=4.0, seed=9, pair=pair, n_order=1,
                             pair_max_level=1)
    g = Simulation(xml, base_dir=tmp_path)
    g.set_path(path)
    before = g.get_path(1)
    with pytest.raises(PimcError, match="max_level > 0"):
        g.sweep([0, 1], [7, 7], n_rep=2)
    with pytest.raises(PimcError, match="max_level > 0"):
        g.move_attempts(1, 3)
    with pytest.raises(PimcError, match="max_level > 0"):
        sweep_chains([g], [0], [3], 1)
    assert np.array_equal(g.get_path(1), before)
    assert g.move_stats(0) == (0, 0, 0)
    g.close()
