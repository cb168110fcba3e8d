"""GPU parity of DavidPairAction (david_pair_action_class.h:7-361) against the FP64 oracle.

Tables are synthetic (simpimc_gb300.tables.david_table) in the reference's schema, expansion order 2
on the trapped system and 1 on the electron gas. Tolerances as for the other pair actions: values
1e-10 relative; the gradient is the base class's central difference (eps = 1e-4, pair_action_class.h:
135-155), which amplifies last-bit differences of the two CalcU values by 1/eps, so 1e-8; bisection
trajectories identical accept counts and positions within 1e-9.
"""
import numpy as np
import pytest

from simpimc_gb300 import PimcError, Simulation
from simpimc_gb300.configs import electron_gas, trapped_coulomb

pytestmark = pytest.mark.gpu


def close(g, c, rel=1e-10):
    g = np.asarray(g, dtype=float)
    c = np.asarray(c, dtype=float)
    return np.all(np.abs(g - c) <= rel * np.maximum(1.0, np.abs(c)))


def perturbed(path, rng, particle, b0, b1, scale=0.3):
    new = path.copy()
    M = path.shape[1]
    for b in range(b0 + 1, b1):
        new[particle, b % M] += scale * rng.standard_normal(path.shape[2])
    return new


@pytest.fixture(scope="module")
def trap_pair(tmp_path_factory, gpu_lib, oracle_mod):
    d = tmp_path_factory.mktemp("david_trap")
    xml, path = trapped_coulomb(d, n_part=8, n_bead=32, n_level=3, seed=11, pair="DavidPairAction", n_order=2)
    g = Simulation(xml, base_dir=d)
    c = oracle_mod.OracleSim(xml, base_dir=d)
    g.set_path(path)
    c.set_path(path)
    yield g, c, path
    g.close()
    c.close()


@pytest.mark.parametrize("b0", [0, 27])
def test_david_trap_actions_and_gradients(trap_pair, b0):
    g, c, path = trap_pair
    new = perturbed(path, np.random.default_rng(b0 + 3), 3, b0, b0 + 8)
    g.set_path(path, 2)
    c.set_path(path, 2)
    g.set_path(new, 1)
    c.set_path(new, 1)
    for mode in (0, 1):
        gv = g.get_action(2, b0, b0 + 8, [(0, 3)], 0, mode)
        cv = c.get_action(2, b0, b0 + 8, [(0, 3)], 0, mode)
        assert close(gv, cv), (mode, gv, cv)
        gg = g.get_action_gradient(2, b0 + 2, b0 + 3, [(0, 3)], 0, mode)
        cg = c.get_action_gradient(2, b0 + 2, b0 + 3, [(0, 3)], 0, mode)
        assert close(gg, cg, 1e-8), (mode, gg, cg)
    g.set_path(path, 2)
    c.set_path(path, 2)
    for a in range(g.n_actions):
        assert close(g.dactiondbeta(a), c.dactiondbeta(a)), a
        assert close(g.potential(a), c.potential(a)), a


def test_david_trap_bisection_replay(tmp_path, gpu_lib, oracle_mod):
    xml, path = trapped_coulomb(tmp_path, n_part=8, n_bead=32, n_level=3, seed=21, pair="DavidPairAction", n_order=2)
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_path(path)
    c.set_path(path)
    for chunk in (1, 37, 400):
        g.move_attempts(0, chunk)
        c.move_attempts(0, chunk)
        assert g.move_stats(0) == c.move_stats(0)
        assert np.max(np.abs(g.get_path(1) - c.get_path(1))) < 1e-9
    g.close()
    c.close()


def test_david_virial_energy_blocks(tmp_path, gpu_lib, oracle_mod):
    xml, path = trapped_coulomb(tmp_path, n_part=6, n_bead=16, n_level=2, seed=3, virial=True, pair="DavidPairAction", n_order=2)
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_path(path)
    c.set_path(path)
    for _ in range(4):
        g.move_attempts(0, 40)
        c.move_attempts(0, 40)
        g.observable_accumulate(0)
        c.observable_accumulate(0)
    eg, ec = g.observable_block(0), c.observable_block(0)
    assert eg.shape == ec.shape and close(eg, ec, 1e-8), (eg, ec)
    g.close()
    c.close()


@pytest.mark.parametrize("wave", [1, 2])
def test_david_egas_actions_and_sweep(tmp_path, gpu_lib, oracle_mod, wave):
    xml, path = electron_gas(tmp_path, n_part=14, n_bead=32, n_level=2, rs=2.0, k_cut_units=4.0, seed=9, pair="DavidPairAction",
                             n_order=1)
    L = ((4.0 * np.pi * 14 / 3.0) ** (1.0 / 3.0)) * 2.0
    path = np.random.default_rng(5).uniform(-L / 2, L / 2, size=path.shape)
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_path(path)
    c.set_path(path)
    for a in range(g.n_actions):
        for mode in (0, 1):
            assert close(g.get_action(a, 3, 7, [(0, 2)], 0, mode), c.get_action(a, 3, 7, [(0, 2)], 0, mode)), (a, mode)
        assert close(g.dactiondbeta(a), c.dactiondbeta(a)), a
        assert close(g.potential(a), c.potential(a)), a
    g.set_sweep_wave(wave)
    g.sweep([0, 1], [7, 7], n_rep=6)
    for _ in range(6):
        c.move_attempts(0, 7)
        c.move_attempts(1, 7)
    for m in range(2):
        assert g.move_stats(m) == c.move_stats(m), m
    assert np.max(np.abs(g.get_path(1) - c.get_path(1))) < 1e-9
    with pytest.raises(PimcError):
        g.total_action()
    g.close()
    c.close()
