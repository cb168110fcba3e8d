"""GPU parity of IlkkaPairAction (ilkka_pair_action_class.h:7-433) against the FP64 oracle.

Tables are synthetic (simpimc_gb300.tables.ilkka_table) in the reference's schema. The GPU's 2-D
spline is the natural bicubic spline stored per cell; the oracle evaluates the same tensor-product
spline as 1-D natural splines along x then y, so the two agree to rounding. Tolerances:
  * action values, gradients, dS/dbeta, potentials, estimator blocks: 1e-10 relative (FP64 both
    sides, different evaluation order of the same spline);
  * bisection trajectories (double-float sweep kernel): identical accept counts, positions within
    1e-9 after the replay.
"""
import numpy as np
import pytest

from simpimc_gb300 import PimcError, Simulation
from simpimc_gb300.configs import electron_gas, trapped_coulomb

pytestmark = pytest.mark.gpu

REL = 1e-10


def close(g, c, rel=REL):
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
    d = tmp_path_factory.mktemp("ilkka_trap")
    xml, path = trapped_coulomb(d, n_part=8, n_bead=32, n_level=3, seed=11, pair="IlkkaPairAction")
    g = Simulation(xml, base_dir=d)
    c = oracle_mod.OracleSim(xml, base_dir=d)
    g.set_path(path)
    c.set_path(path)
    yield g, c, path
    g.close()
    c.close()


@pytest.fixture(scope="module")
def egas_pair(tmp_path_factory, gpu_lib, oracle_mod):
    d = tmp_path_factory.mktemp("ilkka_egas")
    xml, path = electron_gas(d, n_part=14, n_bead=16, n_level=2, rs=2.0, k_cut_units=4.0, seed=5, pair="IlkkaPairAction")
    L = ((4.0 * np.pi * 14 / 3.0) ** (1.0 / 3.0)) * 2.0
    path = np.random.default_rng(17).uniform(-L / 2, L / 2, size=path.shape)  # spread beads
    g = Simulation(xml, base_dir=d)
    c = oracle_mod.OracleSim(xml, base_dir=d)
    g.set_path(path)
    c.set_path(path)
    yield g, c, path
    g.close()
    c.close()


@pytest.mark.parametrize("b0", [0, 5, 28])
def test_ilkka_trap_actions_and_gradients(trap_pair, b0):
    g, c, path = trap_pair
    rng = np.random.default_rng(b0 + 1)
    B = 8
    new = perturbed(path, rng, 3, b0, b0 + B)
    g.set_path(path, 2)
    c.set_path(path, 2)
    g.set_path(new, 1)
    c.set_path(new, 1)
    a = 2  # Kinetic, Trap, Coulomb
    for mode in (0, 1):
        gv = g.get_action(a, b0, b0 + B, [(0, 3)], 0, mode)
        cv = c.get_action(a, b0, b0 + B, [(0, 3)], 0, mode)
        assert close(gv, cv), (mode, gv, cv)
        for b in (b0, b0 + 3):
            gg = g.get_action_gradient(a, b, b + 1, [(0, 3)], 0, mode)
            cg = c.get_action_gradient(a, b, b + 1, [(0, 3)], 0, mode)
            assert close(gg, cg), (mode, b, gg, cg)
    assert g.get_action(a, b0, b0 + B, [(0, 3)], 1, 0) == 0.0  # level > max_level
    g.set_path(path, 2)
    c.set_path(path, 2)


def test_ilkka_trap_estimator_terms(trap_pair):
    g, c, path = trap_pair
    for a in range(g.n_actions):
        assert close(g.dactiondbeta(a), c.dactiondbeta(a)), a
        assert close(g.potential(a), c.potential(a)), a


def test_ilkka_trap_bisection_replay(tmp_path, gpu_lib, oracle_mod):
    xml, path = trapped_coulomb(tmp_path, n_part=8, n_bead=32, n_level=3, seed=21, pair="IlkkaPairAction")
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_path(path)
    c.set_path(path)
    for chunk in (1, 37, 400):
        g.move_attempts(0, chunk)
        c.move_attempts(0, chunk)
        assert g.move_stats(0) == c.move_stats(0)
        assert np.max(np.abs(g.get_path(1) - c.get_path(1))) < 1e-9
    for a in range(g.n_actions):
        assert close(g.dactiondbeta(a), c.dactiondbeta(a), 1e-9)
    g.close()
    c.close()


def test_ilkka_virial_energy_blocks(tmp_path, gpu_lib, oracle_mod):
    """The virial estimator's centroid term uses the analytic Ilkka gradient."""
    xml, path = trapped_coulomb(tmp_path, n_part=6, n_bead=16, n_level=2, seed=3, virial=True, pair="IlkkaPairAction")
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


@pytest.mark.parametrize("b0,particle,species", [(0, 2, 0), (13, 6, 1)])
def test_ilkka_egas_actions(egas_pair, b0, particle, species):
    g, c, path = egas_pair
    rng = np.random.default_rng(b0 + 31 * particle)
    B = 4
    _, off, _ = g.species_info(species)
    new = perturbed(path, rng, off + particle, b0, b0 + B, scale=0.2)
    g.set_path(path, 2)
    c.set_path(path, 2)
    g.set_path(new, 1)
    c.set_path(new, 1)
    for a in range(g.n_actions):
        for mode in (0, 1):
            gv = g.get_action(a, b0, b0 + B, [(species, particle)], 0, mode)
            cv = c.get_action(a, b0, b0 + B, [(species, particle)], 0, mode)
            assert close(gv, cv), (a, mode, gv, cv)
    g.set_path(path, 2)
    c.set_path(path, 2)
    for a in range(2, g.n_actions):
        # stored path: the link gradient plus the long-range bead term once per pair
        gg = g.get_action_gradient(a, b0, b0 + 1, [(species, particle)], 0, 0)
        cg = c.get_action_gradient(a, b0, b0 + 1, [(species, particle)], 0, 0)
        assert close(gg, cg), (a, gg, cg)


def test_ilkka_egas_estimator_terms(egas_pair):
    g, c, path = egas_pair
    g.set_path(path, 2)
    c.set_path(path, 2)
    for a in range(g.n_actions):
        assert close(g.dactiondbeta(a), c.dactiondbeta(a)), a
        assert close(g.potential(a), c.potential(a)), a


@pytest.mark.parametrize("wave", [1, 2])
def test_ilkka_egas_sweep_replay(tmp_path, gpu_lib, oracle_mod, wave):
    xml, path = electron_gas(tmp_path, n_part=14, n_bead=32, n_level=2, rs=2.0, k_cut_units=4.0, seed=9, pair="IlkkaPairAction")
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_sweep_wave(wave)
    g.set_path(path)
    c.set_path(path)
    g.sweep([0, 1], [7, 7], n_rep=10)
    for _ in range(10):
        c.move_attempts(0, 7)
        c.move_attempts(1, 7)
    for m in range(2):
        assert g.move_stats(m) == c.move_stats(m), m
    assert np.max(np.abs(g.get_path(1) - c.get_path(1))) < 1e-9
    for s in range(2):
        assert np.max(np.abs(g.rho_k(s) - c.rho_k(s))) < 1e-9
    for a in range(g.n_actions):
        assert close(g.dactiondbeta(a), c.dactiondbeta(a), 1e-9)
    g.close()
    c.close()


def test_ilkka_refused_by_whole_ring_paths(tmp_path, gpu_lib):
    """The whole-ring action and exact gradient (and HMC on them) cover the bare action only."""
    xml, path = trapped_coulomb(tmp_path, n_part=4, n_bead=8, n_level=2, seed=2, pair="IlkkaPairAction")
    g = Simulation(xml, base_dir=tmp_path)
    g.set_path(path)
    with pytest.raises(PimcError):
        g.total_action()
    assert g.total_action(0) != 0.0  # the kinetic action alone is still available
    g.close()
