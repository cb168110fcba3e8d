"""GPU parity: every action-interface call of the CUDA library against the FP64 oracle.

Tolerances (FP64 on both sides; only summation order and libm last-bit differences separate them):
  * action values, dS/dbeta, potentials, virial energies: |gpu - cpu| <= 1e-10 * max(1, |cpu|);
  * finite-difference pair gradients (eps = 1e-4 central differences of tau*V, as the reference
    computes them): |gpu - cpu| <= 1e-8 * max(1, |cpu|), since the difference quotient amplifies
    last-bit differences of the two CalcU values by 1/eps;
  * bisection trajectories: identical accept counts, positions within 1e-9 after the replay.
"""
import numpy as np
import pytest

from simpimc_gb300 import Simulation
from simpimc_gb300.configs import electron_gas, trapped_coulomb

pytestmark = pytest.mark.gpu

REL = 1e-10


def close(g, c, rel=REL):
    g = np.asarray(g, dtype=float)
    c = np.asarray(c, dtype=float)
    return np.all(np.abs(g - c) <= rel * np.maximum(1.0, np.abs(c)))


@pytest.fixture(scope="module")
def trap_pair(tmp_path_factory, gpu_lib, oracle_mod):
    d = tmp_path_factory.mktemp("trap")
    xml, path = trapped_coulomb(d, n_part=8, n_bead=32, n_level=3, seed=11)
    g = Simulation(xml, base_dir=d)
    c = oracle_mod.OracleSim(xml, base_dir=d)
    g.set_path(path)
    c.set_path(path)
    yield g, c, path
    g.close()
    c.close()


@pytest.fixture(scope="module")
def egas_pair(tmp_path_factory, gpu_lib, oracle_mod):
    d = tmp_path_factory.mktemp("egas")
    xml, path = electron_gas(d, n_part=14, n_bead=16, n_level=2, rs=2.0, k_cut_units=4.0, seed=5)
    g = Simulation(xml, base_dir=d)
    c = oracle_mod.OracleSim(xml, base_dir=d)
    g.set_path(path)
    c.set_path(path)
    yield g, c, path
    g.close()
    c.close()


def perturbed(path, rng, particle, b0, b1, scale=0.3):
    new = path.copy()
    M = path.shape[1]
    for b in range(b0 + 1, b1):
        new[particle, b % M] += scale * rng.standard_normal(path.shape[2])
    return new


@pytest.mark.parametrize("b0,level", [(0, 0), (5, 0), (28, 0), (8, 1), (30, 2)])
def test_trap_actions(trap_pair, b0, level):
    g, c, path = trap_pair
    rng = np.random.default_rng(b0 * 7 + level)
    B = 8
    new = perturbed(path, rng, 3, b0, b0 + B)
    g.set_path(path, 2)
    c.set_path(path, 2)
    g.set_path(new, 1)
    c.set_path(new, 1)
    for a in range(g.n_actions):
        for mode in (0, 1):
            gv = g.get_action(a, b0, b0 + B, [(0, 3)], level, mode)
            cv = c.get_action(a, b0, b0 + B, [(0, 3)], level, mode)
            assert close(gv, cv), (a, mode, gv, cv)
        gg = g.get_action_gradient(a, b0, b0 + 1, [(0, 3)], 0, 1)
        cg = c.get_action_gradient(a, b0, b0 + 1, [(0, 3)], 0, 1)
        assert close(gg, cg, 1e-8), (a, gg, cg)
    g.set_path(path, 2)
    c.set_path(path, 2)


def test_trap_estimator_terms(trap_pair):
    g, c, path = trap_pair
    for a in range(g.n_actions):
        assert close(g.dactiondbeta(a), c.dactiondbeta(a)), a
        assert close(g.potential(a), c.potential(a)), a
        for w in (1, 4, 32):
            assert close(g.virial_energy(a, w), c.virial_energy(a, w)), (a, w)


def test_egas_kspace_and_rho(egas_pair):
    g, c, path = egas_pair
    assert g.n_k == c.n_k > 0
    np.testing.assert_allclose(g.kvecs(), c.kvecs(), rtol=0, atol=1e-14)
    for s in range(2):
        gr, cr = g.rho_k(s), c.rho_k(s)
        assert np.max(np.abs(gr - cr)) < 1e-11


@pytest.mark.parametrize("b0,particle,species", [(0, 2, 0), (13, 6, 1), (7, 0, 0)])
def test_egas_actions(egas_pair, b0, particle, species):
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
    for a in range(g.n_actions):
        assert close(g.dactiondbeta(a), c.dactiondbeta(a)), a
        assert close(g.potential(a), c.potential(a)), a


def test_trap_bisection_replay(tmp_path, gpu_lib, oracle_mod):
    xml, path = trapped_coulomb(tmp_path, n_part=8, n_bead=32, n_level=3, seed=21)
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_path(path)
    c.set_path(path)
    for chunk in (1, 37, 500, 1462):
        g.move_attempts(0, chunk)
        c.move_attempts(0, chunk)
        assert g.move_stats(0) == c.move_stats(0)
        assert np.max(np.abs(g.get_path(1) - c.get_path(1))) < 1e-9
    assert np.max(np.abs(g.get_path(0) - c.get_path(0))) < 1e-9
    for a in range(g.n_actions):
        assert close(g.dactiondbeta(a), c.dactiondbeta(a), 1e-9)


def test_full_ring_bisection_replay(tmp_path, gpu_lib, oracle_mod):
    """A segment of 2^l = M beads: the reference's kinetic walk from the first bead to the bead
    M slices later stops at once (same bead), so only trap, pair and sampling terms decide."""
    xml, path = trapped_coulomb(tmp_path, n_part=5, n_bead=8, n_level=3, seed=23)
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_path(path)
    c.set_path(path)
    g.move_attempts(0, 400)
    c.move_attempts(0, 400)
    assert g.move_stats(0) == c.move_stats(0)
    assert np.max(np.abs(g.get_path(1) - c.get_path(1))) < 1e-9


def test_egas_bisection_replay(tmp_path, gpu_lib, oracle_mod):
    xml, path = electron_gas(tmp_path, n_part=14, n_bead=16, n_level=2, rs=2.0, k_cut_units=4.0, seed=9)
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
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
        assert np.max(np.abs(g.rho_k(s) - c.rho_k(s))) < 1e-9
    for a in range(g.n_actions):
        assert close(g.dactiondbeta(a), c.dactiondbeta(a), 1e-9)


@pytest.mark.parametrize("wave", [0, 1, 2, 4, 8])
def test_concurrent_sweep_replays_oracle(tmp_path, gpu_lib, oracle_mod, wave):
    """Rounds of conflict-free attempts give the sequential chain for every wave size."""
    xml, path = electron_gas(tmp_path, n_part=14, n_bead=64, n_level=3, rs=2.0, k_cut_units=4.0, seed=31)
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_sweep_wave(wave)
    g.set_path(path)
    c.set_path(path)
    g.sweep([0, 1], [7, 7], n_rep=12)
    for _ in range(12):
        c.move_attempts(0, 7)
        c.move_attempts(1, 7)
    for m in range(2):
        assert g.move_stats(m) == c.move_stats(m), (wave, m)
    assert np.max(np.abs(g.get_path(1) - c.get_path(1))) < 1e-9
    for s in range(2):
        assert np.max(np.abs(g.rho_k(s) - c.rho_k(s))) < 1e-9
    g.close()
    c.close()


def test_observables_blocks(tmp_path, gpu_lib, oracle_mod):
    xml, path = trapped_coulomb(tmp_path, n_part=6, n_bead=16, n_level=2, seed=3, virial=True)
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_path(path)
    c.set_path(path)
    for _ in range(5):
        g.move_attempts(0, 50)
        c.move_attempts(0, 50)
        for o in range(2):
            g.observable_accumulate(o)
            c.observable_accumulate(o)
    eg, ec = g.observable_block(0), c.observable_block(0)
    assert eg.shape == ec.shape and close(eg, ec, 1e-8), (eg, ec)
    # g(r): integer bin counts must agree exactly; the shell-volume normalisation is host FP64 and
    # may differ in the last bit with the compilers' contraction choices.
    hg, hc = g.observable_block(1), c.observable_block(1)
    np.testing.assert_array_equal(hg == 0, hc == 0)
    np.testing.assert_allclose(hg, hc, rtol=1e-13, atol=0)
