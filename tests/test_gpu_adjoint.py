"""Exact ("adjoint") action gradient, the whole-ring action, the HMC move and the adjoint virial
estimator on the GPU, against the FP64 oracle, central finite differences and the reference's own
gradient.

Tolerances (FP64 on both sides):
  * whole-ring action and gradient vs the oracle: |gpu - cpu| <= 1e-10 * max(1, |cpu|);
  * gradient vs central differences of the GPU's own action, h = 1e-5: <= 1e-6 * max(1, |g|)
    (O(h^2) truncation plus |S| * 1e-16 / h rounding; 1e-5 on the large electron gas, whose
    action is ~1e5);
  * vs the reference gradient (Action::GetActionGradient): kinetic exact (1e-10); the pair
    action's eps = 1e-4 central difference (pair_action_class.h:135-155) within 1e-6;
  * HMC trajectories: identical accept counts, positions within 1e-8.
"""
import numpy as np
import pytest

from simpimc_gb300 import Simulation
from simpimc_gb300.configs import electron_gas, trapped_coulomb

pytestmark = pytest.mark.gpu


def close(g, c, rel):
    g, c = np.asarray(g, float), np.asarray(c, float)
    return np.all(np.abs(g - c) <= rel * np.maximum(1.0, np.abs(c)))


def egas_random(tmp_path, n_part, n_bead, rs, k_units, seed, beta=None):
    kw = dict(n_part=n_part, n_bead=n_bead, n_level=2, rs=rs, k_cut_units=k_units, seed=seed)
    if beta is not None:
        kw["beta"] = beta
    xml, path = electron_gas(tmp_path, **kw)
    L = (4 * np.pi * n_part / 3) ** (1 / 3) * rs
    path = np.random.default_rng(seed).uniform(-L / 2, L / 2, size=path.shape)
    return xml, path


@pytest.fixture(scope="module")
def systems(tmp_path_factory, gpu_lib, oracle_mod):
    d = tmp_path_factory.mktemp("adj")
    out = []
    xml, path = trapped_coulomb(d, n_part=6, n_bead=16, n_level=2, seed=13)
    out.append((xml, path))
    out.append(egas_random(d, 10, 8, 2.0, 4.0, 17))
    return d, out


def test_total_action_and_gradient_match_oracle(systems, oracle_mod):
    d, items = systems
    for xml, path in items:
        g = Simulation(xml, base_dir=d)
        c = oracle_mod.OracleSim(xml, base_dir=d)
        g.set_path(path)
        c.set_path(path)
        for a in list(range(g.n_actions)) + [-1]:
            assert close(g.total_action(a), c.total_action(a), 1e-10), a
            assert close(g.action_gradient_path(a), c.action_gradient_path(a), 1e-10), a
        g.close()
        c.close()


def test_gradient_matches_central_differences(systems):
    d, items = systems
    rng = np.random.default_rng(3)
    h = 1e-5
    for xml, path in items:
        g = Simulation(xml, base_dir=d)
        g.set_path(path)
        grad = g.action_gradient_path()
        for _ in range(8):
            i = tuple(int(rng.integers(n)) for n in path.shape)
            pp = path.copy()
            pp[i] += h
            g.set_path(pp)
            sp = g.total_action()
            pp[i] -= 2 * h
            g.set_path(pp)
            sm = g.total_action()
            fd = (sp - sm) / (2 * h)
            assert abs(grad[i] - fd) <= 1e-6 * max(1.0, abs(grad[i])), (i, grad[i], fd)
        g.close()


def test_exact_gradient_against_reference_gradient(systems):
    """Action::GetActionGradient of one particle: the reference's kinetic gradient is exact; its pair
    gradient is a central difference with eps = 1e-4 of the same primitive action."""
    d, items = systems
    xml, path = items[0]
    g = Simulation(xml, base_dir=d)
    g.set_path(path)
    for p in range(3):
        for b0 in (0, 5, 15):
            ref_k = g.get_action_gradient(0, b0, b0 + 1, [(0, p)], 0, 0)
            exa_k = g.get_action_gradient_exact(0, b0, b0 + 1, [(0, p)], 0, 0)
            assert close(exa_k, ref_k, 1e-10), (p, b0, exa_k, ref_k)
            ref_p = g.get_action_gradient(2, b0, b0 + 1, [(0, p)], 0, 0)
            exa_p = g.get_action_gradient_exact(2, b0, b0 + 1, [(0, p)], 0, 0)
            assert close(exa_p, ref_p, 1e-6), (p, b0, exa_p, ref_p)
            # the trap, which the reference does not differentiate (trap_class.h), is 2 cofactor_a r
            assert np.all(g.get_action_gradient(1, b0, b0 + 1, [(0, p)], 0, 0) == 0.)
    g.close()


@pytest.mark.parametrize("which", [0, 1])
def test_hmc_replays_oracle(systems, oracle_mod, which):
    d, items = systems
    xml, path = items[which]
    if which == 0:
        xml = xml.replace('<Move name="Bisect" type="Bisect" species="e" n_level="2" />',
                          '<Move name="Bisect" type="HMC" step_size="0.01" n_steps="10" />')
    else:
        xml = xml.replace('<Move name="BisectU" type="Bisect" species="eU" n_level="2" />',
                          '<Move name="BisectU" type="HMC" step_size="0.01" n_steps="10" />')
    g = Simulation(xml, base_dir=d)
    c = oracle_mod.OracleSim(xml, base_dir=d)
    g.set_path(path)
    c.set_path(path)
    g.move_attempts(0, 12)
    c.move_attempts(0, 12)
    assert g.move_counters(0)[3] == c.move_stats(0)[2], (g.move_counters(0), c.move_stats(0))
    assert c.move_stats(0)[2] > 0
    assert np.max(np.abs(g.get_path(0) - c.get_path(0))) < 1e-8
    assert close(g.total_action(), c.total_action(), 1e-10)
    g.close()
    c.close()


def test_adjoint_virial_energy_matches_oracle(tmp_path, gpu_lib, oracle_mod):
    xml, path = trapped_coulomb(tmp_path, n_part=5, n_bead=16, n_level=2, seed=29, virial=True)
    xml = xml.replace('use_virial_estimator="1"', 'use_virial_estimator="1" use_adjoint_gradient="1"')
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_path(path)
    c.set_path(path)
    g.observable_accumulate(0)
    c.observable_accumulate(0)
    assert close(g.observable_block(0), c.observable_block(0), 1e-10)
    g.close()
    c.close()


def test_electron_gas_rs4_gradient_on_32_configurations(tmp_path, gpu_lib, oracle_mod):
    """The adjoint workload's system: r_s = 4, N = 128, beta = 16, M = 256, |k| < 17 (2 pi / L).
    32 seeded random path configurations, 3 coordinates each against central differences of the
    whole-ring action (h = 1e-5, FP64); the pair part against the reference gradient; one
    configuration's full gradient against the oracle."""
    rng = np.random.default_rng(2024)
    for cfg in range(32):
        xml, path = egas_random(tmp_path, 128, 256, 4.0, 17.0, 1000 + cfg, beta=16.0)
        g = Simulation(xml, base_dir=tmp_path)
        if cfg == 0:
            assert 9000 < g.n_k < 11000, g.n_k
        g.set_path(path)
        h = 1e-5
        coords = [tuple(int(rng.integers(n)) for n in path.shape) for _ in range(3)]
        # Per action: on random paths the kinetic action alone is ~1e8, so a difference of the
        # total would carry ~1e-16 |S| / h = 1e-3 of rounding; each action's own difference is
        # compared within its truncation plus that rounding bound.
        for a in range(g.n_actions):
            grad = g.action_gradient_path(a)
            s0 = abs(g.total_action(a))
            for i in coords:
                pp = path.copy()
                pp[i] += h
                g.set_path(pp)
                sp = g.total_action(a)
                pp[i] -= 2 * h
                g.set_path(pp)
                sm = g.total_action(a)
                g.set_path(path)
                fd = (sp - sm) / (2 * h)
                tol = 1e-6 * max(1.0, abs(grad[i])) + 8e-16 * s0 / h
                assert abs(grad[i] - fd) <= tol, (cfg, a, i, grad[i], fd, tol)
        grad = g.action_gradient_path()
        if cfg < 4:
            # The reference differentiates only the short-range pair part (pair_action_class.h:
            # 305-337; no long-range gradient in the Bare action): compare on the same input with
            # the Ewald part switched off.
            x_sr = xml.replace('use_long_range="1"', 'use_long_range="0"')
            gs = Simulation(x_sr, base_dir=tmp_path)
            gs.set_path(path)
            p, b = int(rng.integers(64)), int(rng.integers(256))
            ref = gs.get_action_gradient(2, b, b + 1, [(0, p)], 0, 0)
            exa = gs.get_action_gradient_exact(2, b, b + 1, [(0, p)], 0, 0)
            assert close(exa, ref, 1e-6), (cfg, p, b, exa, ref)
            gs.close()
        if cfg == 0:
            c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
            c.set_path(path)
            assert close(grad, c.action_gradient_path(), 1e-10)
            c.close()
        g.close()
