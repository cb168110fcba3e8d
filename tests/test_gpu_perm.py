"""GPU parity of the permuting bisection (perm_bisect_class.h:7-133, perm_bisect_iterative_class.h:
7-231, perm_bisect_table_class.h:7-240), the plain bisection of exchanging species, the kinetic
action across a permuted ring closure, the sign cofactor and the Sign / Permutation observables
against the FP64 oracle.

The permutation kernel replays the oracle's random streams, so accept counts, per-cycle-length
counters and the path permutation must agree exactly; positions within 1e-9 (FP64 on both sides,
different summation order of the action changes); estimator values 1e-10 relative.
"""
import math

import numpy as np
import pytest

from simpimc_gb300 import PimcError, Simulation, sweep_chains
from simpimc_gb300.configs import electron_gas, trapped_bosons, trapped_coulomb
from simpimc_gb300.tables import read_table

pytestmark = pytest.mark.gpu


def close(g, c, rel=1e-10):
    g = np.asarray(g, dtype=float)
    c = np.asarray(c, dtype=float)
    return np.all(np.abs(g - c) <= rel * np.maximum(1.0, np.abs(c)))


def replay(g, c, n_part, schedule, n_perm_move=1):
    for m, chunk in schedule:
        g.move_attempts(m, chunk)
        c.move_attempts(m, chunk)
        assert g.move_stats(m) == c.move_stats(m), (m, chunk)
        np.testing.assert_array_equal(g.get_perm(0), c.get_perm(0, n_part))
        assert np.max(np.abs(g.get_path(1) - c.get_path(1))) < 1e-9
    ga, gc = g.perm_stats(n_perm_move, n_part)
    ca, cc = c.perm_stats(n_perm_move, n_part)
    np.testing.assert_array_equal(ga, ca)
    np.testing.assert_array_equal(gc, cc)


@pytest.mark.parametrize("perm,k,coulomb", [("PermBisectIterative", 0, False), ("PermBisectIterative", 0, True),
                                            ("PermBisectTable", 2, False), ("PermBisectTable", 3, True)])
def test_perm_bisection_replays_oracle(tmp_path, gpu_lib, oracle_mod, perm, k, coulomb):
    n = 6
    xml, path = trapped_bosons(tmp_path, n_part=n, beta=4.0, n_bead=16, n_level=2, perm=perm, n_perm_part=k, coulomb=coulomb,
                               seed=21)
    path = path * 0.4  # close paths: exchanges are frequent
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_path(path)
    c.set_path(path)
    replay(g, c, n, [(1, 1), (0, 7), (1, 40), (0, 40), (1, 300), (0, 100), (1, 300)])
    assert sum(c.perm_stats(1, n)[1][1:]) > 0, "no exchange was accepted: the case does not test permutations"
    for a in range(g.n_actions):
        assert close(g.dactiondbeta(a), c.dactiondbeta(a)), a
        assert close(g.virial_energy(a, 16.0), c.virial_energy(a, 16.0), 1e-9), a
    g.close()
    c.close()


@pytest.mark.parametrize("n_bead", [16, 8])
def test_perm_with_long_bisection_and_closure(tmp_path, gpu_lib, oracle_mod, n_bead):
    """Segments of half the ring, or of the whole ring (the kinetic walk of a segment that ends on
    its start bead has no link), cross the closure often; the relabelling moves slice data."""
    n = 5
    xml, path = trapped_bosons(tmp_path, n_part=n, beta=4.0, n_bead=n_bead, n_level=2, perm_level=3, seed=5)
    path = path * 0.3
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_path(path)
    c.set_path(path)
    replay(g, c, n, [(1, 50), (0, 20), (1, 400), (0, 50), (1, 400)])
    g.close()
    c.close()


def test_perm_ewald_electron_gas(tmp_path, gpu_lib, oracle_mod):
    """Exchanges of one spin species with the primitive pair action and its Ewald sum: the density
    update of moved beads on both sides of the closure."""
    xml, path = electron_gas(tmp_path, n_part=8, n_bead=16, n_level=2, rs=1.0, beta=4.0, k_cut_units=3.3, seed=4)
    xml = xml.replace('<Move name="BisectD"', '<Move name="PermU" type="PermBisectIterative" species="eU" n_level="2" />\n    <Move name="BisectD"')
    L = (4.0 * math.pi * 8 / 3.0) ** (1.0 / 3.0) * 1.0
    rng = np.random.default_rng(2)
    centre = rng.uniform(-L / 2, L / 2, size=(8, 1, 3))
    path = centre + 0.2 * rng.standard_normal(path.shape)
    path -= np.rint(path / L) * L
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    pm = 1  # BisectU, PermU, BisectD
    g.set_path(path)
    c.set_path(path)
    for m, chunk in [(pm, 30), (0, 10), (pm, 200), (2, 10), (pm, 200)]:
        g.move_attempts(m, chunk)
        c.move_attempts(m, chunk)
        assert g.move_stats(m) == c.move_stats(m), (m, chunk)
        assert np.max(np.abs(g.get_path(1) - c.get_path(1))) < 1e-9
    np.testing.assert_array_equal(g.get_perm(0), c.get_perm(0, 4))
    for s in range(2):
        assert np.max(np.abs(g.rho_k(s) - c.rho_k(s))) < 1e-9
    for a in range(g.n_actions):
        assert close(g.dactiondbeta(a), c.dactiondbeta(a), 1e-9), a
    g.close()
    c.close()


def test_kinetic_terms_across_a_set_permutation(tmp_path, gpu_lib, oracle_mod):
    n = 5
    xml, path = trapped_bosons(tmp_path, n_part=n, beta=2.0, n_bead=16, n_level=2, seed=9)
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_path(path)
    c.set_path(path)
    pi = [3, 0, 4, 1, 2]
    g.set_perm(0, pi)
    c.set_perm(0, pi)
    np.testing.assert_array_equal(g.get_perm(0), pi)
    assert close(g.dactiondbeta(0), c.dactiondbeta(0))
    for w in (1.0, 5.0, 16.0):
        assert close(g.virial_energy(0, w), c.virial_energy(0, w)), w
    for b0, b1, level in [(12, 20, 0), (12, 20, 1), (14, 18, 1), (0, 16, 0), (15, 16, 0), (0, 16, 2)]:
        for p in range(n):
            for mode in (0, 1):
                assert close(g.get_action(0, b0, b1, [(0, p)], level, mode), c.get_action(0, b0, b1, [(0, p)], level, mode)), (b0, b1, p)
            assert close(g.get_action_gradient(0, b0, b0 + (1 << level), [(0, p)], level, 0),
                         c.get_action_gradient(0, b0, b0 + (1 << level), [(0, p)], level, 0)), (b0, p)
    with pytest.raises(PimcError):
        g.set_perm(0, [0, 0, 1, 2, 3])
    with pytest.raises(PimcError):
        g.total_action()  # the whole-ring paths assume no exchanges
    g.close()
    c.close()


def test_sign_and_permutation_observables(tmp_path, gpu_lib, oracle_mod):
    n = 4
    xml, path = trapped_bosons(tmp_path, n_part=n, beta=4.0, n_bead=16, n_level=2, fermi=True, seed=13)
    path = path * 0.4
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_path(path)
    c.set_path(path)
    for _ in range(30):
        for sim in (g, c):
            sim.move_attempts(0, n)
            sim.move_attempts(1, n)
            for o in range(3):
                sim.observable_accumulate(o)
    for o in range(3):
        gb, cb = g.observable_block(o), c.observable_block(o)
        assert gb.shape == cb.shape and close(gb, cb), (o, gb, cb)
    g.close()
    c.close()


def test_perm_output_and_restart(tmp_path, gpu_lib):
    n = 5
    xml, path = trapped_bosons(tmp_path, n_part=n, beta=4.0, n_bead=16, n_level=2, seed=17, n_step_inner=50, n_step_outer=4)
    xml = xml.replace('<Observable name="Sign" type="Sign" />',
                      '<Observable name="Sign" type="Sign" />\n    <Observable name="path_dump" type="PathDump" />')
    g = Simulation(xml, base_dir=tmp_path)
    g.set_path(path * 0.4)
    g.run()
    g.write_output(tmp_path / "bosons.0.pat")
    d = read_table(tmp_path / "bosons.0.pat")
    att = d["Moves/Perm/perm_attempt"].reshape(-1, n)
    acc = d["Moves/Perm/perm_accept"].reshape(-1, n)
    assert att.shape[0] == 4 and np.all(acc <= att)
    assert d["Moves/Perm/n_perm_type"][0] == n
    perm = d["Observables/path_dump/b/permutation"].reshape(-1, n, 2)
    pi = g.get_perm(0)
    np.testing.assert_array_equal(perm[-1, :, 1], pi)
    np.testing.assert_array_equal(perm[-1, pi, 0], np.arange(n))
    cyc = d["Observables/Permutation/cycles/y"].reshape(4, n)
    np.testing.assert_allclose(cyc.sum(axis=1), 1.0)
    xml2 = xml.replace('init_type="File" file_name="init.xyz" all_beads="1"', 'init_type="Restart" prefix="bosons"')
    r = Simulation(xml2, base_dir=tmp_path)
    np.testing.assert_array_equal(r.get_perm(0), pi)
    np.testing.assert_array_equal(r.get_path(0), g.get_path(0))
    assert r.dactiondbeta(0) == g.dactiondbeta(0)
    r.close()
    g.close()


@pytest.mark.parametrize("pair", ["IlkkaPairAction", "DavidPairAction"])
def test_perm_off_diagonal_pair_actions(tmp_path, gpu_lib, oracle_mod, pair):
    """Off-diagonal pair links keep the reference's label pairing across the permuted link."""
    n = 5
    xml, path = trapped_coulomb(tmp_path, n_part=n, n_bead=16, n_level=2, seed=2, pair=pair, beta=4.0)
    xml = xml.replace('<Move name="Bisect" type="Bisect" species="e" n_level="2" />',
                      '<Move name="Bisect" type="Bisect" species="e" n_level="2" />\n    '
                      '<Move name="Perm" type="PermBisectIterative" species="e" n_level="2" />')
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    path = path * 0.5
    g.set_path(path)
    c.set_path(path)
    replay(g, c, n, [(1, 30), (0, 20), (1, 300), (0, 50), (1, 300)])
    for a in range(g.n_actions):
        assert close(g.dactiondbeta(a), c.dactiondbeta(a), 1e-9), a
    g.close()
    c.close()


def test_sweep_chains_matches_chain_by_chain(tmp_path, gpu_lib, oracle_mod):
    """Many chains in one launch (one CTA per chain) give each chain the results of its own sweep
    calls, bit for bit; one of them replays the oracle."""
    n, sweeps = 6, 5
    together, apart, paths, xmls = [], [], [], []
    for c in range(5):
        d = tmp_path / f"chain{c}"
        xml, path = trapped_bosons(d, n_part=n, beta=4.0, n_bead=16, n_level=2, seed=40 + c)
        xmls.append((xml, d))
        paths.append(path * 0.4)
        for lst in (together, apart):
            s = Simulation(xml, base_dir=d, chain=c)
            s.set_path(paths[-1])
            lst.append(s)
    sweep_chains(together, [0, 1], [n, n], sweeps)
    for s in apart:
        s.sweep([0, 1], [n, n], sweeps)
    for a, b in zip(together, apart):
        for m in range(2):
            assert a.move_stats(m) == b.move_stats(m)
        np.testing.assert_array_equal(a.get_path(0), b.get_path(0))
        np.testing.assert_array_equal(a.get_perm(0), b.get_perm(0))
        ga, _ = a.perm_stats(1, n)
        gb, _ = b.perm_stats(1, n)
        np.testing.assert_array_equal(ga, gb)
    xml, d = xmls[3]
    c = oracle_mod.OracleSim(xml, base_dir=d, chain=3)
    c.set_path(paths[3])
    for _ in range(sweeps):
        c.move_attempts(0, n)
        c.move_attempts(1, n)
    assert together[3].move_stats(1) == c.move_stats(1)
    assert np.max(np.abs(together[3].get_path(1) - c.get_path(1))) < 1e-9
    c.close()
    for s in together + apart:
        s.close()


@pytest.mark.parametrize("n,perm,k", [(80, "PermBisectIterative", 0), (20, "PermBisectTable", 3)])
def test_perm_global_memory_tables(tmp_path, gpu_lib, oracle_mod, n, perm, k):
    """Weight tables past 64 particles and cycle tables past 4096 cycles (20 choose 3 x 3! = 6840)
    live in global memory instead of shared memory; the replay is unchanged."""
    xml, path = trapped_bosons(tmp_path, n_part=n, beta=4.0, n_bead=16, n_level=2, perm=perm, n_perm_part=k, seed=8, sector_max=100)
    path = path * 0.4
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_path(path)
    c.set_path(path)
    replay(g, c, n, [(1, 40), (0, 40), (1, 200)])
    g.close()
    c.close()


def test_signed_pair_correlation_and_structure_factor(tmp_path, gpu_lib, oracle_mod):
    """g(r) and S(k) accumulate with the sign cofactor of fermion species (pair_correlation_class.h:17,
    structure_factor_class.h:17): one exchanging spin species of the electron gas, fermi="1"."""
    xml, path = electron_gas(tmp_path, n_part=8, n_bead=16, n_level=2, rs=1.0, beta=4.0, k_cut_units=3.3, seed=6, structure_factor=True)
    xml = xml.replace('<Species name="eU" n_part="4" lambda="0.5" fermi="0"', '<Species name="eU" n_part="4" lambda="0.5" fermi="1"')
    xml = xml.replace('<Move name="BisectD"', '<Move name="PermU" type="PermBisectIterative" species="eU" n_level="2" />\n    <Move name="BisectD"')
    xml = xml.replace('</Observables>', '  <Observable name="gr" type="PairCorrelation" species_a="eU" species_b="eU" r_min="0." n_r="40" />\n  </Observables>')
    assert 'fermi="1"' in xml and "PermU" in xml
    L = (4.0 * math.pi * 8 / 3.0) ** (1.0 / 3.0)
    rng = np.random.default_rng(3)
    path = rng.uniform(-L / 2, L / 2, size=(8, 1, 3)) + 0.2 * rng.standard_normal(path.shape)
    path -= np.rint(path / L) * L
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_path(path)
    c.set_path(path)
    n_obs = g.n_observables
    signs = []
    for _ in range(40):
        for sim in (g, c):
            sim.move_attempts(1, 8)
            sim.move_attempts(0, 4)
            for o in range(n_obs):
                sim.observable_accumulate(o)
        pi = g.get_perm(0)
        signs.append(pi.tolist())
    assert any(sorted(p) == list(range(4)) and p != list(range(4)) for p in signs), "no exchange happened"
    for o in range(n_obs):
        gb, cb = g.observable_block(o), c.observable_block(o)
        assert gb.shape == cb.shape and close(gb, cb, 1e-9), (o, gb[:8], cb[:8])
    g.close()
    c.close()


def test_sweep_chains_rejects_mismatched_chains(tmp_path, gpu_lib):
    xml_a, path_a = trapped_bosons(tmp_path / "a", n_part=4, beta=2.0, n_bead=8, n_level=2, seed=1)
    xml_b, path_b = trapped_coulomb(tmp_path / "b", n_part=4, n_bead=8, n_level=2, seed=2)
    a = Simulation(xml_a, base_dir=tmp_path / "a")
    b = Simulation(xml_b, base_dir=tmp_path / "b")
    a.set_path(path_a)
    b.set_path(path_b)
    with pytest.raises(PimcError):
        sweep_chains([a, b], [0, 1], [4, 4], 1)  # b has one move
    with pytest.raises(PimcError):
        sweep_chains([b, b], [0], [4], 1)  # one chain twice
    sweep_chains([b], [0], [4], 2)
    assert b.move_stats(0)[0] == 8
    a.close()
    b.close()


@pytest.mark.parametrize("pair", ["BarePairAction", "IlkkaPairAction"])
def test_sweep_chains_plain_bisection_any_actions(tmp_path, gpu_lib, oracle_mod, pair):
    """Chains without exchanges (the electron gas with its Ewald sums, bare or Ilkka pair action)
    also run in one launch, on the permutation kernel's plain bisection; each chain replays the
    oracle."""
    sims, refs = [], []
    for c in range(3):
        d = tmp_path / f"egas{c}"
        xml, path = electron_gas(d, n_part=14, n_bead=16, n_level=2, rs=2.0, k_cut_units=4.0, seed=9 + c, pair=pair)
        L = ((4.0 * math.pi * 14 / 3.0) ** (1.0 / 3.0)) * 2.0
        path = np.random.default_rng(50 + c).uniform(-L / 2, L / 2, size=path.shape)
        g = Simulation(xml, base_dir=d, chain=c)
        o = oracle_mod.OracleSim(xml, base_dir=d, chain=c)
        g.set_path(path)
        o.set_path(path)
        sims.append(g)
        refs.append(o)
    sweep_chains(sims, [0, 1], [7, 7], 6)
    for g, o in zip(sims, refs):
        for _ in range(6):
            o.move_attempts(0, 7)
            o.move_attempts(1, 7)
        for m in range(2):
            assert g.move_stats(m) == o.move_stats(m), m
        assert np.max(np.abs(g.get_path(1) - o.get_path(1))) < 1e-9
        for s in range(2):
            assert np.max(np.abs(g.rho_k(s) - o.rho_k(s))) < 1e-9
        g.close()
        o.close()
