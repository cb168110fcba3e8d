"""The oracle against the reference itself (CPU).

tests/golden/reference_*.npz hold the answers of simpimc's own Action, Bisect and Observable classes
— the reference checkout's headers, unmodified, compiled against the shim in oracle/refshim/ — on
seeded inputs: GetAction / GetActionGradient queries, DActionDBeta, Potential, VirialEnergy, and the
input's whole Algorithm loop (bisection with the oracle's random stream, measurements, Write events,
adaptive bisection levels). Cases: the 8-particle trapped Coulomb system (N = 8, M = 32, level 3), an
adaptive-level trap, a trap with actions of max_level 2, two species of different masses in one trap,
DavidPairAction with tables at levels 0-2, 14-electron gases with the bare
Ewald, Ilkka and David pair actions, one with periodic images in the kinetic action
(n_images = 10 on a small box) and one measuring the periodic g(r) and S(k), the virial estimator
on an electron gas and on IlkkaPairAction and DavidPairAction traps, trapped Coulomb bosons with the permuting moves
(PermBisectIterative; PermBisectTable over every particle), whose per-cycle-length counters and
final path permutation are compared too, trapped Coulomb fermions (the Sign observable and the
energy's sign cofactor), trapped bosons with DavidPairAction / IlkkaPairAction tables above
level 0 under PermBisectIterative, electron gases whose up spins exchange by either permuting
move (Ewald sums), and runs with a PathDump observable (its dumps are compared on the GPU only).

The oracle must reproduce every number (tolerances in tests/reference_cases.py). Where the reference
checkout is present, the fixtures are also regenerated from it and must equal the committed files,
which pins the fixtures to the reference code as built here.
"""
import numpy as np
import pytest

from reference_cases import check_against_fixture, fixture_names, generator, load, n_observables, species_counts


def _oracle_blocks(sim, xml):
    sim.run()
    # the oracle builds no PathDump (bookkeeping only), which the cases place after the others
    return {o: sim.blocks(o) for o in range(sim.n_observables)}


def _oracle_move_writes(sim, xml):
    return {m: sim.move_writes(m)[:, :3] for m in range(sim.n_moves)}


def _oracle_perm_writes(sim, xml):
    out = {}
    for m in range(sim.n_moves):
        rows = sim.move_writes(m)
        if rows.shape[1] > 3:
            out[m] = rows[:, 3:].reshape(rows.shape[0], 2, -1)
    return out


@pytest.mark.parametrize("name", fixture_names())
def test_oracle_matches_reference_fixture(tmp_path, oracle_mod, name):
    def make(xml, d):
        return oracle_mod.OracleSim(xml, base_dir=d)

    sim, errs = check_against_fixture(make, name, tmp_path, _oracle_blocks, lambda s: s.get_path(1), _oracle_move_writes,
                                      perm_writes=_oracle_perm_writes, final_perm=lambda s, xml: s.get_perm(0, species_counts(xml)[0]))
    sim.close()
    assert not errs, errs[:10]


def test_fixture_cases_cover_the_hot_path_classes():
    names = fixture_names()
    assert len(names) >= 22
    xmls = " ".join(str(load(n)["xml"]) for n in names)
    for cls in ("Kinetic", "HarmonicTrap", "BarePairAction", "IlkkaPairAction", "DavidPairAction", 'adaptive="1"', 'n_images="10"',
                "StructureFactor", "PairCorrelation", "use_virial_estimator", "PermBisectIterative", "PermBisectTable", 'fermi="1"', 'type="Sign"'):
        assert cls in xmls, cls


@pytest.mark.parametrize("name", fixture_names())
def test_reference_build_reproduces_fixture(tmp_path, name):
    """Regenerates one fixture from the reference checkout (skipped where it is absent)."""
    from oracle import ref
    if not ref.available():
        pytest.skip("reference checkout absent")
    gen = generator()
    fresh = gen.reference_answers(name, str(tmp_path))
    old = load(name)
    assert sorted(fresh) == sorted(old)
    for k, v in fresh.items():
        if k in ("xml", "action_queries", "gradient_queries"):
            assert str(v) == str(old[k]), k
        else:
            np.testing.assert_array_equal(np.asarray(v), old[k], err_msg=k)
