"""Run output under the reference's dataset paths and restart from its path dump.

`pimc_write_output` writes Moves/<name>/{type, n_attempt, n_accept, x}, the Energy / g(r) datasets
and Observables/<path dump>/<species>/{n_dump, positions, permutation} (move_class.h:45-53,
energy_class.h:232-272, pair_correlation_class.h:76-120, path_dump_class.h:28-66) in the table
container. The checks compare every dataset with the blocks and counters the library holds, and a
species created with init_type="Restart" (species_class.h:336-377) with the last dump, bit for bit.
"""
import numpy as np
import pytest

from simpimc_gb300 import Simulation
from simpimc_gb300.configs import trapped_coulomb
from simpimc_gb300.tables import read_table

pytestmark = pytest.mark.gpu


def with_path_dump(xml):
    return xml.replace('<Observable name="gr"', '<Observable name="path_dump" type="PathDump" skip="2" />\n    <Observable name="gr"')


def test_output_datasets_and_restart(tmp_path, gpu_lib):
    xml, path = trapped_coulomb(tmp_path, n_part=6, n_bead=16, n_level=2, seed=3, n_step_inner=20, n_step_outer=5, virial=True)
    xml = with_path_dump(xml)
    g = Simulation(xml, base_dir=tmp_path)
    g.set_path(path)
    g.run()
    out = tmp_path / "run.0.pat"
    g.write_output(out)
    d = read_table(out)

    # Moves: one value per Write event (5), summing to the move's counters.
    assert d["Moves/Bisect/type"] == "Bisect"
    att, acc = d["Moves/Bisect/n_attempt"], d["Moves/Bisect/n_accept"]
    cnt = g.move_counters(0)  # total attempts, block attempts, block accepts, total accepts, level-0 tests
    assert att.size == 5 and int(att.sum()) == int(cnt[0]) and int(acc.sum()) == int(cnt[3])
    np.testing.assert_array_equal(d["Moves/Bisect/x"], acc / att)

    # Energy: total and per-action series equal the library's blocks.
    e_blocks = np.array(g.blocks(0))
    np.testing.assert_array_equal(d["Observables/Energy/total/x"], e_blocks[:, 0])
    for i, name in enumerate(["Kinetic", "Trap", "Coulomb"]):
        np.testing.assert_array_equal(d[f"Observables/Energy/{name}/x"], e_blocks[:, 1 + i])
    assert d["Observables/Energy/total/data_type"] == "scalar"

    # g(r): histogram blocks appended, bin centres of the reference's formula.
    gr = np.array(g.blocks(2))
    np.testing.assert_array_equal(d["Observables/gr/y"], gr.ravel())
    assert d["Observables/gr/x"].size == 199 and d["Observables/gr/species_a"] == "e"

    # Path dump: every second Write (skip = 2) of 5: dumps at calls 0, 2, 4.
    assert d["Observables/path_dump/type"] == "PathDump"
    n_dump = int(d["Observables/path_dump/e/n_dump"][0])
    assert n_dump == 3
    pos = d["Observables/path_dump/e/positions"].reshape(n_dump, 6, 16, 3)
    np.testing.assert_array_equal(pos[-1], g.get_path(0))
    perm = d["Observables/path_dump/e/permutation"].reshape(n_dump, 6, 2)
    np.testing.assert_array_equal(perm[..., 0], np.tile(np.arange(6), (n_dump, 1)))

    # Restart: a new simulation of the same system starts from the last dump.
    xml2 = xml.replace('init_type="File" file_name="init.xyz" all_beads="1"', 'init_type="Restart" prefix="run"')
    assert xml2 != xml
    r = Simulation(xml2, base_dir=tmp_path)
    np.testing.assert_array_equal(r.get_path(0), pos[-1])
    np.testing.assert_array_equal(r.get_path(1), pos[-1])
    # and its actions see that path
    assert r.dactiondbeta(0) == g.dactiondbeta(0)
    r.close()
    g.close()


def test_restart_without_dump_is_an_input_error(tmp_path, gpu_lib):
    xml, path = trapped_coulomb(tmp_path, n_part=4, n_bead=8, n_level=2, seed=2)
    (tmp_path / "empty.0.pat").write_text("# nothing\nObservables/path_dump/e/n_dump 1\n0\n")
    xml2 = xml.replace('init_type="File" file_name="init.xyz" all_beads="1"', 'init_type="Restart" prefix="empty"')
    with pytest.raises(Exception):
        Simulation(xml2, base_dir=tmp_path)
