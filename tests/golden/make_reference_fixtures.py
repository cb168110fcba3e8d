"""Writes the reference fixtures: outputs of simpimc's own classes (the reference checkout's headers,
compiled against oracle/refshim/ by oracle/build_ref.sh) on seeded inputs.

Each case is one input built by simpimc_gb300.configs with the stated keyword arguments, one path,
and the reference's answers on it:
- GetAction of every action on a list of (b0, b1, particles, level, mode) queries, the NEW copy
  displaced from the stored one on some beads, the density latch set again before each query;
- GetActionGradient on per-bead queries, DActionDBeta and Potential of every action, the kinetic
  VirialEnergy at two windows (NaN where the reference's call fails: DavidPairAction's Potential
  with a long-range part reads its table-ordered v_long_k by the stored k-vector index,
  david_pair_action_class.h:60-61, past the end of that array);
- the input's Algorithm loop (Simulation::Run) with bisection draws from the oracle's counter-based
  stream: every Write's move counters and bisection level, every observable block, the final path;
  for the permuting moves (PermBisectIterative, PermBisectTable) also every Write's per-cycle-length
  counters and the final path permutation at the ring closure. Observable blocks are keyed by the
  observable's place in the input; the Permutation observable is left out (the reference's sector
  lookup has no entries: species_class.h:178-180 generates the sectors only when some already
  exist), and the Sign observable and the sign cofactor of the energy are in the fermion case. A
  PathDump observable's dumps are kept under their own key (`path_dumps_<index>`).

PermBisectTable's cases cycle every particle of their species (n_perm_part = N): with fewer, the
reference leaves the particles owning the end beads out of the action's particle list when the
segment passes a permuted ring closure (perm_bisect_table_class.h:133-141, against
perm_bisect_iterative_class.h:141-146), which the oracle and the GPU library do not copy.

The tests compare the oracle (tests/test_reference_pins.py, CPU) and the GPU library
(tests/test_gpu_reference_fixtures.py) with these numbers; neither needs the reference checkout.
The path dumps are compared with the library's output only (the oracle writes none).

Usage: python tests/golden/make_reference_fixtures.py   (needs the checkout; see oracle/ref.py)
"""
from __future__ import annotations

import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

# name: (config function, keyword arguments, noise added to the generated path)
CASES = {
    "trap_n8_m32": ("trapped_coulomb", dict(n_part=8, n_bead=32, n_level=3, seed=1234, virial=True, n_step_outer=4,
                                            n_step_inner=60), 0.0),
    "trap_adaptive": ("trapped_coulomb", dict(n_part=6, n_bead=32, n_level=2, seed=77, adaptive=True, target_ratio=0.7,
                                              n_step_outer=6, n_step_inner=40), 0.0),
    "david_trap_levels": ("trapped_coulomb", dict(n_part=6, n_bead=32, n_level=3, seed=9, pair="DavidPairAction", n_order=2,
                                                  pair_max_level=2, n_step_outer=3, n_step_inner=50), 0.0),
    "egas_n14": ("electron_gas", dict(n_part=14, n_bead=16, n_level=2, rs=2.0, k_cut_units=4.0, seed=3, structure_factor=True,
                                      n_step_outer=3, n_step_inner=30), 0.3),
    "egas_images": ("electron_gas", dict(n_part=14, n_bead=8, n_level=2, rs=0.5, beta=2.0, k_cut_units=3.0, seed=5, n_images=10,
                                         n_step_outer=3, n_step_inner=30), 0.15),
    "ilkka_egas": ("electron_gas", dict(n_part=14, n_bead=16, n_level=2, rs=2.0, k_cut_units=4.0, seed=11, pair="IlkkaPairAction",
                                        n_step_outer=2, n_step_inner=30), 0.3),
    "david_egas": ("electron_gas", dict(n_part=14, n_bead=16, n_level=2, rs=2.0, k_cut_units=4.0, seed=13, pair="DavidPairAction",
                                        n_order=1, n_step_outer=2, n_step_inner=30), 0.3),
    "bosons_iterative": ("trapped_bosons", dict(n_part=5, n_bead=16, n_level=2, seed=31, coulomb=True, perm="PermBisectIterative",
                                                n_step_outer=3, n_step_inner=80), 0.0),
    "bosons_table": ("trapped_bosons", dict(n_part=4, n_bead=16, n_level=2, seed=37, coulomb=True, perm="PermBisectTable", n_perm_part=4,
                                            n_step_outer=3, n_step_inner=80), 0.0),
    "fermions_iterative": ("trapped_bosons", dict(n_part=4, n_bead=16, n_level=2, seed=43, coulomb=True, fermi=True,
                                                  perm="PermBisectIterative", n_step_outer=3, n_step_inner=80), 0.0),
    "david_bosons": ("trapped_bosons", dict(n_part=4, n_bead=16, n_level=2, seed=53, coulomb=True, perm="PermBisectIterative",
                                            pair="DavidPairAction", n_order=2, pair_max_level=2, n_step_outer=3, n_step_inner=80), 0.0),
    "ilkka_bosons": ("trapped_bosons", dict(n_part=4, n_bead=16, n_level=2, seed=59, coulomb=True, perm="PermBisectIterative",
                                            pair="IlkkaPairAction", pair_max_level=2, n_step_outer=3, n_step_inner=80), 0.0),
    "egas_observables": ("electron_gas", dict(n_part=14, n_bead=16, n_level=2, rs=1.5, beta=4.0, k_cut_units=4.0, seed=79,
                                              structure_factor=True, measure_all=True, n_step_outer=3, n_step_inner=20), 0.2),
    "egas_virial": ("electron_gas", dict(n_part=14, n_bead=16, n_level=2, rs=2.0, k_cut_units=4.0, seed=83, virial=True,
                                         n_step_outer=3, n_step_inner=20), 0.3),
    "ilkka_trap_virial": ("trapped_coulomb", dict(n_part=6, n_bead=32, n_level=3, seed=89, pair="IlkkaPairAction", virial=True,
                                                  n_step_outer=3, n_step_inner=40), 0.0),
    "david_trap_virial": ("trapped_coulomb", dict(n_part=6, n_bead=32, n_level=3, seed=97, pair="DavidPairAction", n_order=2,
                                                  virial=True, n_step_outer=3, n_step_inner=40), 0.0),
    "trap_levels": ("trapped_coulomb", dict(n_part=6, n_bead=32, n_level=3, seed=101, trap_max_level=2, pair_max_level=2,
                                            n_step_outer=3, n_step_inner=40), 0.0),
    "two_species_trap": ("two_species_trap", dict(seed=103), 0.0),
    "egas_perm_table": ("electron_gas", dict(n_part=14, n_bead=16, n_level=2, rs=1.0, beta=4.0, k_cut_units=3.0, seed=107,
                                             perm="PermBisectTable", n_step_outer=2, n_step_inner=30), 0.15),
    "trap_dump": ("trapped_coulomb", dict(n_part=5, n_bead=16, n_level=2, seed=109, path_dump=2, n_step_outer=5, n_step_inner=30),
                  0.0),
    "bosons_dump": ("trapped_bosons", dict(n_part=4, n_bead=16, n_level=2, seed=113, coulomb=True, perm="PermBisectIterative",
                                           path_dump=1, n_step_outer=4, n_step_inner=60), 0.0),
    "egas_perm": ("electron_gas", dict(n_part=14, n_bead=16, n_level=2, rs=1.0, beta=4.0, k_cut_units=3.0, seed=71,
                                       perm="PermBisectIterative", structure_factor=True, n_step_outer=2, n_step_inner=40), 0.15),
}


def build_case(name, workdir):
    """(xml, path) of a case; writes its tables into `workdir`."""
    from simpimc_gb300 import configs
    fn, kw, noise = CASES[name]
    xml, path = getattr(configs, fn)(workdir, **kw)
    path = np.array(path, dtype=np.float64)
    if noise:
        path = path + noise * np.random.default_rng(len(name) * 7919).standard_normal(path.shape)
    return xml, path


def displaced(path, seed):
    """The NEW copy used by the action queries: particle 1 (and the first particle of the second
    species, when there is one) moved on a run of slices."""
    new = path.copy()
    rng = np.random.default_rng(seed)
    M = path.shape[1]
    for p in {1, path.shape[0] // 2 + 1}:
        for b in range(2, min(M, 9)):
            new[p, b] += 0.2 * rng.standard_normal(3)
    return new


def queries(n_actions, n_species, n_total, M, levels):
    """(action, b0, b1, particles, level, mode) of the GetAction queries."""
    parts = [[(0, 1)], [(0, 1), (0, 2)]]
    if n_species > 1:
        parts.append([(1, 1)])
        parts.append([(0, 1), (1, 1)])
    out = []
    for a in range(n_actions):
        for lvl in levels:
            skip = 1 << lvl
            links = min(4, M // skip)
            if links < 2:
                continue
            for pp in parts:
                for mode in (0, 1):
                    out.append((a, 2, 2 + links * skip, pp, lvl, mode))
                    out.append((a, M - skip, M - skip + 2 * skip, pp, lvl, mode))  # across the ring closure
    return out


def gradient_queries(n_actions, n_species, M):
    out = []
    for a in range(n_actions):
        for b in (0, 3, M - 1):
            for mode in (0, 1):
                out.append((a, b, b + 1, [(0, 1)], 0, mode))
                if n_species > 1:
                    out.append((a, b, b + 1, [(1, 1)], 0, mode))
    return out


def reference_answers(name, workdir):
    from oracle import ref
    xml, path = build_case(name, workdir)
    r = ref.RefSim(xml, base_dir=workdir)
    n_actions = xml.count("<Action ")
    n_species = xml.count("<Species ")
    M = path.shape[1]
    levels = [0, 1, 2]
    out = {"xml": xml, "path": path}
    r.set_path(path)
    new = displaced(path, 5)
    r.set_path(new, 1)
    q = queries(n_actions, n_species, path.shape[0], M, levels)
    vals = []
    for a, b0, b1, pp, lvl, mode in q:
        r.reset_rho_k_latch()
        vals.append(r.get_action(a, b0, b1, pp, lvl, mode))
    out["action_queries"] = json.dumps(q)
    out["action_values"] = np.array(vals)
    gq = gradient_queries(n_actions, n_species, M)
    grads = []
    for a, b0, b1, pp, lvl, mode in gq:
        r.reset_rho_k_latch()
        grads.append(r.get_action_gradient(a, b0, b1, pp, lvl, mode))
    out["gradient_queries"] = json.dumps(gq)
    out["gradient_values"] = np.array(grads)
    r.set_path(path)

    def value(f, *args):
        # NaN where the reference's own code fails (an index past the end of one of its arrays)
        try:
            return f(*args)
        except RuntimeError:
            return float("nan")

    out["dactiondbeta"] = np.array([value(r.dactiondbeta, a) for a in range(n_actions)])
    out["potential"] = np.array([value(r.potential, a) for a in range(n_actions)])
    out["virial_energy"] = np.array([[value(r.virial_energy, a, w) for w in (M, 4)] for a in range(n_actions)])
    mstats, blocks, pstats = r.run(xml)
    for m, rows in mstats.items():
        out[f"move_writes_{m}"] = np.array(rows, dtype=np.int64)  # (n_attempt, n_accept, n_level or -1) per Write
    for m, rows in pstats.items():
        out[f"perm_writes_{m}"] = np.array(rows, dtype=np.int64)  # (attempts, accepts) per cycle length, per Write
    import xml.etree.ElementTree as ET
    obs_types = [o.get("type") for o in ET.fromstring(xml).find("Observables")]
    for o, rows in blocks.items():
        # PathDump's rows are its dumps (positions, then (prev, next) per particle, per species)
        out[f"path_dumps_{o}" if obs_types[o] == "PathDump" else f"blocks_{o}"] = np.array(rows)
    out["final_path"] = r.get_path(1)
    if pstats:
        first_species = min(r._species.values())  # (index, n_part) of species 0
        out["final_perm"] = r.get_perm(0, first_species[1])
    r.close()
    return out


def main():
    for name in CASES:
        with tempfile.TemporaryDirectory() as d:
            res = reference_answers(name, d)
        np.savez_compressed(os.path.join(HERE, f"reference_{name}.npz"), **res)
        print(name, {k: np.shape(v) for k, v in res.items() if k != "xml"})


if __name__ == "__main__":
    main()
