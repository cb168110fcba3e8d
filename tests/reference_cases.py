"""Shared driver of the reference-fixture tests (tests/golden/reference_*.npz).

`check_against_fixture(sim, name, workdir, ...)` replays a fixture's queries and Algorithm run on any
object with the Simulation / OracleSim surface and compares the answers with the ones the reference's
own classes gave (tests/golden/make_reference_fixtures.py). Tolerances are the parity tests' FP64
ones: action values, dS/dbeta, potentials, virial energies and energy blocks 1e-10 relative; the
central-difference pair gradients (eps = 1e-4, pair_action_class.h:135-155) 1e-8 relative; path
coordinates 1e-9; g(r) and S(k) blocks 1e-10 relative; move counters, bisection levels, the permuting
moves' per-cycle-length counters and the final path permutation exact.
"""
from __future__ import annotations

import importlib.util
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def generator():
    spec = importlib.util.spec_from_file_location("make_reference_fixtures", os.path.join(GOLDEN, "make_reference_fixtures.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def fixture_names():
    return sorted(f[len("reference_"):-4] for f in os.listdir(GOLDEN) if f.startswith("reference_") and f.endswith(".npz"))


def load(name):
    with np.load(os.path.join(GOLDEN, f"reference_{name}.npz")) as z:
        return {k: z[k] for k in z.files}


def n_observables(xml):
    """Observables declared in the input's <Observables> section."""
    import xml.etree.ElementTree as ET
    return len(list(ET.fromstring(xml).find("Observables")))


def species_counts(xml):
    """n_part of each species, in input order."""
    import xml.etree.ElementTree as ET
    return [int(s.get("n_part")) for s in ET.fromstring(xml).find("Particles")]


def permuting_moves(xml):
    """{move index: species index} of the input's permuting moves."""
    import xml.etree.ElementTree as ET
    root = ET.fromstring(xml)
    names = [s.get("name") for s in root.find("Particles")]
    return {i: names.index(m.get("species")) for i, m in enumerate(root.find("Moves"))
            if m.get("type") in ("PermBisectIterative", "PermBisectTable")}


def _close(a, b, rel):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    return a.shape == b.shape and bool(np.all(np.abs(a - b) <= rel * np.maximum(1.0, np.abs(b))))


def check_against_fixture(make_sim, name, workdir, run_blocks, final_path, move_writes=None, grad_rel=1e-8, perm_writes=None,
                          final_perm=None, path_dumps=None):
    """make_sim(xml, workdir) -> a fresh simulation; run_blocks(sim, xml) -> {obs: [blocks]} after
    running the Algorithm; final_path(sim) -> positions; move_writes(sim, xml) -> {move: rows} or None;
    perm_writes(sim, xml) -> {permuting move: [Write, (attempts, accepts), cycle length]} and
    final_perm(sim, xml) -> the first species' path permutation, required when the fixture has them;
    path_dumps(sim, xml) -> {PathDump observable: [dump, values]} (None: not compared)."""
    gen = generator()
    fx = load(name)
    xml, path = gen.build_case(name, workdir)
    assert xml == str(fx["xml"]), "the case's input no longer matches the fixture (regenerate the fixtures)"
    assert np.array_equal(path, fx["path"])
    sim = make_sim(xml, workdir)
    sim.set_path(path)
    sim.set_path(gen.displaced(path, 5), 1)
    has_latch = hasattr(sim, "reset_rho_k_latch")
    errs = []
    for (a, b0, b1, pp, lvl, mode), want in zip(json.loads(str(fx["action_queries"])), fx["action_values"]):
        if has_latch:
            sim.reset_rho_k_latch()
        got = sim.get_action(a, b0, b1, [tuple(p) for p in pp], lvl, mode)
        if not _close(got, want, 1e-10):
            errs.append(("action", a, b0, b1, pp, lvl, mode, got, float(want)))
    for (a, b0, b1, pp, lvl, mode), want in zip(json.loads(str(fx["gradient_queries"])), fx["gradient_values"]):
        if has_latch:
            sim.reset_rho_k_latch()
        got = sim.get_action_gradient(a, b0, b1, [tuple(p) for p in pp], lvl, mode)
        if not _close(got, want, grad_rel):
            errs.append(("gradient", a, b0, b1, pp, lvl, mode, list(got), list(want)))
    sim.set_path(path)
    n_actions = len(fx["dactiondbeta"])
    M = path.shape[1]
    for a in range(n_actions):
        for key, got in (("dactiondbeta", sim.dactiondbeta(a)), ("potential", sim.potential(a))):
            if np.isnan(fx[key][a]):  # the reference's call fails there (see the fixture generator)
                continue
            if not _close(got, fx[key][a], 1e-10):
                errs.append((key, a, got, float(fx[key][a])))
        for i, w in enumerate((M, 4)):
            got = sim.virial_energy(a, w)
            if not _close(got, fx["virial_energy"][a][i], 1e-10):
                errs.append(("virial", a, w, got, float(fx["virial_energy"][a][i])))
    blocks = run_blocks(sim, xml)
    for o, rows in blocks.items():
        want = fx.get(f"blocks_{o}")
        if want is None:
            continue
        got = np.array(rows)
        if want.size == 0:
            if got.size:
                errs.append(("blocks", o, "unexpected blocks"))
            continue
        if not _close(got, want, 1e-10):
            errs.append(("blocks", o, got.shape, want.shape, float(np.max(np.abs(got - want))) if got.shape == want.shape else None))
    if move_writes is not None:
        for m, rows in move_writes(sim, xml).items():
            want = fx[f"move_writes_{m}"]
            got = np.array(rows, dtype=np.int64)
            if want[:, 2].max() < 0:  # not adaptive: no level dataset
                want, got = want[:, :2], got[:, :2]
            if not np.array_equal(got, want):
                errs.append(("move writes", m, got.tolist(), want.tolist()))
    perm_keys = [k for k in fx if k.startswith("perm_writes_")]
    if perm_keys:
        assert perm_writes is not None and final_perm is not None, "a permuting-move fixture needs its counters and permutation"
        got_pw = perm_writes(sim, xml)
        for k in perm_keys:
            m = int(k[len("perm_writes_"):])
            got = np.asarray(got_pw.get(m, []), dtype=np.int64)
            if not np.array_equal(got, fx[k]):
                errs.append(("perm writes", m, got.tolist(), fx[k].tolist()))
        got = np.asarray(final_perm(sim, xml), dtype=np.int64)
        if not np.array_equal(got, fx["final_perm"]):
            errs.append(("final perm", got.tolist(), fx["final_perm"].tolist()))
    if path_dumps is not None:
        got_pd = path_dumps(sim, xml)
        for k in [k for k in fx if k.startswith("path_dumps_")]:
            o = int(k[len("path_dumps_"):])
            got, want = np.asarray(got_pd.get(o, []), dtype=float), fx[k]
            if got.shape != want.shape or np.max(np.abs(got - want)) >= 1e-9:
                errs.append(("path dumps", o, got.shape, want.shape))
    fp = final_path(sim)
    if not (fp.shape == fx["final_path"].shape and np.max(np.abs(fp - fx["final_path"])) < 1e-9):
        errs.append(("final path", float(np.max(np.abs(fp - fx["final_path"]))) if fp.shape == fx["final_path"].shape else None))
    return sim, errs
