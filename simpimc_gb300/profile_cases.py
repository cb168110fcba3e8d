"""Small fixed workloads for profiler captures (one warm-up launch, then the launches to capture).

    python -m simpimc_gb300.profile_cases batch    # 256 uneven trapped-Coulomb chains: 1 + 1 sweep launches
    python -m simpimc_gb300.profile_cases hmc      # the same chains with the HMC move: 1 + 1 HMC launches
    python -m simpimc_gb300.profile_cases hmc_egas # single-chain HMC on the 128-electron gas: 1 + 1 attempts
    python -m simpimc_gb300.profile_cases egas     # 66-electron gas: 1 + 1 sweep launches (528 attempts each)
    python -m simpimc_gb300.profile_cases egas_phases  # the same system: per-attempt phase cycles of the
                                                       # sweep kernel's block 0 at one and two groups
    python -m simpimc_gb300.profile_cases large32  # 1024-electron gas, FP32 mode: 1 + 1 launches of 64 attempts
    python -m simpimc_gb300.profile_cases bosons   # 32 trapped bosons: Bisect and PermBisectIterative, 1 + 1 sweeps
    python -m simpimc_gb300.profile_cases chains   # 608 such chains: 1 + 1 launches of one sweep each (pimc_sweep_chains)
    python -m simpimc_gb300.profile_cases egas_chains  # 38, 152 and 304 66-electron-gas chains: a warm-up
                                                       # launch, then one timed sweep each (pimc_sweep_chains)
    python -m simpimc_gb300.profile_cases egas_chains32  # the same in the FP32 density mode

The first two hold well under 100 MB on the device, the third about 1.3 GB; a capture of the
second launch (`-k regex:<Kernel> -s 1 -c 1`) ends in seconds (the large case with one or two
sections rather than the full set).
"""
from __future__ import annotations

import math
import sys
import tempfile

import numpy as np


def batch_case(d):
    from . import ChainBatch
    from .configs import batched_trap_chains
    items = batched_trap_chains(d, n_chains=256, seed0=1000, n_level=3)
    b = ChainBatch([x for x, _ in items], base_dir=d)
    b.set_paths(np.concatenate([p.ravel() for _, p in items]))
    b.set_tiles(8, 16, 8)
    b.sweeps(1)
    b.sweeps(1)
    b.synchronize()
    att, acc = b.counters()
    print(f"batch ok: {int(att.sum())} attempts, acceptance {acc.sum() / att.sum():.4f}")


def hmc_case(d):
    """One HMC attempt per chain (leapfrog step 0.005, 10 steps) on clusters of 4 blocks per chain."""
    from . import ChainBatch
    from .configs import batched_trap_chains
    items = batched_trap_chains(d, n_chains=256, seed0=1000, n_level=3, hmc=(0.005, 10))
    b = ChainBatch([x for x, _ in items], base_dir=d)
    b.set_paths(np.concatenate([p.ravel() for _, p in items]))
    b.sweeps(2)
    b.hmc_cluster = 4
    b.hmc_attempts(1)
    b.hmc_attempts(1)
    b.synchronize()
    att, acc = b.hmc_counters()
    print(f"hmc ok: {int(att.sum())} attempts, acceptance {acc.sum() / att.sum():.4f}")


def egas_case(d):
    from . import Simulation
    from .configs import electron_gas
    xml, path = electron_gas(d, n_part=66, rs=2.0, beta=8.0, n_bead=128, k_cut_units=12.0, n_level=4, seed=20261203)
    s = Simulation(xml, base_dir=d)
    s.set_path(path)
    reps = 33 * math.ceil(128 / 16)
    s.sweep([0, 1], [1, 1], reps)
    s.sweep([0, 1], [1, 1], reps)
    s.synchronize()
    print(f"egas ok: {s.move_counters(0)[0] + s.move_counters(1)[0]} attempts")


def hmc_egas_case(d):
    """The single-chain HMC move (leapfrog 0.01 x 10 on the exact gradient, FP64) on the 128-electron
    gas (r_s = 4, beta = 16, M = 256, |k| < 17 (2 pi / L)) after two bisection sweeps."""
    from . import Simulation
    from .configs import electron_gas
    xml, path = electron_gas(d, n_part=128, rs=4.0, beta=16.0, n_bead=256, k_cut_units=17.0, n_level=4, seed=4242)
    xml = xml.replace('<Move name="BisectD" type="Bisect" species="eD" n_level="4" />',
                      '<Move name="BisectD" type="Bisect" species="eD" n_level="4" />\n'
                      '    <Move name="HMC" type="HMC" step_size="0.01" n_steps="10" />')
    s = Simulation(xml, base_dir=d)
    s.set_path(path)
    s.sweep([0, 1], [1, 1], 2 * 64 * 16)
    s.move_attempts(2, 1)
    s.move_attempts(2, 1)
    s.synchronize()
    print(f"hmc_egas ok: {s.move_counters(2)[0]} attempts, {s.n_k} k-vectors")
    s.close()


def egas_phases_case(d):
    """Per-attempt cycles of each phase of the sweep kernel's block 0 (pimc_sweep_timing) on the
    66-electron gas, one sweep at one group (wave 1) and at the automatic group count."""
    from . import Simulation
    from .configs import electron_gas
    xml, path = electron_gas(d, n_part=66, rs=2.0, beta=8.0, n_bead=128, k_cut_units=12.0, n_level=4, seed=20261203)
    s = Simulation(xml, base_dir=d)
    s.set_path(path)
    reps = 33 * math.ceil(128 / 16)
    for wave in (1, 0):
        s.set_sweep_wave(wave)
        s.sweep([0, 1], [1, 1], reps)  # warm-up
        s.synchronize()
        s.sweep_timing(1)
        a0 = s.move_counters(0)[0] + s.move_counters(1)[0]
        s.sweep([0, 1], [1, 1], reps)
        s.synchronize()
        n = s.move_counters(0)[0] + s.move_counters(1)[0] - a0
        ph = s.sweep_timing(0)
        print(f"wave {wave or 'auto'}: cycles per attempt of block 0 over {n} attempts")
        print("  " + ", ".join(f"{k} {v / n:.0f}" for k, v in ph.items() if v))
    s.close()


def large32_case(d):
    from . import Simulation
    from .configs import electron_gas
    xml, path = electron_gas(d, n_part=1024, rs=1.0, beta=4.0, n_bead=512, k_cut_units=23.0, n_level=4, seed=777)
    s = Simulation(xml, base_dir=d)
    s.set_precision(32)
    s.set_path(path)
    s.sweep([0, 1], [1, 1], 32)
    s.sweep([0, 1], [1, 1], 32)
    s.synchronize()
    print(f"large32 ok: {s.move_counters(0)[0] + s.move_counters(1)[0]} attempts, {s.n_k} k-vectors")


def bosons_case(d):
    from . import Simulation
    from .configs import trapped_bosons
    xml, path = trapped_bosons(d, n_part=32, beta=4.0, n_bead=32, n_level=3, seed=77)
    s = Simulation(xml, base_dir=d)
    s.set_path(path * 0.4)
    s.sweep([0, 1], [32, 32], 1)
    s.sweep([0, 1], [32, 32], 1)
    s.synchronize()
    print(f"bosons ok: {s.move_counters(0)[0] + s.move_counters(1)[0]} attempts")


def chains_case(d):
    import os

    from . import Simulation, sweep_chains
    from .configs import trapped_bosons
    sims = []
    for c in range(608):
        dc = os.path.join(d, f"c{c}")
        xml, path = trapped_bosons(dc, n_part=32, beta=4.0, n_bead=32, n_level=3, seed=77 + c)
        s = Simulation(xml, base_dir=dc, chain=c)
        s.set_path(path * 0.4)
        sims.append(s)
    sweep_chains(sims, [0, 1], [32, 32], 1)
    sweep_chains(sims, [0, 1], [32, 32], 1)
    print(f"chains ok: {sum(s.move_counters(0)[0] + s.move_counters(1)[0] for s in sims)} attempts")


def egas_chains_case(d, precision=64):
    """Throughput of many 66-electron-gas chains (r_s = 2, beta = 8, M = 128, level 4) in one
    launch: one sweep is 33 attempts of each species' move, 8 times (528 attempts, 15
    moved beads each). Wall clock around the call, which returns after its launch has finished.
    precision=32: the chains' FP32 density mode."""
    import os
    import time

    from . import Simulation, sweep_chains
    from .configs import electron_gas
    for nc in (38, 152, 304):
        sims = []
        for c in range(nc):
            dc = os.path.join(d, f"c{nc}_{c}")
            xml, path = electron_gas(dc, n_part=66, rs=2.0, beta=8.0, n_bead=128, k_cut_units=12.0, n_level=4, seed=20261203 + c)
            s = Simulation(xml, base_dir=dc, chain=c)
            s.set_precision(precision)
            s.set_path(path)
            sims.append(s)
        sweep_chains(sims, [0, 1], [33, 33], 1)  # warm-up
        b0 = sum(s.move_counters(0)[0] + s.move_counters(1)[0] for s in sims)
        t0 = time.perf_counter()
        sweep_chains(sims, [0, 1], [33, 33], 8)
        el = time.perf_counter() - t0
        att = sum(s.move_counters(0)[0] + s.move_counters(1)[0] for s in sims) - b0
        print(f"{nc} chains: {att * 15 / el / 1e6:.3f} M bead-moves/s, {el:.3f} s per sweep", flush=True)
        for s in sims:
            s.close()


def main(argv):
    case = argv[1] if len(argv) > 1 else "batch"
    with tempfile.TemporaryDirectory() as d:
        {"batch": batch_case, "hmc": hmc_case, "egas": egas_case, "egas_phases": egas_phases_case, "hmc_egas": hmc_egas_case, "large32": large32_case, "bosons": bosons_case, "chains": chains_case,
         "egas_chains": egas_chains_case, "egas_chains32": lambda dd: egas_chains_case(dd, 32)}[case](d)


if __name__ == "__main__":
    main(sys.argv)
