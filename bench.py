#!/usr/bin/env python3
"""Benchmark: bead-moves/s of path-integral Monte Carlo on one GB300, batched + adjoint.

Headline workload (one "step" = one measurement cycle, replayed as a CUDA graph: one bisection sweep
of every chain, one hybrid Monte Carlo attempt of every chain on the exact (adjoint) gradient, then
one thermal-energy measurement of every chain): 256 independent chains of distinguishable unit-mass
particles in an isotropic 3-D harmonic trap (omega = 1) with bare Coulomb repulsion (primitive
action), open boundaries, beta = 2; chain c has seed 1000 + c, N drawn uniformly from {16..128} and
M from {32, 64, 128} by a generator seeded with 1000. Bisection level 3 (7 resampled beads per
attempt; a sweep of a chain is N ceil(M / 8) attempts); HMC step 0.005 with 10 leapfrog steps
(every one of the chain's N M beads moves per attempt). FP32 positions, action terms and forces,
compensated sums, double-float acceptance, FP64 estimators. Synthetic data: beads i.i.d. N(0, 1)
from each chain's seed, then untimed warm-up cycles.

Also reported on the same line:
  components         the bisection sweep kernel and the HMC kernel timed alone (bead-moves/s each,
                     HMC acceptance), with a roofline for each;
  plain_same_system  the single-chain GPU path (double-float sweep kernel, FP64-grade HMC) running the
                     same cycle on a sample of the same chains, one chain at a time (what the
                     batched kernels replace);
  same_shape_chains  152 chains of the heaviest shape (N = 127, M = 128) swept as one batch and as
                     single-chain contexts through pimc_sweep_chains (one CTA per chain);
  energy_gate        per-chain energies and blocking error bars of the batched FP32 chains
                     against the single-chain path on the same chains and seeds, after an
                     equilibration of the paths, for the full cycle (statistical agreement: the
                     FP32 and FP64 leapfrogs part) and for the bisection cycle alone
                     (energy_gate_bisection: the same decisions, error bars equal within 1 %);
  plain_electron_gas the single-chain FP64 kernel on the 66-electron gas (r_s = 2, beta = 8,
                     M = 128, Ewald |k| < 12 (2 pi / L), 3561 half-space k-vectors, level 4);
  exchange_bosons    32 trapped bosons with PermBisectIterative on the permutation kernel, with
                     the oracle on one core beside it
  mixed_precision_large  the N = 1024, M = 512, |k| < 23 (2 pi / L) electron gas in the FP32 mode
                     and the double-float mode: speed, HBM fraction, energy and S(k) differences;
  hmc_adjoint        the r_s = 4, N = 128, M = 256 electron gas moved by the HMC path move on the
                     exact gradient: gradient time and whole-path bead-moves/s.

Arms:
  (default)          the CUDA library. `value` = device-timed cycles with the paths resident in
                     HBM; `e2e` = the same cycles through the C interface with every chain's path
                     uploaded from and downloaded to host memory and the energies read back.
  --impl reference   the FP64 CPU restatement of the reference hot path (the reference's own headers
                     build only against oracle/refshim where its checkout exists, which is not where
                     the bench runs; the restatement is pinned to that build) running the same cycle on the same
                     chains, one group of chains per host thread, on a bounded sample per step.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

from simpimc_gb300.stats import blocking_error  # noqa: E402

METRIC = "bead-moves/s"
N_CHAINS, SEED0, CHAIN_LEVEL = 256, 1000, 3
HMC = (0.005, 10)  # leapfrog step, steps per attempt
WORKLOAD = ("256 independent harmonic-trap Coulomb chains (omega=1, beta=2, open), N~U{16..128}, M in {32,64,128}, "
            "seeds 1000+c; one step = one bisection sweep (level 3) + one HMC attempt (step 0.005 x 10, exact gradient) "
            "of every chain + one energy measurement (CUDA graph); FP32 positions/terms/forces, compensated sums, "
            "double-float acceptance")
EGAS = dict(n_part=66, rs=2.0, beta=8.0, n_bead=128, k_cut_units=12.0, n_level=4)


def rank_chain_seed0(rank):
    """First chain seed of a rank's replica: rank r runs chains seeded SEED0 + r N_CHAINS + c, the same
    shapes as every other rank (drawn from SEED0) but independent Markov chains, as the reference's
    clones each draw their own seed (framework_class.h:84-101)."""
    return SEED0 + rank * N_CHAINS


def chains_workload(tmp, rank=0):
    from simpimc_gb300.configs import batched_trap_chains
    return batched_trap_chains(tmp, n_chains=N_CHAINS, seed0=SEED0, n_level=CHAIN_LEVEL, chain_seed0=rank_chain_seed0(rank), hmc=HMC)


def chain_cycle_moves(n, m):
    """Bead-moves of one chain's cycle: a bisection sweep (N ceil(M / 2^l) attempts of 2^l - 1
    beads) and one HMC attempt (all N M beads)."""
    B = 1 << CHAIN_LEVEL
    return n * math.ceil(m / B) * (B - 1) + n * m


def hmc_pair_flops(shapes):
    """Algorithmic FP32 flops of one HMC attempt of every chain: (steps + 1) gradient passes, each
    N (N - 1) M pair evaluations of 16 flops (3 differences, r^2 in 5, r^-3 in 2, three force FMAs in
    6, an FMA counted as two) plus N M beads of 24 flops (kinetic links and trap)."""
    per = 0
    for n, m, _ in shapes:
        per += n * (n - 1) * m * 16 + n * m * 24
    return (HMC[1] + 1) * per


def fp32_peak_tflops(device, sm_mhz):
    """Nominal FP32 CUDA-core peak: SMs x 128 FP32 lanes x 2 flops (FMA) x SM clock."""
    import torch
    n_sm = torch.cuda.get_device_properties(device).multi_processor_count
    return n_sm * 128 * 2 * sm_mhz * 1e6 / 1e12


def clocks_sampler(out_path):
    cmd = ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
           "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
           "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits",
           "-lms", "50"]
    try:
        return subprocess.Popen(cmd, stdout=open(out_path, "w"), stderr=subprocess.DEVNULL)
    except Exception:
        return None


def clocks_summary(path, device):
    sm, mx, reasons = [], [], set()
    try:
        for line in Path(path).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9 or f[0] != str(device):
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
    except FileNotFoundError:
        pass
    if not sm:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
    return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def measured_hbm_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def reduce_max_over_ranks(values, dist=None, device=None):
    """Element-wise maximum of per-rank timings: the slowest replica sets the job time. Chains are
    independent replicas (no data exchange), so this is the only collective of the benchmark."""
    if dist is None or not dist.is_initialized():
        return [float(v) for v in values]
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


def batch_algorithmic_bytes(batch, att, acc):
    """Bytes one sweep launch touches once each (float4 = 16 B per bead): the moved particle's
    2^l + 1 beads and every other particle's beads on the 2^l - 1 inner slices (loaded for every
    attempt), plus the 2^l - 1 beads written back on acceptance."""
    total = 0
    for c, (n, m, lvl) in enumerate(batch.shapes):
        B = 1 << lvl
        total += int(att[c]) * ((B + 1) + (n - 1) * (B - 1)) * 16 + int(acc[c]) * (B - 1) * 16
    return total


def time_plain_chains(items, tmp, local, sample, cycles=2):
    """The single-chain GPU path (double-float sweep kernel, FP64-grade HMC) running the batch's cycle on
    `sample` chains, one after the other: device time and bead-moves."""
    import torch
    from simpimc_gb300 import Simulation
    moves, secs = 0, 0.0
    for c in sample:
        xml, path = items[c]
        s = Simulation(xml, base_dir=tmp, device=local, chain=c)
        s.set_path(path)
        n, m = s.species_info(0)[0], s.n_bead
        reps = n * math.ceil(m / (1 << CHAIN_LEVEL))
        st = torch.cuda.ExternalStream(s._lib.pimc_stream(s._h), device=torch.device("cuda", local))
        s.sweep([0, 1], [reps, 1], 1)  # warm-up cycle
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        s.sweep([0, 1], [reps, 1], cycles)
        e1.record(st)
        e1.synchronize()
        secs += e0.elapsed_time(e1) / 1e3
        moves += cycles * chain_cycle_moves(n, m)
        s.close()
    return moves, secs


def energy_gate(items, tmp, local, chains, equil, cycles, hmc=True):
    """Batched FP32 chains against the single-chain path (double-float bisection, FP64-grade HMC) on the same
    chains and seeds: `equil` untimed cycles to equilibrate the paths, then per chain the mean energy
    and its blocking error bar over `cycles` measurements (one per cycle). With hmc=False the cycle is
    the bisection sweep alone: both paths then make the same accept decisions, so the two series
    match measurement by measurement and the error bars agree far inside 1 %. With the HMC attempt the
    FP32 and FP64 leapfrog trajectories part (the dynamics are chaotic), the chains become independent
    samples, and the comparison is statistical: means within their combined error bars, error bars
    within the resolution of blocking estimates from >= 16 blocks (about 1 / sqrt(15) relative)."""
    from simpimc_gb300 import ChainBatch, Simulation
    sub = [items[c] for c in chains]
    b = ChainBatch([x for x, _ in sub], base_dir=tmp, device=local)
    # The batch numbers its chains 0..k-1; the single-chain contexts use the same chain indices.
    for i, (_, p) in enumerate(sub):
        b.set_path(i, p)
    b.set_hmc_per_cycle(1 if hmc else 0)
    b.run(equil, 1)
    b.reset_energy()
    b.run(cycles, 1)
    rows = []
    for i, (xml, p) in enumerate(sub):
        e32, n = b.energy(i, cap=cycles)
        s = Simulation(xml, base_dir=tmp, device=local, chain=i)
        s.set_path(p)
        reps = s.species_info(0)[0] * math.ceil(s.n_bead / (1 << CHAIN_LEVEL))
        mv, ct = ([0, 1], [reps, 1]) if hmc else ([0], [reps])
        s.sweep(mv, ct, equil)
        e64 = []
        for _ in range(cycles):
            s.sweep(mv, ct, 1)
            s.observable_accumulate(0)
            e64.append(s.observable_block(0)[0])
        hacc = s.move_counters(1)[3]
        s.close()
        a32, a64 = e32[:, 0], np.asarray(e64)
        err32, err64 = blocking_error(a32), blocking_error(a64)
        both = math.hypot(err32, err64)
        rows.append({"chain": chains[i], "shape": list(b.shapes[i][:2]), "E_fp32": float(a32.mean()), "err_fp32": err32,
                     "E_fp64": float(a64.mean()), "err_fp64": err64,
                     "err_ratio": err32 / err64 if err64 > 0 else None,
                     "z_means": float((a32.mean() - a64.mean()) / both) if both > 0 else 0.0,
                     "max_abs_diff_per_measurement": float(np.max(np.abs(a32 - a64))),
                     "hmc_acceptance": hacc / max(equil + cycles, 1) if hmc else None})
    b.close()
    ratios = [r["err_ratio"] for r in rows if r["err_ratio"]]
    dev = max(abs(r - 1.0) for r in ratios) if ratios else None
    resolution = 1.0 / math.sqrt(15.0)
    ok = (dev is not None and dev < 0.01) if not hmc else (dev is not None and dev < 2 * resolution and
                                                            all(abs(r["z_means"]) < 2.0 for r in rows))
    return {"cycle": "bisection sweep + HMC attempt" if hmc else "bisection sweep", "equilibration_cycles": equil, "cycles": cycles,
            "chains": rows, "max_err_ratio_deviation": dev, "err_ratio_resolution": resolution if hmc else None, "pass": bool(ok),
            "note": "chain i of the batch and the single-chain context with chain=i draw the same random streams; "
                    "the paths are equilibrated before the measured cycles"}


def egas_plain(local, steps, warmup, tmp, flush):
    """The single-chain FP64 sweep kernel on the 66-electron gas: device time, e2e, bytes."""
    import torch
    from simpimc_gb300 import Simulation
    from simpimc_gb300.configs import electron_gas
    xml, path = electron_gas(tmp, seed=20261203, **EGAS)
    sim = Simulation(xml, base_dir=tmp, device=local, chain=0)
    sim.set_path(path)
    st = torch.cuda.ExternalStream(sim._lib.pimc_stream(sim._h), device=torch.device("cuda", local))
    B = 1 << EGAS["n_level"]
    reps = EGAS["n_part"] // 2 * math.ceil(EGAS["n_bead"] / B)
    for _ in range(warmup):
        sim.sweep([0, 1], [1, 1], reps)
    c0 = [sim.move_counters(m) for m in range(sim.n_moves)]
    ms = 0.0
    for _ in range(steps):
        with torch.cuda.stream(st):
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        sim.sweep([0, 1], [1, 1], reps)
        e1.record(st)
        e1.synchronize()
        ms += e0.elapsed_time(e1)
    c1 = [sim.move_counters(m) for m in range(sim.n_moves)]
    host = sim.get_path(1)
    e2e_ms = 0.0
    for _ in range(steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.set_path(host)
        sim.sweep([0, 1], [1, 1], reps)
        host = sim.get_path(1)
        e2e_ms += (time.perf_counter() - t0) * 1e3
    moves = 2 * reps * (B - 1) * steps
    n_k = sim.n_k
    att = sum(c1[m][0] - c0[m][0] for m in range(2))
    acc = sum(c1[m][3] - c0[m][3] for m in range(2))
    lv0 = sum(c1[m][4] - c0[m][4] for m in range(2))
    n = EGAS["n_part"]
    alg = (att * (B + 1) * 24 + lv0 * ((n - 1) * (B + 1) * 24 + B * n_k * 32) + acc * ((B - 1) * n_k * 16 + 2 * (B - 1) * 24)) / steps
    peak, kind = measured_hbm_peak()
    achieved = alg / (ms / steps / 1e3) / 1e9
    out = {"workload": "electron gas N=66 (33+33) r_s=2 beta=8 M=128 Ewald |k|<12(2pi/L) bisection level 4, FP64-grade, single chain",
           "value": moves / (ms / 1e3), "unit": METRIC, "ms_per_sweep": ms / steps, "n_k_half_space": n_k,
           "acceptance": acc / max(att, 1),
           "e2e": {"value": moves / (e2e_ms / 1e3), "unit": METRIC, "h2d_bytes_per_step": n * EGAS["n_bead"] * 24,
                   "d2h_bytes_per_step": n * EGAS["n_bead"] * 24},
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                        "peak_kind": kind, "kernel": "BisectSweepKernel", "algorithmic_bytes_per_launch": alg}}
    return out, xml, host, reps


def large_mixed_precision(local, tmp, sweeps=3):
    """The large electron gas (r_s = 1, N = 1024 as 512 + 512, beta = 4, M = 512, |k| < 23 (2 pi / L),
    bisection level 4) in FP32 mode and in the double-float mode from the same start and seeds:
    device-timed sweeps of each, the FP32 kernel's bytes against the HBM peak, and the energy and
    S(k) (first 200 |k| shells) differences between the two runs."""
    import torch
    from simpimc_gb300 import Simulation
    from simpimc_gb300.configs import electron_gas
    xml, path = electron_gas(tmp, n_part=1024, rs=1.0, beta=4.0, n_bead=512, k_cut_units=23.0, n_level=4, seed=777,
                             structure_factor=True)
    B = 16
    reps = 512 * math.ceil(512 / B)
    runs = {}
    for bits in (32, 64):
        s = Simulation(xml, base_dir=tmp, device=local, chain=0)
        s.set_precision(bits)
        s.set_path(path)
        st = torch.cuda.ExternalStream(s._lib.pimc_stream(s._h), device=torch.device("cuda", local))
        s.sweep([0, 1], [1, 1], reps)  # warm-up sweep
        c0 = [s.move_counters(m) for m in range(2)]
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        energies = []
        ms = 0.0
        for _ in range(sweeps):
            e0.record(st)
            s.sweep([0, 1], [1, 1], reps)
            e1.record(st)
            e1.synchronize()
            ms += e0.elapsed_time(e1)
            s.observable_accumulate(0)
            energies.append(s.observable_block(0)[0])
            s.observable_accumulate(2)
        c1 = [s.move_counters(m) for m in range(2)]
        sk = s.observable_block(2)
        kv = s.kvecs()
        runs[bits] = dict(ms=ms, energies=np.asarray(energies), sk=np.asarray(sk), kmag=np.linalg.norm(kv, axis=1), n_k=s.n_k,
                          att=sum(c1[m][0] - c0[m][0] for m in range(2)), acc=sum(c1[m][3] - c0[m][3] for m in range(2)),
                          lv0=sum(c1[m][4] - c0[m][4] for m in range(2)))
        s.close()
    r32, r64 = runs[32], runs[64]
    moves = 2 * reps * (B - 1) * sweeps
    n_k = r32["n_k"]
    alg = (r32["att"] * (B + 1) * 24 + r32["lv0"] * (1023 * (B + 1) * 24 + B * n_k * 16) + r32["acc"] * (B - 1) * n_k * 8) / sweeps
    peak, kind = measured_hbm_peak()
    achieved = alg / (r32["ms"] / sweeps / 1e3) / 1e9
    mags = np.round(r32["kmag"], 9)
    shells = np.unique(mags)[:200]
    sk_diff = max(float(np.max(np.abs(r32["sk"][mags == m] - r64["sk"][mags == m]))) for m in shells) if r32["sk"].size else None
    de = r32["energies"] - r64["energies"]
    return {"workload": "electron gas N=1024 (512+512) r_s=1 beta=4 M=512 Ewald |k|<23(2pi/L) bisection level 4",
            "n_k_half_space": n_k, "sweeps": sweeps,
            "fp32": {"value": moves / (r32["ms"] / 1e3), "unit": METRIC, "ms_per_sweep": r32["ms"] / sweeps,
                     "acceptance": r32["acc"] / max(r32["att"], 1),
                     "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                                  "peak_kind": kind, "algorithmic_bytes_per_sweep": alg}},
            "fp64_grade": {"value": moves / (r64["ms"] / 1e3), "unit": METRIC, "ms_per_sweep": r64["ms"] / sweeps,
                           "acceptance": r64["acc"] / max(r64["att"], 1)},
            "energy_fp32": r32["energies"].tolist(), "energy_fp64": r64["energies"].tolist(),
            "energy_max_rel_diff": float(np.max(np.abs(de) / np.abs(r64["energies"]))),
            "sk_shells": int(len(shells)), "sk_max_abs_diff_200_shells": sk_diff,
            "note": "same start, seeds and draws; FP32 densities rebuilt from the positions at every sweep call"}


def hmc_adjoint(local, tmp, attempts=4, equil_sweeps=10):
    """The adjoint workload's system (r_s = 4, N = 128 as 64 + 64, beta = 16, M = 256, |k| < 17 (2 pi / L))
    moved by the HMC path move (leapfrog step 0.01, 10 steps, every bead of both species per
    attempt) on the exact gradient: device time per gradient evaluation and per attempt."""
    import torch
    from simpimc_gb300 import Simulation
    from simpimc_gb300.configs import electron_gas
    xml, path = electron_gas(tmp, n_part=128, rs=4.0, beta=16.0, n_bead=256, k_cut_units=17.0, n_level=4, seed=4242)
    xml = xml.replace('<Move name="BisectD" type="Bisect" species="eD" n_level="4" />',
                      '<Move name="BisectD" type="Bisect" species="eD" n_level="4" />\n'
                      '    <Move name="HMC" type="HMC" step_size="0.01" n_steps="10" />')
    s = Simulation(xml, base_dir=tmp, device=local, chain=0)
    # The electron gas's classical start (every bead of a particle at one uniform point), then
    # bisection sweeps until the paths have spread; HMC from there.
    s.set_path(path)
    for _ in range(equil_sweeps):
        s.sweep([0, 1], [1, 1], 64 * 16)
    st = torch.cuda.ExternalStream(s._lib.pimc_stream(s._h), device=torch.device("cuda", local))
    s.action_gradient_path()  # warm-up
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    for _ in range(3):
        s.action_gradient_path()
    grad_s = (time.perf_counter() - t0) / 3
    s.move_attempts(2, 1)  # warm-up attempt
    torch.cuda.synchronize()
    c0 = s.move_counters(2)
    e0.record(st)
    s.move_attempts(2, attempts)
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    c1 = s.move_counters(2)
    beads = 128 * 256
    out = {"workload": "electron gas N=128 (64+64) r_s=4 beta=16 M=256 Ewald |k|<17(2pi/L), HMC step 0.01 x 10 on the exact gradient",
           "n_k_half_space": s.n_k, "attempts": attempts, "ms_per_attempt": ms / attempts,
           "gradient_s_host_timed": grad_s, "acceptance": (c1[3] - c0[3]) / max(c1[0] - c0[0], 1),
           "value": beads * attempts / (ms / 1e3), "unit": METRIC,
           "equilibration": f"{equil_sweeps} bisection sweeps (level 4) from the classical start",
           "note": "one HMC attempt moves all 32768 beads; 11 gradient and 2 whole-ring action evaluations per attempt; densities, Ewald sums and pair forces in double-float, other terms and totals FP64"}
    s.close()
    return out


def exchange_bosons(local, tmp, sweeps=20, cpu_seconds=6.0):
    """Exchanging bosons on the permutation kernel: N = 32 in the harmonic trap (omega = 1, beta = 4,
    M = 32), plain bisection and PermBisectIterative at level 3, one sweep = N attempts of each.
    Bead-moves count 2^l - 1 per plain attempt and (cycle length) x (2^l - 1) per permuting attempt
    whose cycle was selected. The oracle runs the same chain on one host core beside it."""
    import torch
    import oracle
    from simpimc_gb300 import Simulation
    from simpimc_gb300.configs import trapped_bosons
    n, m_beads, lvl = 32, 32, 3
    B1 = (1 << lvl) - 1
    xml, path = trapped_bosons(tmp, n_part=n, beta=4.0, n_bead=m_beads, n_level=lvl, seed=77)
    path = path * 0.4
    s = Simulation(xml, base_dir=tmp, device=local, chain=0)
    s.set_path(path)
    s.sweep([0, 1], [n, n], 5)  # warm-up
    st = torch.cuda.ExternalStream(s._lib.pimc_stream(s._h), device=torch.device("cuda", local))

    def moved(sim, pstats):
        att, _ = pstats
        return sum(int(att[i]) * (i + 1) * B1 for i in range(n))

    b0 = s.move_counters(0)[0]
    p0 = moved(s, s.perm_stats(1, n))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    s.sweep([0, 1], [n, n], sweeps)
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    beads = (s.move_counters(0)[0] - b0) * B1 + moved(s, s.perm_stats(1, n)) - p0
    att, acc = s.perm_stats(1, n)
    cycles = {int(i + 1): [int(att[i]), int(acc[i])] for i in range(n) if att[i]}
    s.close()
    oracle.build()
    o = oracle.OracleSim(xml, base_dir=tmp)
    o.set_path(path)
    o.move_attempts(0, n)
    o.move_attempts(1, n)
    cb0, cp0 = o.move_stats(0)[0], moved(o, o.perm_stats(1, n))
    t0, done = time.perf_counter(), 0
    while time.perf_counter() - t0 < cpu_seconds:
        o.move_attempts(0, n)
        o.move_attempts(1, n)
        done += 1
    el = time.perf_counter() - t0
    cbeads = (o.move_stats(0)[0] - cb0) * B1 + moved(o, o.perm_stats(1, n)) - cp0
    o.close()
    return {"workload": f"trapped bosons N={n} omega=1 beta=4 M={m_beads}, Bisect + PermBisectIterative at level {lvl}",
            "sweeps": sweeps, "ms_per_sweep": ms / sweeps, "value": beads / (ms / 1e3), "unit": METRIC,
            "perm_attempts_accepts_by_cycle_length": cycles,
            "cpu_oracle_1_core": {"value": cbeads / el, "unit": METRIC, "sweeps": done, "seconds": el},
            "note": "one CTA per chain runs the attempts in order (PermBisectKernelDD, double-float); device time of "
                    "the sweep calls, host gaps between the per-move launches included"}


def exchange_bosons_chains(local, tmp, n_chains=608, sweeps=10):
    """The exchanging-boson chain of exchange_bosons, n_chains independent copies (seeds 77 + c),
    one context per chain, all swept by pimc_sweep_chains: one launch with one CTA per chain.
    Wall-clock time of the call, device synchronised on both sides."""
    import torch
    from simpimc_gb300 import Simulation
    from simpimc_gb300.configs import trapped_bosons
    n, m_beads, lvl = 32, 32, 3
    B1 = (1 << lvl) - 1
    sims = []
    for c in range(n_chains):
        d = os.path.join(tmp, f"bosons{c}")
        xml, path = trapped_bosons(d, n_part=n, beta=4.0, n_bead=m_beads, n_level=lvl, seed=77 + c)
        s = Simulation(xml, base_dir=d, device=local, chain=c)
        s.set_path(path * 0.4)
        sims.append(s)

    from simpimc_gb300 import sweep_chains

    def run_all(k):
        sweep_chains(sims, [0, 1], [n, n], k)

    run_all(2)  # warm-up
    before = [(s.move_counters(0)[0], s.perm_stats(1, n)[0]) for s in sims]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    run_all(sweeps)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    beads = 0
    for s, (b0, pa0) in zip(sims, before):
        pa1 = s.perm_stats(1, n)[0]
        beads += (s.move_counters(0)[0] - b0) * B1 + sum(int(pa1[i] - pa0[i]) * (i + 1) * B1 for i in range(n))
    for s in sims:
        s.close()
    return {"workload": f"{n_chains} independent chains of the exchange_bosons system (seeds 77 + c)", "sweeps_per_chain": sweeps,
            "seconds": el, "value": beads / el, "unit": METRIC,
            "note": "pimc_sweep_chains: one launch, one CTA per chain; wall-clock time including argument upload and counter reads"}


def same_shape_chains(local, tmp, n_chains=152, sweeps=2, shape=(127, 128)):
    """Bisection sweeps of n_chains trapped Coulomb chains of one shape (the headline's heaviest,
    N = 127, M = 128, level 3; seeds 5000 + c), as one ChainBatch and as n_chains single-chain
    contexts swept by pimc_sweep_chains (one launch, one CTA per chain, double-float): device time
    of `sweeps` sweeps on each side, after a warm-up sweep."""
    import torch
    from simpimc_gb300 import ChainBatch, Simulation, sweep_chains
    from simpimc_gb300.configs import trapped_coulomb
    n, m = shape
    d = Path(tmp) / "same_shape"
    items = [trapped_coulomb(d, n_part=n, n_bead=m, n_level=CHAIN_LEVEL, seed=5000 + c, write_table=(c == 0)) for c in range(n_chains)]
    reps = n * math.ceil(m / (1 << CHAIN_LEVEL))
    b = ChainBatch([x for x, _ in items], base_dir=d, device=local)
    for c, (_, p) in enumerate(items):
        b.set_path(c, p)
    b.autotune(1)
    b.sweeps(1)
    st = torch.cuda.ExternalStream(b.stream(), device=torch.device("cuda", local))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    b.sweeps(sweeps)
    e1.record(st)
    e1.synchronize()
    batch_s = e0.elapsed_time(e1) / 1e3
    b.close()
    sims = []
    for c, (x, p) in enumerate(items):
        s = Simulation(x, base_dir=d, device=local, chain=c)
        s.set_path(p)
        sims.append(s)
    sweep_chains(sims, [0], [reps], 1)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sweep_chains(sims, [0], [reps], sweeps)
    torch.cuda.synchronize()
    chains_s = time.perf_counter() - t0
    for s in sims:
        s.close()
    moves = n_chains * sweeps * reps * ((1 << CHAIN_LEVEL) - 1)
    return {"workload": f"{n_chains} trapped Coulomb chains N={n} M={m} level {CHAIN_LEVEL}, bisection sweeps", "sweeps": sweeps,
            "batch": {"value": moves / batch_s, "unit": METRIC, "seconds": batch_s, "note": "ChainBatch, FP32 positions, device time"},
            "sweep_chains": {"value": moves / chains_s, "unit": METRIC, "seconds": chains_s,
                             "note": "pimc_sweep_chains on single-chain contexts (double-float), one CTA per chain; wall-clock "
                                     "time of the call with the device synchronised on both sides"},
            "ratio": chains_s / batch_s}


def cpu_oracle_chains(items, tmp, seconds, chains):
    """The oracle on one host core, running the batch's cycle (bisection sweep + HMC attempt) on
    `chains` round robin."""
    import oracle
    oracle.build()
    sims = []
    for c in chains:
        xml, p = items[c]
        o = oracle.OracleSim(xml, base_dir=tmp, chain=c)
        o.set_path(p)
        n, m = p.shape[0], p.shape[1]
        sims.append((o, n * math.ceil(m / (1 << CHAIN_LEVEL)), chain_cycle_moves(n, m)))
    moves, cycles, t0 = 0, 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        for o, reps, mv in sims:
            o.move_attempts(0, reps)
            o.move_attempts(1, 1)
            moves += mv
            cycles += 1
            if time.perf_counter() - t0 >= seconds:
                break
    el = time.perf_counter() - t0
    for o, _, _ in sims:
        o.close()
    return moves, el, cycles


def time_launches(stream, flush, steps, fn):
    """Device milliseconds of `steps` calls of fn() on `stream`, with an L2 flush before each."""
    import torch
    ms = 0.0
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        ms += e0.elapsed_time(e1)
    return ms


def run_ours(args):
    import torch
    from simpimc_gb300 import ChainBatch

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    if args.gpus != world:
        raise SystemExit(f"--gpus {args.gpus} needs {args.gpus} ranks (launch with torchrun --nproc-per-node {args.gpus}); "
                         f"WORLD_SIZE is {world}")
    tmp = tempfile.mkdtemp(prefix="pimc_bench_")
    items = chains_workload(tmp, rank)
    flat0 = np.concatenate([p.ravel() for _, p in items])
    batch = ChainBatch([x for x, _ in items], base_dir=tmp, device=local)
    batch.set_paths(flat0)
    stream = torch.cuda.ExternalStream(batch.stream(), device=torch.device("cuda", local))
    per_sweep = batch.stats()["bead_moves_per_sweep"]
    per_hmc = sum(n * m for n, m, _ in batch.shapes)
    per_step = per_sweep + per_hmc
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")  # 256 MB > L2

    # Clock samples cover the autotuner, the warm-up and the timed loops below (the timed loops alone
    # are too short for the sampler's period); the GPU runs the same kernels throughout.
    clk_file = Path(tmp) / "clocks.csv"
    sampler = clocks_sampler(clk_file) if rank == 0 else None
    ipl, mw, wave, tune_s = batch.autotune(2)
    batch.set_hmc_per_cycle(1)
    batch.run(args.warmup, 1)
    batch.synchronize()
    att0, acc0 = batch.counters()
    hatt0, hacc0 = batch.hmc_counters()
    launches0 = batch.stats()["kernel_launches"]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t_wall = time.perf_counter()
    ms = time_launches(stream, flush, args.steps, lambda: batch.run(1, 1))
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall
    launches = batch.stats()["kernel_launches"] - launches0
    att1, acc1 = batch.counters()
    hatt1, hacc1 = batch.hmc_counters()

    # The two kernels alone (for their rooflines): one launch per step, same flush.
    rounds1 = batch.rounds()
    k_ms = time_launches(stream, flush, args.steps, lambda: batch.sweeps(1))
    att2, acc2 = batch.counters()
    rounds2 = batch.rounds()
    h_ms = time_launches(stream, flush, args.steps, lambda: batch.hmc_attempts(1))

    # e2e: every chain's path from pinned host memory, one cycle, energies and paths back, every step.
    host = torch.empty(batch.get_paths().size, dtype=torch.float64, pin_memory=True).numpy()
    batch.get_paths(out=host)
    e2e_ms = 0.0
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        batch.set_paths(host)
        batch.run(1, 1)
        energies = batch.last_energy()
        batch.get_paths(out=host)
        e2e_ms += (time.perf_counter() - t0) * 1e3
    if sampler:
        sampler.terminate()
        sampler.wait()
    assert np.all(np.isfinite(energies))

    ms_max, e2e_max, k_max, h_max = reduce_max_over_ranks([ms, e2e_ms, k_ms, h_ms], dist, device=f"cuda:{local}")
    value = per_step * args.steps * world / (ms_max / 1e3)
    e2e_value = per_step * args.steps * world / (e2e_max / 1e3)
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    clocks = clocks_summary(clk_file, local)
    peak, peak_kind = measured_hbm_peak()
    alg = batch_algorithmic_bytes(batch, att2 - att1, acc2 - acc1) / args.steps
    achieved = alg / (k_max / args.steps / 1e3) / 1e9
    traffic = None
    tf = ROOT / "profiles" / "batch_sweep_traffic.json"
    if tf.exists():
        traffic = json.loads(tf.read_text()).get("dram_bytes_per_sweep")
    sweep_roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                  "peak_kind": peak_kind, "kernel": "BatchSweepKernel", "algorithmic_bytes_per_launch": alg,
                  "ms_per_launch": k_max / args.steps,
                  "note": "secondary view: operands are re-read from shared memory and L2, so HBM does not bind this "
                          "kernel; its bound is the heaviest chain's serial rounds (critical_path)"}
    sm_mhz = clocks.get("sm_mhz") or 2070.0
    # The sweep launch's binding resource: the heaviest chain's serial scheduling rounds on its SM.
    d_rounds = (rounds2 - rounds1).astype(np.float64) / args.steps
    d_att = (att2 - att1).astype(np.float64) / args.steps
    crit = int(np.argmax(d_rounds))
    launch_cycles = k_max / args.steps * 1e-3 * sm_mhz * 1e6
    critical_path = {"bound": "sm-issue: the heaviest chain's scheduling rounds, one SM", "chain": crit,
                     "shape": list(batch.shapes[crit]), "attempts_per_sweep": float(d_att[crit]), "rounds_per_sweep": float(d_rounds[crit]),
                     "attempts_per_round": float(d_att[crit] / d_rounds[crit]) if d_rounds[crit] else None,
                     "cycles_per_round": launch_cycles / d_rounds[crit] if d_rounds[crit] else None,
                     "mean_attempts_per_round_all_chains": float(d_att.sum() / d_rounds.sum()) if d_rounds.sum() else None,
                     "note": "cycles_per_round = launch time x median SM clock / the heaviest chain's rounds: the launch ends "
                             "with that chain; ncu issue and occupancy figures in profiles/batch_sweep_256chains.md"}
    fp32_peak = fp32_peak_tflops(local, sm_mhz)
    flops = hmc_pair_flops(batch.shapes)
    h_achieved = flops / (h_max / args.steps / 1e3) / 1e12
    hmc_roof = {"bound": "fp32", "achieved": h_achieved, "peak": fp32_peak, "unit": "TFLOP/s", "frac": h_achieved / fp32_peak,
                "traffic": None, "peak_kind": "nominal: SMs x 128 FP32 lanes x 2 flops (FMA) x the median sampled SM clock "
                                             "(no measured FP32 peak in MEASURED_PEAKS.json)",
                "kernel": "BatchHmcKernel", "algorithmic_flops_per_launch": flops, "ms_per_launch": h_max / args.steps}
    dominant = hmc_roof if h_max >= k_max else sweep_roof
    sample = list(range(0, N_CHAINS, N_CHAINS // 8))
    pm, psec = time_plain_chains(items, tmp, local, sample)
    plain = {"value": pm / psec, "unit": METRIC, "chains": sample,
             "note": "single-chain path (double-float sweep kernel + FP64-grade HMC), the same cycle, one chain after another, device time"}
    mid = sorted(range(N_CHAINS), key=lambda c: batch.shapes[c][0] ** 2 * batch.shapes[c][1])
    gate_chains = [mid[len(mid) // 8], mid[len(mid) // 4], mid[3 * len(mid) // 8], mid[len(mid) // 2]]
    gate = energy_gate(items, tmp, local, chains=gate_chains, equil=args.gate_equil, cycles=args.gate_sweeps)
    gate_bisect = energy_gate(items, tmp, local, chains=gate_chains, equil=args.gate_equil, cycles=args.gate_sweeps, hmc=False)
    eg, _, _, _ = egas_plain(local, args.steps, args.warmup, tmp, flush)
    large = large_mixed_precision(local, tmp) if not args.no_large else None
    hmc = hmc_adjoint(local, tmp) if not args.no_large else None
    exch = exchange_bosons(local, tmp)
    exch["many_chains"] = exchange_bosons_chains(local, tmp)
    same_shape = same_shape_chains(local, tmp)
    cpu = None
    if not args.no_cpu_baseline:
        moves, el, cyc = cpu_oracle_chains(items, tmp, 12.0, sample)
        cpu = {"value": moves / el, "unit": METRIC, "cores": 1, "kind": "port",
               "sample": f"{cyc} chain cycles (bisection sweep + HMC attempt, {el:.1f} s) on chains {sample}, round robin"}
    path_bytes_h2d = int(host.nbytes)  # every chain's path as doubles, copied as they are
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Gaussian beads per chain, warmed up)",
        "config": {"workload": WORKLOAD, "n_chains": N_CHAINS, "bead_moves_per_step": per_step,
                   "bead_moves_per_step_bisection": per_sweep, "bead_moves_per_step_hmc": per_hmc,
                   "tile": {"items_per_lane": ipl, "max_warps": mw, "wave": wave, "autotune_s_per_sweep": tune_s},
                   "hmc_cluster": batch.hmc_cluster, "overlap_heavy_chains": batch.overlap, "split_chains": batch.split,
                   "bisection_acceptance": float((acc1 - acc0).sum() / max((att1 - att0).sum(), 1)),
                   "hmc_acceptance": float((hacc1 - hacc0).sum() / max((hatt1 - hatt0).sum(), 1)),
                   "l2": "256 MB flush between timed steps", "parallelism": "replicas (independent chains per GPU)"},
        "clocks": dict(clocks, window="autotune, warm-up and the timed loops, 50 ms period"),
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": path_bytes_h2d,
                "d2h_bytes_per_step": path_bytes_h2d + N_CHAINS * 4 * 8,
                "note": "pimc_batch_set_paths + pimc_batch_run(1 cycle) + pimc_batch_last_energy + pimc_batch_get_paths per step, "
                        "paths in pinned host memory"},
        "gpu_launches": launches,
        "roofline": dominant,
        "components": {
            "bisection_sweep": {"value": per_sweep / (k_max / args.steps / 1e3), "unit": METRIC, "ms_per_launch": k_max / args.steps,
                                "critical_path": critical_path, "roofline": sweep_roof},
            "hmc": {"value": per_hmc / (h_max / args.steps / 1e3), "unit": METRIC, "ms_per_launch": h_max / args.steps,
                    "leapfrog": {"step": HMC[0], "n_steps": HMC[1]}, "roofline": hmc_roof},
        },
        "cpu_baseline": cpu,
        "plain_same_system": plain,
        "same_shape_chains": same_shape,
        "speedup_vs_plain_same_system": value / plain["value"],
        "energy_gate": gate,
        "energy_gate_bisection": gate_bisect,
        "plain_electron_gas": eg,
        "mixed_precision_large": large,
        "hmc_adjoint": hmc,
        "exchange_bosons": exch,
        "wall_s": wall,
    }
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def _oracle_worker(items, tmp, chains, seconds, results, idx):
    """One host thread: the oracle running the batch's cycle (bisection sweep + HMC attempt) on its
    share of the chains, round robin, for `seconds`."""
    import oracle
    sims = []
    for c in chains:
        xml, p = items[c]
        o = oracle.OracleSim(xml, base_dir=tmp, chain=c)
        o.set_path(p)
        n, m = p.shape[0], p.shape[1]
        sims.append((o, n * math.ceil(m / (1 << CHAIN_LEVEL)), chain_cycle_moves(n, m)))
    moves, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        for o, reps, mv in sims:
            o.move_attempts(0, reps)
            o.move_attempts(1, 1)
            moves += mv
            if time.perf_counter() - t0 >= seconds:
                break
    results[idx] = (moves, time.perf_counter() - t0)
    for o, _, _ in sims:
        o.close()


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    oracle.build()
    tmp = tempfile.mkdtemp(prefix="pimc_ref_")
    items = chains_workload(tmp)
    threads = max(1, os.cpu_count() or 1)
    per_step_s = 4.0
    for _ in range(args.warmup):  # untimed: start-up of every thread's chains
        _oracle_worker(items, tmp, [0], 0.05, [None], 0)
    total_moves, total_s = 0, 0.0
    for _ in range(args.steps):
        res = [None] * threads
        groups = [list(range(i, N_CHAINS, threads)) for i in range(threads)]
        ths = [threading.Thread(target=_oracle_worker, args=(items, tmp, groups[i], per_step_s, res, i)) for i in range(threads)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        # each thread times its own cycles (after building its chains); the step lasts as long as the slowest
        total_s += max(r[1] for r in res)
        total_moves += sum(r[0] for r in res)
    value = total_moves / total_s
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_s / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Gaussian beads per chain)",
        "config": {"workload": WORKLOAD, "n_chains": N_CHAINS, "l2": "n/a (host)"}, "impl": "reference",
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                         "sample": f"{threads} threads, each running the cycle (bisection sweep + HMC attempt) on its share of "
                                   f"the 256 chains for {per_step_s:.0f} s per step (the FP64 CPU restatement: the reference's "
                                   "own headers build only against oracle/refshim with the reference checkout, which is not "
                                   "where the bench runs; tests/test_reference_pins.py pins the restatement to that build bit "
                                   "for bit, and oracle/time_reference.py measured the restatement 2.6-3.3x faster than the "
                                   "reference's Move::DoEvent on the same bisection attempts, one thread each)"},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--gate-sweeps", type=int, default=300, help="measured cycles of the energy gate")
    ap.add_argument("--gate-equil", type=int, default=100, help="equilibration cycles of the energy gate")
    ap.add_argument("--no-large", action="store_true", help="skip the N=1024 mixed-precision leg")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
