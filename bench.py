#!/usr/bin/env python3
"""Benchmark: bead-moves/s of the bisection sweep on the 66-electron gas (one GB300).

Workload (one "step" = one sweep): N = 66 Boltzmannon electrons (33 up, 33 down) in a periodic
cube at r_s = 2 (L = 13.0289), beta = 8, M = 128 slices, Coulomb as primitive short-range part
plus an Ewald k-sum with |k| < 12 (2 pi / L) (3561 stored half-space k-vectors), bisection
level 4 (2^4 - 1 = 15 resampled beads per attempt), FP64. A sweep is N_s * M / 2^4 attempts of
each species' move, alternating up/down as the reference's Loop of Move events does:
528 attempts = 7920 bead-moves. Synthetic data: beads uniform in the box from a fixed seed,
then untimed warm-up sweeps.

Arms:
  (default)          the CUDA library: `value` = device-timed sweeps with the path resident in
                     HBM; `e2e` = the same sweeps through the C interface with the path uploaded
                     from and downloaded to host memory every step.
  --impl reference   the CPU restatement of the reference hot path (the reference itself does not
                     build here: its scaffold/einspline/Armadillo/HDF5 dependencies are absent),
                     one independent chain per host thread, on a bounded sample per step.
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

N_PART, RS, BETA, N_BEAD, K_UNITS, N_LEVEL = 66, 2.0, 8.0, 128, 12.0, 4
METRIC = "bead-moves/s"
WORKLOAD = "electron gas N=66 (33+33) r_s=2 beta=8 M=128 Ewald |k|<12(2pi/L) bisection level 4, FP64, single chain"


def workload(tmp):
    from simpimc_gb300.configs import electron_gas
    xml, path = electron_gas(tmp, n_part=N_PART, rs=RS, beta=BETA, n_bead=N_BEAD, k_cut_units=K_UNITS, n_level=N_LEVEL,
                             seed=20261203)
    n_up = N_PART // 2
    reps = n_up * math.ceil(N_BEAD / (1 << N_LEVEL))  # per-species attempts per sweep
    return xml, path, reps


def base_config(extra=None):
    cfg = {"workload": WORKLOAD, "n_part": N_PART, "r_s": RS, "beta": BETA, "n_bead": N_BEAD, "k_cut": "12*2pi/L",
           "n_k_half_space": None, "bisection_level": N_LEVEL, "attempts_per_step": 2 * N_PART // 2 * math.ceil(N_BEAD / 16),
           "bead_moves_per_attempt": (1 << N_LEVEL) - 1, "parallelism": "replicas (independent chains per GPU)"}
    if extra:
        cfg.update(extra)
    return cfg


def clocks_sampler(out_path):
    cmd = ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
           "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
           "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits",
           "-lms", "200"]
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


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def algorithmic_bytes(sim, counters_before, counters_after, n_k):
    """Bytes one sweep touches once each (8-byte doubles): the moved particle's segment
    (read, and written twice on accept), the partners' positions on the segment, and the
    per-slice charge densities of the segment: read for the moved species and the other species
    of the cross action, written for the moved species on accept."""
    B = 1 << N_LEVEL
    D = 3
    total = 0
    for m in range(sim.n_moves):
        a0, _, _, acc0, l00 = counters_before[m]
        a1, _, _, acc1, l01 = counters_after[m]
        att, acc, lv0 = a1 - a0, acc1 - acc0, l01 - l00
        seg = (B + 1) * D * 8
        total += att * seg
        total += lv0 * ((N_PART - 1) * (B + 1) * D * 8 + B * n_k * 16 * 2)
        total += acc * ((B - 1) * n_k * 16 + 2 * (B - 1) * D * 8)
    return total


def reduce_max_over_ranks(values, dist=None, device=None):
    """Element-wise maximum of per-rank timings: the slowest replica sets the job time. Chains are
    independent replicas (no data exchange), so this is the only collective of the benchmark."""
    if dist is None or not dist.is_initialized():
        return [float(v) for v in values]
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


def run_ours(args):
    import torch
    from simpimc_gb300 import Simulation

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    tmp = tempfile.mkdtemp(prefix="pimc_bench_")
    xml, path, reps = workload(tmp)
    sim = Simulation(xml, base_dir=tmp, device=local, chain=rank)
    sim.set_path(path)
    stream = torch.cuda.ExternalStream(sim._lib.pimc_stream(sim._h), device=torch.device("cuda", local))
    moves, counts = [0, 1], [1, 1]
    B = 1 << N_LEVEL
    bead_moves_per_step = 2 * reps * (B - 1)

    for _ in range(args.warmup):
        sim.sweep(moves, counts, reps)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")  # 256 MB > L2
    counters0 = [sim.move_counters(m) for m in range(sim.n_moves)]
    clk_file = Path(tmp) / "clocks.csv"
    sampler = clocks_sampler(clk_file) if rank == 0 else None
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ms = 0.0
    t_wall = time.perf_counter()
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()  # L2 flush between timed steps (untimed)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        sim.sweep(moves, counts, reps)
        e1.record(stream)
        e1.synchronize()
        ms += e0.elapsed_time(e1)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall
    counters1 = [sim.move_counters(m) for m in range(sim.n_moves)]

    # e2e: host buffers in, sweep, host buffers out, every step, through the C interface.
    host_path = sim.get_path(1)
    e2e_ms = 0.0
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.set_path(host_path)
        sim.sweep(moves, counts, reps)
        host_path = sim.get_path(1)
        e2e_ms += (time.perf_counter() - t0) * 1e3
    if sampler:
        sampler.terminate()
        sampler.wait()

    ms_max, e2e_max = reduce_max_over_ranks([ms, e2e_ms], dist, device=f"cuda:{local}")
    total_moves = bead_moves_per_step * args.steps * world
    value = total_moves / (ms_max / 1e3)
    e2e_value = total_moves / (e2e_max / 1e3)
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    acc = sum(counters1[m][3] - counters0[m][3] for m in range(sim.n_moves))
    att = sum(counters1[m][0] - counters0[m][0] for m in range(sim.n_moves))
    lv0 = sum(counters1[m][4] - counters0[m][4] for m in range(sim.n_moves))
    peak, peak_kind = measured_peaks()
    alg = algorithmic_bytes(sim, counters0, counters1, sim.n_k) / args.steps
    achieved = alg / (ms_max / args.steps / 1e3) / 1e9
    traffic = None
    tf = ROOT / "profiles" / "sweep_traffic.json"
    if tf.exists():
        traffic = json.loads(tf.read_text()).get("dram_bytes_per_sweep")

    cpu = cpu_baseline(xml, tmp, host_path, reps) if not args.no_cpu_baseline else None
    path_bytes = N_PART * N_BEAD * 3 * 8
    line = {
        "metric": METRIC, "value": value, "unit": "bead-moves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded uniform beads, warmed up)",
        "config": base_config({"n_k_half_space": sim.n_k, "l2": "256 MB flush between timed steps",
                               "acceptance": acc / max(att, 1), "level0_fraction": lv0 / max(att, 1),
                               "sweep_grid_ctas": None}),
        "clocks": clocks_summary(clk_file, local),
        "e2e": {"value": e2e_value, "unit": "bead-moves/s", "h2d_bytes_per_step": path_bytes, "d2h_bytes_per_step": path_bytes,
                "note": "pimc_set_path (upload + charge-density rebuild) + pimc_sweep + pimc_get_path per step"},
        "gpu_launches": args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": "BisectSweepKernel", "algorithmic_bytes_per_launch": alg},
        "cpu_baseline": cpu,
        "wall_s": wall,
    }
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def _oracle_sample(xml, tmp, path, seconds, chain, reps, results, idx):
    import oracle
    o = oracle.OracleSim(xml, base_dir=tmp, chain=chain)
    o.set_path(path)
    B = 1 << N_LEVEL
    done = 0
    t0 = time.perf_counter()
    chunk = 8
    while time.perf_counter() - t0 < seconds:
        for _ in range(chunk):
            o.move_attempts(0, 1)
            o.move_attempts(1, 1)
        done += 2 * chunk
    el = time.perf_counter() - t0
    results[idx] = (done * (B - 1), el)
    o.close()


def cpu_baseline(xml, tmp, path, reps, seconds=12.0):
    """The oracle on one host core, from the GPU run's warmed-up path, for a bounded time."""
    res = [None]
    _oracle_sample(xml, tmp, path, seconds, 0, reps, res, 0)
    moves, el = res[0]
    return {"value": moves / el, "unit": "bead-moves/s", "cores": 1, "kind": "port",
            "sample": f"{moves // ((1 << N_LEVEL) - 1)} alternating up/down bisection attempts ({el:.1f} s) from the warmed-up GPU path"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    oracle.build()
    tmp = tempfile.mkdtemp(prefix="pimc_ref_")
    xml, path, reps = workload(tmp)
    threads = max(1, os.cpu_count() or 1)
    # Warm-up (untimed): equilibrate one chain briefly, then give every thread that path.
    o = oracle.OracleSim(xml, base_dir=tmp, chain=0)
    o.set_path(path)
    for _ in range(max(1, args.warmup)):
        for _ in range(16):
            o.move_attempts(0, 1)
            o.move_attempts(1, 1)
    start = o.get_path(1)
    o.close()
    per_step_s = 4.0
    total_moves, total_s = 0, 0.0
    for _ in range(args.steps):
        res = [None] * threads
        ths = [threading.Thread(target=_oracle_sample, args=(xml, tmp, start, per_step_s, i + 1, reps, res, i)) for i in range(threads)]
        t0 = time.perf_counter()
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        el = time.perf_counter() - t0
        total_moves += sum(r[0] for r in res)
        total_s += el
    value = total_moves / total_s
    line = {
        "metric": METRIC, "value": value, "unit": "bead-moves/s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")),
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_s / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded uniform beads)",
        "config": base_config({"l2": "n/a (host)"}), "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "bead-moves/s", "cores": threads, "kind": "port",
                         "sample": f"{threads} independent chains x {per_step_s:.0f} s per step (CPU restatement; the reference's own build needs absent dependencies)"},
        "e2e": {"value": value, "unit": "bead-moves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
