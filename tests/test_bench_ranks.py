"""Multi-process (replica) logic of bench.py on CPU: world size 2 over gloo on 127.0.0.1.

Chains are independent Markov chains, one set per GPU (the reference's MPI clones,
framework_class.h:44-53): the only collective is the maximum of the per-rank timings, and every
rank runs its own chains, with seeds no other rank uses."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    out[rank] = bench.reduce_max_over_ranks([1.0 + rank, 10.0 - rank, 3.0], dist)
    dist.barrier()
    dist.destroy_process_group()


def test_reduce_max_over_two_ranks():
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == out[1] == [2.0, 10.0, 3.0]


def _seed_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import re
    import tempfile

    import bench
    with tempfile.TemporaryDirectory() as d:
        items = bench.chains_workload(d, int(os.environ["RANK"]))
        seeds = [int(re.search(r'<RNG seed="(\d+)"', x).group(1)) for x, _ in items]
        shapes = [p.shape for _, p in items]
        first = items[0][1][0, 0].tolist()
    gathered = [None] * world
    dist.all_gather_object(gathered, seeds)
    out[rank] = (seeds, shapes, first, gathered)
    dist.destroy_process_group()


def test_ranks_run_disjoint_chains():
    """Rank r's replica: the same chain shapes on every rank, chain seeds SEED0 + r N_CHAINS + c."""
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_seed_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(300)
        assert p.exitcode == 0
    s0, sh0, f0, g0 = out[0]
    s1, sh1, f1, _ = out[1]
    assert len(s0) == len(s1) == 256
    assert not set(s0) & set(s1)
    assert g0[0] == s0 and g0[1] == s1
    assert sh0 == sh1
    assert f0 != f1  # different starting beads


def test_single_process_is_identity():
    import bench
    assert bench.reduce_max_over_ranks([1.5, 2.5]) == [1.5, 2.5]


def test_reference_arm_non_zero_rank_exits_quietly(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("RANK", "1")

    class A:
        steps, warmup = 1, 3

    bench.run_reference(A())
    assert capsys.readouterr().out == ""


def test_reference_arm_prints_the_contract_line():
    """`bench.py --impl reference` (host cores only) prints one JSON line with the contract's keys:
    the same metric and unit as the GPU arm, impl "reference", its cpu_baseline and an e2e block
    with zero copies."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3"], cwd=root, env=env,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    import bench
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.METRIC
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 3 and d["higher_is_better"] is True
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
