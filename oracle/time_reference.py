"""Speed of the FP64 restatement (oracle/oracle.cc) against the reference's own classes on the same
bisection attempts — test infrastructure, run where the reference checkout exists.

The bench's CPU legs time the restatement, because the reference's headers build only against
oracle/refshim/ with the checkout present. This script says how that stand-in compares with the
reference itself: on chains of the 256-chain trapped Coulomb workload (bisection level 3, the
chain seeds of rank 0), it runs one bisection sweep of each chain (N ceil(M/8) attempts) through
the reference's Move::DoEvent (oracle/ref.py, built -O3 -ffast-math by oracle/build_ref.sh) and
through the restatement, from the same path with the same draws, on one host thread each, and
prints both rates and their ratio. The two final paths must agree (same Markov chain).

The reference's draws are decoded before its timed loop; the ctypes cost of its per-attempt calls
is measured with a call of the same marshalling and subtracted.

`--egas` times the single-chain 66-electron gas instead (N = 66, r_s = 2, beta = 8, M = 128, Ewald
|k| < 12 (2 pi / L), level 4; the bench's plain_electron_gas workload): 200 attempts of each spin's
Bisect, alternating, through both codes.

With SIMPIMC_REF_OPENMP=1 the reference runs from its OpenMP build (oracle/build_ref.sh with
REF_OPENMP=1: its action loops over OMP_NUM_THREADS threads, the reference's own model for one
chain); its reductions then run in thread order, so its path may part from the restatement's in
the last bits, which is reported rather than refused.

Usage: python oracle/time_reference.py [chain ...]   (default: chains 0, 32, ..., 224)
       [SIMPIMC_REF_OPENMP=1 OMP_NUM_THREADS=n] python oracle/time_reference.py --egas
"""
from __future__ import annotations

import math
import os
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

N_CHAINS, SEED0, LEVEL = 256, 1000, 3


def time_chain(items, tmp, c):
    import oracle
    from oracle import ref
    xml, path = items[c]
    n, m = path.shape[0], path.shape[1]
    reps = n * math.ceil(m / (1 << LEVEL))
    o = oracle.OracleSim(xml, base_dir=tmp, chain=c)
    o.set_path(path)
    r = ref.RefSim(xml, base_dir=tmp, chain=c)
    r.set_path(path)
    draws = []
    for a in range(reps):
        pb, z, lu = oracle.bisect_draws(r._seed, c, 0, a, n, m, LEVEL)
        draws.append((int(pb[0]), int(pb[1]), np.ascontiguousarray(z, dtype=np.float64), np.exp(np.asarray(lu, dtype=np.float64))))
    L, h = r._L, r._h
    t0 = time.perf_counter()
    for pa, b0, zz, uu in draws:
        if L.refsim_move_attempt(h, 0, pa, b0, zz.ctypes.data_as(ref._DP), len(zz), uu.ctypes.data_as(ref._DP), len(uu)) != 0:
            raise RuntimeError(L.refsim_last_error().decode())
    t_ref = time.perf_counter() - t0
    cnt = np.zeros(3, dtype=np.uint64)
    t0 = time.perf_counter()
    for _ in draws:
        L.refsim_move_counters(h, 0, cnt.ctypes.data_as(ref._U64P))
    t_call = time.perf_counter() - t0
    t0 = time.perf_counter()
    o.move_attempts(0, reps)
    t_port = time.perf_counter() - t0
    same = bool(np.allclose(o.get_path(1), r.get_path(1), rtol=0, atol=1e-9))
    o.close()
    r.close()
    moves = reps * ((1 << LEVEL) - 1)
    return n, m, moves / (t_ref - t_call), moves / t_port, same


def time_egas(n_each=200):
    """The 66-electron gas: n_each attempts of each spin's move, alternating, through the reference
    and the restatement from the same start; returns (bead-moves/s of each, same path)."""
    import oracle
    from oracle import ref
    from simpimc_gb300.configs import electron_gas
    tmp = tempfile.mkdtemp(prefix="pimc_timeref_")
    level = 4
    xml, path = electron_gas(tmp, n_part=66, rs=2.0, beta=8.0, n_bead=128, k_cut_units=12.0, n_level=level, seed=20261203)
    r = ref.RefSim(xml, base_dir=tmp)
    r.set_path(path)
    o = oracle.OracleSim(xml, base_dir=tmp)
    o.set_path(path)
    draws = []
    for a in range(n_each):
        for m in (0, 1):
            pb, z, lu = oracle.bisect_draws(r._seed, 0, m, a, 33, 128, level)
            draws.append((m, int(pb[0]), int(pb[1]), np.ascontiguousarray(z, dtype=np.float64), np.exp(np.asarray(lu, dtype=np.float64))))
    L, h = r._L, r._h
    t0 = time.perf_counter()
    for m, pa, b0, zz, uu in draws:
        if L.refsim_move_attempt(h, m, pa, b0, zz.ctypes.data_as(ref._DP), len(zz), uu.ctypes.data_as(ref._DP), len(uu)) != 0:
            raise RuntimeError(L.refsim_last_error().decode())
    t_ref = time.perf_counter() - t0
    t0 = time.perf_counter()
    for _ in range(n_each):
        o.move_attempts(0, 1)
        o.move_attempts(1, 1)
    t_port = time.perf_counter() - t0
    same = bool(np.allclose(o.get_path(1), r.get_path(1), rtol=0, atol=1e-9))
    moves = 2 * n_each * ((1 << level) - 1)
    return moves / t_ref, moves / t_port, same


def main():
    if sys.argv[1:] == ["--egas"]:
        from oracle import ref
        v_ref, v_port, same = time_egas()
        if not same and not ref.OPENMP:
            raise RuntimeError("the reference and the restatement left different paths")
        threads = os.environ.get("OMP_NUM_THREADS", str(os.cpu_count())) if ref.OPENMP else "1"
        print(f"66-electron gas: reference ({threads} thread{'' if threads == '1' else 's'}) {v_ref / 1e3:.2f} k bead-moves/s, "
              f"restatement (1 thread) "
              f"{v_port / 1e3:.2f} k, restatement / reference {v_port / v_ref:.2f}, same path {same}")
        return
    from simpimc_gb300.configs import batched_trap_chains
    chains = [int(a) for a in sys.argv[1:]] or list(range(0, N_CHAINS, N_CHAINS // 8))
    tmp = tempfile.mkdtemp(prefix="pimc_timeref_")
    items = batched_trap_chains(tmp, n_chains=N_CHAINS, seed0=SEED0, n_level=LEVEL, chain_seed0=SEED0, hmc=None)
    ratios = []
    for c in chains:
        n, m, v_ref, v_port, same = time_chain(items, tmp, c)
        if not same:
            raise RuntimeError(f"chain {c}: the reference and the restatement left different paths")
        ratios.append(v_port / v_ref)
        print(f"chain {c:3d} N={n:3d} M={m:3d}: reference {v_ref / 1e3:7.1f} k bead-moves/s, restatement {v_port / 1e3:7.1f} k, "
              f"restatement / reference {v_port / v_ref:.2f}", flush=True)
    print(f"restatement / reference over {len(ratios)} chains: min {min(ratios):.2f}, median {float(np.median(ratios)):.2f}, "
          f"max {max(ratios):.2f}")


if __name__ == "__main__":
    main()
