"""Reference harness wrapper — test infrastructure only (tests/ and the fixture generator in
tests/golden/).

`RefSim` drives simpimc's own classes, compiled from the reference checkout's unmodified headers
against oracle/refshim/ by oracle/build_ref.sh (oracle/refharness.cc is the C surface). Its methods
match `oracle.OracleSim`. Bisection draws come from the oracle's counter-based stream, so a
RefSim, an OracleSim and the GPU library replay the same Markov chain.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
# SIMPIMC_REF_OPENMP=1 selects the OpenMP build (timing only; the fixtures use the serial one)
OPENMP = os.environ.get("SIMPIMC_REF_OPENMP", "0") == "1"
LIB = HERE / "_ref" / ("libsimpimc_ref_omp.so" if OPENMP else "libsimpimc_ref.so")
SOURCES = [HERE / "refharness.cc", HERE / "build_ref.sh", *sorted((HERE / "refshim").rglob("*.h"))]
DEFAULT_REFERENCE = "/root/reference"

_DP = C.POINTER(C.c_double)
_U32P = C.POINTER(C.c_uint32)
_U64P = C.POINTER(C.c_uint64)
_lib = None


def reference_dir() -> str | None:
    d = os.environ.get("SIMPIMC_REFERENCE", DEFAULT_REFERENCE)
    return d if os.path.isdir(os.path.join(d, "src", "actions")) else None


def available() -> bool:
    return reference_dir() is not None


def build(force: bool = False) -> Path:
    ref = reference_dir()
    if ref is None:
        raise RuntimeError("the reference checkout is not present; the reference harness cannot be built here")
    if force or not LIB.exists() or any(s.stat().st_mtime > LIB.stat().st_mtime for s in SOURCES):
        env = dict(os.environ, REF_OPENMP="1" if OPENMP else "0")
        r = subprocess.run(["sh", str(HERE / "build_ref.sh"), ref], capture_output=True, text=True, env=env)
        if r.returncode != 0:
            raise RuntimeError(f"reference harness build failed:\n{r.stderr}")
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        L.refsim_last_error.restype = C.c_char_p
        L.refsim_destroy.restype = None
        L.refsim_destroy.argtypes = [C.c_void_p]
        sigs = {
            "refsim_create": [C.c_char_p, C.c_char_p, C.POINTER(C.c_void_p)],
            "refsim_info": [C.c_void_p, _U32P],
            "refsim_set_path": [C.c_void_p, C.c_int, _DP],
            "refsim_get_path": [C.c_void_p, C.c_int, _DP],
            "refsim_get_rho_k": [C.c_void_p, C.c_uint32, C.c_int, _DP],
            "refsim_kvecs": [C.c_void_p, _DP],
            "refsim_reset_rho_k_latch": [C.c_void_p],
            "refsim_get_action": [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, _U32P, _U32P, C.c_uint32, C.c_uint32, C.c_int, _DP],
            "refsim_get_action_gradient": [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, _U32P, _U32P, C.c_uint32, C.c_uint32, C.c_int,
                                           _DP],
            "refsim_dactiondbeta": [C.c_void_p, C.c_uint32, _DP],
            "refsim_potential": [C.c_void_p, C.c_uint32, _DP],
            "refsim_virial_energy": [C.c_void_p, C.c_uint32, C.c_double, _DP],
            "refsim_move_attempt": [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, _DP, C.c_uint32, _DP, C.c_uint32],
            "refsim_move_counters": [C.c_void_p, C.c_uint32, _U64P],
            "refsim_perm_attempt": [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, _DP, C.c_uint32, _DP, C.c_uint32, _DP, C.c_uint32],
            "refsim_perm_counters": [C.c_void_p, C.c_uint32, _U64P],
            "refsim_get_perm": [C.c_void_p, C.c_uint32, _U32P],
            "refsim_move_write": [C.c_void_p, C.c_uint32, C.POINTER(C.c_int64)],
            "refsim_obs_accumulate": [C.c_void_p, C.c_uint32],
            "refsim_obs_write": [C.c_void_p, C.c_uint32, _DP, C.c_uint64, _U64P],
        }
        for name, args in sigs.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = C.c_int
        _lib = L
    return _lib


def _seed_of(xml: str) -> int:
    import re
    m = re.search(r'<RNG\s+seed="(\d+)"', xml)
    return int(m.group(1)) if m else 0


MOVE_TYPES = ("Bisect", "PermBisectIterative", "PermBisectTable")
OBSERVABLE_TYPES = ("Energy", "PairCorrelation", "StructureFactor", "Sign", "PathDump")


def _moves(xml: str):
    """(type, species name, n_level) of each move the harness builds, in input order."""
    import re
    out = []
    for m in re.finditer(r"<Move\s[^>]*>", xml):
        tag = m.group(0)
        t = re.search(r'type="([^"]+)"', tag)
        if t is None or t.group(1) not in MOVE_TYPES:  # the Algorithm's event tags carry no type
            continue
        t = t.group(1)
        sp = re.search(r'species="([^"]+)"', tag).group(1)
        lvl = int(re.search(r'n_level="(\d+)"', tag).group(1))
        out.append((t, sp, lvl))
    return out


class RefSim:
    """The reference's classes on one path; same surface as oracle.OracleSim."""

    def __init__(self, xml: str, base_dir=".", chain: int = 0):
        L = lib()
        h = C.c_void_p()
        if L.refsim_create(xml.encode(), str(base_dir).encode(), C.byref(h)) != 0:
            raise RuntimeError(L.refsim_last_error().decode())
        self._L, self._h = L, h
        info = np.zeros(4, dtype=np.uint32)
        self._ok(L.refsim_info(h, info.ctypes.data_as(_U32P)))
        self.n_species, self.n_total, self.n_bead, self.n_k = (int(x) for x in info)
        self.n_d = 3
        self._seed, self._chain = _seed_of(xml), chain
        import re
        names = re.findall(r'<Species\s[^>]*name="([^"]+)"[^>]*n_part="(\d+)"', xml)
        self._species = {n: (i, int(c)) for i, (n, c) in enumerate(names)}
        self._moves = _moves(xml)
        self._attempts = [0] * len(self._moves)

    def _ok(self, rc):
        if rc != 0:
            raise RuntimeError(self._L.refsim_last_error().decode())

    def close(self):
        if self._h:
            self._L.refsim_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_path(self, pos, which: int = 2):
        a = np.ascontiguousarray(pos, dtype=np.float64)
        self._ok(self._L.refsim_set_path(self._h, which, a.ctypes.data_as(_DP)))

    def get_path(self, which: int = 1):
        out = np.zeros((self.n_total, self.n_bead, self.n_d))
        self._ok(self._L.refsim_get_path(self._h, which, out.ctypes.data_as(_DP)))
        return out

    def rho_k(self, species: int, which: int = 1):
        out = np.zeros((self.n_bead, self.n_k, 2))
        self._ok(self._L.refsim_get_rho_k(self._h, species, which, out.ctypes.data_as(_DP)))
        return out[..., 0] + 1j * out[..., 1]

    def kvecs(self):
        out = np.zeros((self.n_k, self.n_d))
        if self.n_k:
            self._ok(self._L.refsim_kvecs(self._h, out.ctypes.data_as(_DP)))
        return out

    def reset_rho_k_latch(self):
        self._ok(self._L.refsim_reset_rho_k_latch(self._h))

    @staticmethod
    def _parts(particles):
        sp = np.array([p[0] for p in particles], dtype=np.uint32)
        pi = np.array([p[1] for p in particles], dtype=np.uint32)
        return sp, pi

    def get_action(self, action, b0, b1, particles, level=0, mode=1):
        sp, pi = self._parts(particles)
        out = C.c_double()
        self._ok(self._L.refsim_get_action(self._h, action, b0, b1, sp.ctypes.data_as(_U32P), pi.ctypes.data_as(_U32P), len(sp), level,
                                           mode, C.byref(out)))
        return out.value

    def get_action_gradient(self, action, b0, b1, particles, level=0, mode=1):
        sp, pi = self._parts(particles)
        out = np.zeros(3)
        self._ok(self._L.refsim_get_action_gradient(self._h, action, b0, b1, sp.ctypes.data_as(_U32P), pi.ctypes.data_as(_U32P), len(sp),
                                                    level, mode, out.ctypes.data_as(_DP)))
        return out

    def dactiondbeta(self, action):
        out = C.c_double()
        self._ok(self._L.refsim_dactiondbeta(self._h, action, C.byref(out)))
        return out.value

    def potential(self, action):
        out = C.c_double()
        self._ok(self._L.refsim_potential(self._h, action, C.byref(out)))
        return out.value

    def virial_energy(self, action, window):
        out = C.c_double()
        self._ok(self._L.refsim_virial_energy(self._h, action, window, C.byref(out)))
        return out.value

    def move_attempts(self, move, n):
        """n Move::DoEvent calls of move `move` (Bisect or a permuting bisection) with the oracle's
        draws for its next attempts."""
        import oracle
        kind, sp_name, _ = self._moves[move]
        _, n_part = self._species[sp_name]
        for _ in range(n):
            n_level = self.move_level(move)
            a = self._attempts[move]
            if kind == "Bisect":
                pb, z, lu = oracle.bisect_draws(self._seed, self._chain, move, a, n_part, self.n_bead, n_level)
                zz = np.ascontiguousarray(z, dtype=np.float64)
                uu = np.exp(np.asarray(lu, dtype=np.float64))
                self._ok(self._L.refsim_move_attempt(self._h, move, int(pb[0]), int(pb[1]), zz.ctypes.data_as(_DP), len(zz),
                                                     uu.ctypes.data_as(_DP), len(uu)))
            else:
                idx, steps, sel_table, z, lu, fin = oracle.perm_draws(self._seed, self._chain, move, a, n_part, self.n_bead, n_level)
                sel = np.ascontiguousarray(steps.reshape(-1) if kind == "PermBisectIterative" else [sel_table], dtype=np.float64)
                zz = np.ascontiguousarray(z, dtype=np.float64)
                uu = np.ascontiguousarray(np.concatenate([np.exp(np.asarray(lu, dtype=np.float64)), [fin]]))
                self._ok(self._L.refsim_perm_attempt(self._h, move, int(idx[0]), int(idx[1]), zz.ctypes.data_as(_DP), len(zz),
                                                     sel.ctypes.data_as(_DP), len(sel), uu.ctypes.data_as(_DP), len(uu)))
            self._attempts[move] += 1

    def perm_stats(self, move, n_part):
        """Per cycle length: the permuting move's attempts and accepts in its current block."""
        out = np.zeros(2 * n_part, dtype=np.uint64)
        self._ok(self._L.refsim_perm_counters(self._h, move, out.ctypes.data_as(_U64P)))
        return out[:n_part].astype(np.int64), out[n_part:].astype(np.int64)

    def get_perm(self, species, n_part):
        """The path permutation at the ring closure (particle p's last bead links to slice 0 of out[p])."""
        out = np.zeros(n_part, dtype=np.uint32)
        self._ok(self._L.refsim_get_perm(self._h, species, out.ctypes.data_as(_U32P)))
        return out.astype(np.int64)

    def _counters(self, move):
        out = np.zeros(3, dtype=np.uint64)
        self._ok(self._L.refsim_move_counters(self._h, move, out.ctypes.data_as(_U64P)))
        return [int(x) for x in out]

    def move_level(self, move):
        return self._counters(move)[2]

    def move_write(self, move):
        """The move's Write event: block counters appended and reset, adaptive level updated.
        Returns the appended (n_attempt, n_accept, n_level or -1)."""
        out = np.zeros(3, dtype=np.int64)
        self._ok(self._L.refsim_move_write(self._h, move, out.ctypes.data_as(C.POINTER(C.c_int64))))
        return tuple(int(x) for x in out)

    def move_stats(self, move):
        """(total attempts, attempts in block, accepts in block), as OracleSim.move_stats."""
        c = self._counters(move)
        return (self._attempts[move], c[0], c[1])

    def observable_accumulate(self, obs):
        self._ok(self._L.refsim_obs_accumulate(self._h, obs))

    def observable_block(self, obs, cap=1 << 20):
        out = np.zeros(cap)
        n = C.c_uint64()
        self._ok(self._L.refsim_obs_write(self._h, obs, out.ctypes.data_as(_DP), cap, C.byref(n)))
        return out[: n.value].copy()

    def run(self, xml: str):
        """Simulation::Run (simulation_class.h:42-45): the input's <Algorithm> loop of Move, Observable
        and Write events (loop_class.h:34-60; a Write writes every move, then every observable,
        write_class.h:31-42), one attempt per Move event. Returns ({move: [(n_attempt, n_accept,
        n_level)] per Write}, {observable (its place among the input's observables): [block] per Write
        that appended one}, {permuting move:
        [(attempts, accepts) per cycle length] per Write})."""
        import xml.etree.ElementTree as ET
        root = ET.fromstring(xml)
        moves = [m.get("name") for m in root.find("Moves") if m.get("type") in MOVE_TYPES]
        all_obs = [o.get("name") for o in root.find("Observables")]
        obs = [o.get("name") for o in root.find("Observables") if o.get("type") in OBSERVABLE_TYPES]
        mstats = {i: [] for i in range(len(moves))}
        blocks = {all_obs.index(n): [] for n in obs}  # keyed by the observable's place in the input
        pstats = {i: [] for i, mv in enumerate(self._moves) if mv[0] != "Bisect"}

        def loop(node):
            for _ in range(int(node.get("n_step", "1"))):
                for ev in node:
                    if ev.tag == "Move" and ev.get("name") in moves:
                        self.move_attempts(moves.index(ev.get("name")), 1)
                    elif ev.tag == "Observable" and ev.get("name") in obs:
                        self.observable_accumulate(obs.index(ev.get("name")))
                    elif ev.tag == "Write":
                        for m in range(len(moves)):
                            if m in pstats:  # the block's counters, which the Write appends and resets
                                pstats[m].append(np.stack(self.perm_stats(m, self._species[self._moves[m][1]][1])))
                            mstats[m].append(self.move_write(m))
                        for o in range(len(obs)):
                            b = self.observable_block(o)
                            if b.size:
                                blocks[all_obs.index(obs[o])].append(b)
                    elif ev.tag == "Loop":
                        loop(ev)

        loop(root.find("Algorithm"))
        return mstats, blocks, pstats
