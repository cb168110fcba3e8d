"""ORACLE — test infrastructure only (tests/, the smoke check and the bench's CPU-baseline leg).

ctypes wrapper of oracle/oracle.cc, the FP64 CPU restatement of simpimc's action, move and
estimator hot path. The product library never imports this package.
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "lib" / "liboracle.so"
SRC = HERE / "oracle.cc"
DEPS = [SRC, HERE.parent / "simpimc_gb300" / "src" / "framework" / "input.h",
        HERE.parent / "simpimc_gb300" / "src" / "framework" / "table_io.h"]


def build(force: bool = False) -> Path:
    """Compile the oracle with the host C++ compiler (-O3, IEEE arithmetic, no fast-math)."""
    LIB.parent.mkdir(exist_ok=True)
    if force or not LIB.exists() or any(d.stat().st_mtime > LIB.stat().st_mtime for d in DEPS):
        cxx = os.environ.get("CXX") or shutil.which("g++") or "c++"
        cmd = [cxx, "-std=c++17", "-O3", "-ffp-contract=off", "-fPIC", "-shared", "-fopenmp", str(SRC), "-o", str(LIB)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:  # without OpenMP the lean-density sums run on one thread
            r = subprocess.run([c for c in cmd if c != "-fopenmp"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stderr}")
    return LIB


_lib = None
_DP = C.POINTER(C.c_double)
_U32P = C.POINTER(C.c_uint32)
_U64P = C.POINTER(C.c_uint64)


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        L.oracle_last_error.restype = C.c_char_p
        L.oracle_create.argtypes = [C.c_char_p, C.c_char_p, C.c_uint32, C.POINTER(C.c_void_p)]
        L.oracle_destroy.argtypes = [C.c_void_p]
        L.oracle_destroy.restype = None
        for name, args in {
            "oracle_info": [C.c_void_p, _U32P],
            "oracle_seed": [C.c_void_p, C.c_uint32],
            "oracle_set_path": [C.c_void_p, C.c_int, _DP],
            "oracle_get_path": [C.c_void_p, C.c_int, _DP],
            "oracle_kvecs": [C.c_void_p, _DP],
            "oracle_get_rho_k": [C.c_void_p, C.c_uint32, C.c_int, _DP],
            "oracle_get_action": [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, _U32P, _U32P, C.c_uint32, C.c_uint32, C.c_int, _DP],
            "oracle_get_action_gradient": [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, _U32P, _U32P, C.c_uint32, C.c_uint32, C.c_int, _DP],
            "oracle_reset_rho_k_latch": [C.c_void_p],
            "oracle_dactiondbeta": [C.c_void_p, C.c_uint32, _DP],
            "oracle_potential": [C.c_void_p, C.c_uint32, _DP],
            "oracle_virial_energy": [C.c_void_p, C.c_uint32, C.c_double, _DP],
            "oracle_move_attempts": [C.c_void_p, C.c_uint32, C.c_uint64],
            "oracle_total_action": [C.c_void_p, C.c_int, C.c_int, _DP],
            "oracle_action_gradient_path": [C.c_void_p, C.c_int, C.c_int, _DP],
            "oracle_move_stats": [C.c_void_p, C.c_uint32, _U64P],
            "oracle_obs_accumulate": [C.c_void_p, C.c_uint32],
            "oracle_obs_block": [C.c_void_p, C.c_uint32, _DP, C.c_uint64, _U64P],
            "oracle_run": [C.c_void_p],
            "oracle_n_blocks": [C.c_void_p, C.c_uint32, _U64P],
            "oracle_get_block": [C.c_void_p, C.c_uint32, C.c_uint64, _DP, C.c_uint64, _U64P],
            "oracle_move_writes": [C.c_void_p, C.c_uint32, C.POINTER(C.c_int64), C.c_uint64, _U64P, _U64P],
            "oracle_philox": [_U32P, _U32P, _U32P],
            "oracle_perm_stats": [C.c_void_p, C.c_uint32, _U64P],
            "oracle_get_perm": [C.c_void_p, C.c_uint32, _U32P],
            "oracle_set_perm": [C.c_void_p, C.c_uint32, _U32P],
            "oracle_set_lean_densities": [C.c_int],
        }.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = C.c_int
        _lib = L
    return _lib


def bisect_draws(seed, chain, move, attempt, n_part, n_bead, n_level):
    """(particle, first bead), normals [(2^l - 1), 3] and per-level log-uniforms of one attempt."""
    L = lib()
    fn = L.oracle_bisect_draws
    fn.restype = C.c_int
    fn.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, _U32P,
                   C.POINTER(C.c_float), C.POINTER(C.c_float)]
    B = 1 << n_level
    pb = np.zeros(2, dtype=np.uint32)
    z = np.zeros((B - 1, 3), dtype=np.float32)
    lu = np.zeros(n_level, dtype=np.float32)
    fn(seed, chain, move, attempt, n_part, n_bead, n_level, pb.ctypes.data_as(_U32P), z.ctypes.data_as(C.POINTER(C.c_float)),
       lu.ctypes.data_as(C.POINTER(C.c_float)))
    return pb, z, lu


def perm_draws(seed, chain, move, attempt, n_part, n_bead, n_level):
    """Draws of one permuting-bisection attempt in the order the reference's moves consume them:
    (first bead, iterative cycle's first particle), the iterative walk's uniforms [N, 2]
    (continuation, choice per step), the table's selection uniform, normals [N (2^l - 1), 3] in
    sampling order, the level tests' log-uniforms (top level first) and the table's final uniform."""
    L = lib()
    fn = L.oracle_perm_draws
    fn.restype = C.c_int
    fn.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, _U32P, _DP,
                   C.POINTER(C.c_float), C.POINTER(C.c_float), _DP]
    B = 1 << n_level
    idx = np.zeros(2, dtype=np.uint32)
    sel = np.zeros(2 * n_part + 1)
    z = np.zeros((n_part * (B - 1), 3), dtype=np.float32)
    lu = np.zeros(n_level, dtype=np.float32)
    fin = np.zeros(1)
    fn(seed, chain, move, attempt, n_part, n_bead, n_level, idx.ctypes.data_as(_U32P), sel.ctypes.data_as(_DP),
       z.ctypes.data_as(C.POINTER(C.c_float)), lu.ctypes.data_as(C.POINTER(C.c_float)), fin.ctypes.data_as(_DP))
    return idx, sel[:2 * n_part].reshape(n_part, 2), float(sel[2 * n_part]), z, lu, float(fin[0])


def philox(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().oracle_philox(c.ctypes.data_as(_U32P), k.ctypes.data_as(_U32P), out.ctypes.data_as(_U32P))
    return out


class OracleSim:
    """Same surface as simpimc_gb300.Simulation, evaluated by the CPU restatement.

    lean_densities=True keeps only the per-slice charge densities and recomputes each bead's density
    from its position (identical results; needed where the reference's per-bead storage, N M K
    complex numbers twice, does not fit in host memory)."""

    def __init__(self, xml: str, base_dir=".", chain: int = 0, lean_densities: bool = False):
        L = lib()
        h = C.c_void_p()
        L.oracle_set_lean_densities(1 if lean_densities else 0)
        try:
            rc = L.oracle_create(xml.encode(), str(base_dir).encode(), chain, C.byref(h))
        finally:
            L.oracle_set_lean_densities(0)
        if rc != 0:
            raise RuntimeError(L.oracle_last_error().decode())
        self._L, self._h = L, h
        info = np.zeros(8, dtype=np.uint32)
        L.oracle_info(h, info.ctypes.data_as(_U32P))
        (self.n_d, self.n_bead, self.n_species, self.n_total, self.n_k, self.n_actions, self.n_moves,
         self.n_observables) = (int(x) for x in info)

    def _ok(self, rc):
        if rc != 0:
            raise RuntimeError(self._L.oracle_last_error().decode())

    def close(self):
        if self._h:
            self._L.oracle_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def path_shape(self):
        return (self.n_total, self.n_bead, self.n_d)

    def set_seed(self, seed: int):
        self._L.oracle_seed(self._h, seed)

    def set_path(self, pos, which: int = 2):
        a = np.ascontiguousarray(pos, dtype=np.float64)
        assert a.shape == self.path_shape
        self._ok(self._L.oracle_set_path(self._h, which, a.ctypes.data_as(_DP)))

    def get_path(self, which: int = 1):
        a = np.empty(self.path_shape, dtype=np.float64)
        self._ok(self._L.oracle_get_path(self._h, which, a.ctypes.data_as(_DP)))
        return a

    def kvecs(self):
        a = np.empty((self.n_k, self.n_d), dtype=np.float64)
        if self.n_k:
            self._L.oracle_kvecs(self._h, a.ctypes.data_as(_DP))
        return a

    def rho_k(self, species: int, which: int = 1):
        a = np.empty((self.n_bead, self.n_k, 2), dtype=np.float64)
        self._ok(self._L.oracle_get_rho_k(self._h, species, which, a.ctypes.data_as(_DP)))
        return a[..., 0] + 1j * a[..., 1]

    @staticmethod
    def _parts(particles):
        sp = np.array([p[0] for p in particles], dtype=np.uint32)
        pi = np.array([p[1] for p in particles], dtype=np.uint32)
        return sp, pi

    def get_action(self, action, b0, b1, particles, level=0, mode=1):
        sp, pi = self._parts(particles)
        out = C.c_double()
        if mode:
            self._L.oracle_reset_rho_k_latch(self._h)
        self._ok(self._L.oracle_get_action(self._h, action, b0, b1, sp.ctypes.data_as(_U32P), pi.ctypes.data_as(_U32P), len(sp),
                                           level, mode, C.byref(out)))
        return out.value

    def get_action_gradient(self, action, b0, b1, particles, level=0, mode=1):
        sp, pi = self._parts(particles)
        out = np.zeros(3, dtype=np.float64)
        self._ok(self._L.oracle_get_action_gradient(self._h, action, b0, b1, sp.ctypes.data_as(_U32P), pi.ctypes.data_as(_U32P),
                                                    len(sp), level, mode, out.ctypes.data_as(_DP)))
        return out[: self.n_d].copy()

    def dactiondbeta(self, action):
        out = C.c_double()
        self._ok(self._L.oracle_dactiondbeta(self._h, action, C.byref(out)))
        return out.value

    def potential(self, action):
        out = C.c_double()
        self._ok(self._L.oracle_potential(self._h, action, C.byref(out)))
        return out.value

    def virial_energy(self, action, window):
        out = C.c_double()
        self._ok(self._L.oracle_virial_energy(self._h, action, float(window), C.byref(out)))
        return out.value

    def total_action(self, action=-1, mode=0):
        out = C.c_double()
        self._ok(self._L.oracle_total_action(self._h, action, mode, C.byref(out)))
        return out.value

    def action_gradient_path(self, action=-1, mode=0):
        n_total, n_bead, n_d = self.n_total, self.n_bead, self.n_d
        out = np.zeros((n_total, n_bead, n_d), dtype=np.float64)
        self._ok(self._L.oracle_action_gradient_path(self._h, action, mode, out.ctypes.data_as(_DP)))
        return out

    def move_attempts(self, move, n):
        self._ok(self._L.oracle_move_attempts(self._h, move, n))

    def move_stats(self, move):
        out = np.zeros(3, dtype=np.uint64)
        self._L.oracle_move_stats(self._h, move, out.ctypes.data_as(_U64P))
        return int(out[0]), int(out[1]), int(out[2])

    def perm_stats(self, move, n_part):
        out = np.zeros(2 * n_part, dtype=np.uint64)
        self._ok(self._L.oracle_perm_stats(self._h, move, out.ctypes.data_as(_U64P)))
        return out[:n_part].astype(np.int64), out[n_part:].astype(np.int64)

    def get_perm(self, species, n_part):
        out = np.zeros(n_part, dtype=np.uint32)
        self._ok(self._L.oracle_get_perm(self._h, species, out.ctypes.data_as(_U32P)))
        return out.astype(np.int64)

    def set_perm(self, species, perm):
        pi = np.ascontiguousarray(perm, dtype=np.uint32)
        self._ok(self._L.oracle_set_perm(self._h, species, pi.ctypes.data_as(_U32P)))

    def observable_accumulate(self, obs):
        self._ok(self._L.oracle_obs_accumulate(self._h, obs))

    def observable_block(self, obs, cap=1 << 20):
        out = np.zeros(cap, dtype=np.float64)
        n = C.c_uint64()
        self._ok(self._L.oracle_obs_block(self._h, obs, out.ctypes.data_as(_DP), cap, C.byref(n)))
        return out[: n.value].copy()

    def run(self):
        self._ok(self._L.oracle_run(self._h))

    def move_writes(self, move, cap=1 << 20):
        """Rows recorded at each Write of run(): (n_attempt, n_accept, level or -1), then for a
        permuting move its per-cycle-length attempts and accepts."""
        buf = np.zeros(cap, dtype=np.int64)
        n, k = C.c_uint64(), C.c_uint64()
        self._ok(self._L.oracle_move_writes(self._h, move, buf.ctypes.data_as(C.POINTER(C.c_int64)), cap, C.byref(n), C.byref(k)))
        return buf[: n.value * k.value].reshape(n.value, k.value).copy()

    def blocks(self, obs, cap=1 << 20):
        n = C.c_uint64()
        if self._L.oracle_n_blocks(self._h, obs, C.byref(n)) != 0:
            raise IndexError(f"observable {obs} out of range")
        buf = np.zeros(cap, dtype=np.float64)
        out = []
        for b in range(n.value):
            m = C.c_uint64()
            self._ok(self._L.oracle_get_block(self._h, obs, b, buf.ctypes.data_as(_DP), cap, C.byref(m)))
            out.append(buf[: m.value].copy())
        return out
