"""simpimc_gb300: GB300 (sm_103a) path-integral Monte Carlo action/estimator library.

Python binding of the C interface in include/simpimc_gb300.h (ctypes, no torch types). The
`Simulation` class mirrors the reference's Simulation/Action/Move/Observable surface:
``get_action`` is Action::GetAction, ``dactiondbeta`` is Action::DActionDBeta, ``move_attempts``
is Move::DoEvent repeated, ``observable_block`` is Observable::Write, ``run`` is Simulation::Run.

There is no CPU fallback: if the CUDA library has not been built, importing the binding's
library raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

__all__ = ["Simulation", "ChainBatch", "PimcError", "load_library", "LIB_PATH", "sweep_chains"]

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libsimpimc_gb300.so"

_ERRORS = {
    -1: "PIMC_ERR_ARG",
    -2: "PIMC_ERR_INPUT",
    -3: "PIMC_ERR_CUDA",
    -4: "PIMC_ERR_TIMEOUT",
    -5: "PIMC_ERR_NONFINITE",
    -6: "PIMC_ERR_UNSUPPORTED",
    -7: "PIMC_ERR_STATE",
}


class PimcError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_ERRORS.get(code, code)}: {msg}")
        self.code = code


class _Info(C.Structure):
    _fields_ = [("n_d", C.c_uint32), ("n_bead", C.c_uint32), ("n_species", C.c_uint32), ("n_total", C.c_uint32),
                ("n_k", C.c_uint32), ("n_actions", C.c_uint32), ("n_moves", C.c_uint32), ("n_observables", C.c_uint32),
                ("beta", C.c_double), ("tau", C.c_double), ("L", C.c_double), ("volume", C.c_double), ("pbc", C.c_int32)]


# Exported symbols and argtypes (kept in step with include/simpimc_gb300.h).
_P = C.c_void_p
_U32P = C.POINTER(C.c_uint32)
_U64P = C.POINTER(C.c_uint64)
_DP = C.POINTER(C.c_double)
_SZP = C.POINTER(C.c_size_t)
SIGNATURES = {
    "pimc_create": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int, C.c_uint32, C.POINTER(_P)]),
    "pimc_destroy": (None, [_P]),
    "pimc_last_error": (C.c_char_p, [_P]),
    "pimc_get_info": (C.c_int, [_P, C.POINTER(_Info)]),
    "pimc_set_seed": (C.c_int, [_P, C.c_uint32]),
    "pimc_get_name": (C.c_int, [_P, C.c_int, C.c_uint32, C.c_char_p, C.c_size_t]),
    "pimc_species_info": (C.c_int, [_P, C.c_uint32, _U32P, _U32P, _DP]),
    "pimc_set_path": (C.c_int, [_P, C.c_int, _DP]),
    "pimc_get_path": (C.c_int, [_P, C.c_int, _DP]),
    "pimc_get_rho_k": (C.c_int, [_P, C.c_uint32, _DP]),
    "pimc_get_kvecs": (C.c_int, [_P, _DP]),
    "pimc_get_action": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.c_uint32, _U32P, _U32P, C.c_uint32, C.c_uint32, C.c_int, _DP]),
    "pimc_get_action_gradient": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.c_uint32, _U32P, _U32P, C.c_uint32, C.c_uint32, C.c_int, _DP]),
    "pimc_get_action_gradient_exact": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.c_uint32, _U32P, _U32P, C.c_uint32, C.c_uint32, C.c_int, _DP]),
    "pimc_total_action": (C.c_int, [_P, C.c_int, C.c_int, _DP]),
    "pimc_set_precision": (C.c_int, [_P, C.c_int]),
    "pimc_action_gradient_path": (C.c_int, [_P, C.c_int, C.c_int, _DP]),
    "pimc_dactiondbeta": (C.c_int, [_P, C.c_uint32, _DP]),
    "pimc_potential": (C.c_int, [_P, C.c_uint32, _DP]),
    "pimc_virial_energy": (C.c_int, [_P, C.c_uint32, C.c_double, _DP]),
    "pimc_move_attempts": (C.c_int, [_P, C.c_uint32, C.c_uint64]),
    "pimc_sweep": (C.c_int, [_P, _U32P, _U64P, C.c_uint32, C.c_uint64]),
    "pimc_move_stats": (C.c_int, [_P, C.c_uint32, _U64P]),
    "pimc_get_perm": (C.c_int, [_P, C.c_uint32, _U32P]),
    "pimc_sweep_chains": (C.c_int, [C.POINTER(_P), C.c_uint32, _U32P, _U64P, C.c_uint32, C.c_uint64]),
    "pimc_set_perm": (C.c_int, [_P, C.c_uint32, _U32P]),
    "pimc_perm_stats": (C.c_int, [_P, C.c_uint32, _U64P, C.c_size_t]),
    "pimc_observable_accumulate": (C.c_int, [_P, C.c_uint32]),
    "pimc_observable_block": (C.c_int, [_P, C.c_uint32, _DP, C.c_size_t, _SZP]),
    "pimc_run": (C.c_int, [_P]),
    "pimc_write_output": (C.c_int, [_P, C.c_char_p]),
    "pimc_n_blocks": (C.c_int, [_P, C.c_uint32, _SZP]),
    "pimc_get_block": (C.c_int, [_P, C.c_uint32, C.c_size_t, _DP, C.c_size_t, _SZP]),
    "pimc_synchronize": (C.c_int, [_P]),
    "pimc_set_sweep_grid": (C.c_int, [_P, C.c_int]),
    "pimc_set_timeout_ns": (C.c_int, [_P, C.c_uint64]),
    "pimc_check_wait_limit": (C.c_int, [_P, C.c_uint64, _U64P]),
    "pimc_set_sweep_wave": (C.c_int, [_P, C.c_int]),
    "pimc_stream": (_P, [_P]),
    "pimc_sweep_timing": (C.c_int, [_P, C.c_int, _U64P]),
    "pimc_batch_create": (C.c_int, [C.POINTER(C.c_char_p), C.c_uint32, C.c_char_p, C.c_int, C.POINTER(_P)]),
    "pimc_batch_destroy": (None, [_P]),
    "pimc_batch_last_error": (C.c_char_p, [_P]),
    "pimc_batch_chain_info": (C.c_int, [_P, C.c_uint32, _U32P]),
    "pimc_batch_set_path": (C.c_int, [_P, C.c_uint32, _DP]),
    "pimc_batch_get_path": (C.c_int, [_P, C.c_uint32, _DP]),
    "pimc_batch_set_paths": (C.c_int, [_P, _DP]),
    "pimc_batch_get_paths": (C.c_int, [_P, _DP]),
    "pimc_batch_last_energy": (C.c_int, [_P, _DP]),
    "pimc_batch_attempts": (C.c_int, [_P, C.c_uint64]),
    "pimc_batch_sweeps": (C.c_int, [_P, C.c_uint64]),
    "pimc_batch_measure": (C.c_int, [_P]),
    "pimc_batch_run": (C.c_int, [_P, C.c_uint64, C.c_uint64]),
    "pimc_batch_sync": (C.c_int, [_P]),
    "pimc_batch_energy": (C.c_int, [_P, C.c_uint32, _DP, C.c_uint64, _U64P]),
    "pimc_batch_reset_energy": (C.c_int, [_P]),
    "pimc_batch_counters": (C.c_int, [_P, _U64P, _U64P]),
    "pimc_batch_rounds": (C.c_int, [_P, _U64P]),
    "pimc_batch_set_overlap": (C.c_int, [_P, C.c_uint32]),
    "pimc_batch_get_overlap": (C.c_int, [_P, _U32P]),
    "pimc_batch_set_split": (C.c_int, [_P, C.c_uint32]),
    "pimc_batch_get_split": (C.c_int, [_P, _U32P]),
    "pimc_batch_hmc_attempts": (C.c_int, [_P, C.c_uint64]),
    "pimc_batch_hmc_counters": (C.c_int, [_P, _U64P, _U64P]),
    "pimc_batch_set_hmc_per_cycle": (C.c_int, [_P, C.c_uint64]),
    "pimc_batch_set_hmc_cluster": (C.c_int, [_P, C.c_uint32]),
    "pimc_batch_get_hmc_cluster": (C.c_int, [_P, _U32P]),
    "pimc_batch_set_tiles": (C.c_int, [_P, C.c_uint32, C.c_uint32, C.c_uint32]),
    "pimc_batch_autotune": (C.c_int, [_P, C.c_uint32, _U32P, _U32P, _U32P, _DP]),
    "pimc_batch_stats": (C.c_int, [_P, _U64P]),
    "pimc_batch_stream": (C.c_int, [_P, C.POINTER(_P)]),
}

SWEEP_PHASES = ("segment+rng", "sampling", "level terms", "grid work", "grid barrier", "final sum", "decision", "commit",
                "role:sampling chain", "role:stored level sums", "role:old tables", "role:stored pair links",
                "role:working level sums", "role:new tables", "role:old Ewald phases", "role:grid pair+Ewald")

_lib = None


def load_library(path: os.PathLike | None = None):
    """Load the CUDA library (raises if it has not been built: there is no fallback)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"simpimc_gb300 CUDA library not built: {p} is missing (run __graft_entry__.build())")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_DP)


class Simulation:
    """One simulation on one GPU, built from a simpimc XML input."""

    def __init__(self, xml: str, base_dir: str | os.PathLike = ".", device: int = 0, chain: int = 0):
        self._lib = load_library()
        h = _P()
        rc = self._lib.pimc_create(xml.encode(), str(base_dir).encode(), device, chain, C.byref(h))
        if rc != 0:
            raise PimcError(rc, self._lib.pimc_last_error(None).decode())
        self._h = h
        info = _Info()
        self._check(self._lib.pimc_get_info(self._h, C.byref(info)))
        self.n_d, self.n_bead, self.n_species = info.n_d, info.n_bead, info.n_species
        self.n_total, self.n_k = info.n_total, info.n_k
        self.n_actions, self.n_moves, self.n_observables = info.n_actions, info.n_moves, info.n_observables
        self.beta, self.tau, self.L, self.volume, self.pbc = info.beta, info.tau, info.L, info.volume, bool(info.pbc)

    # -- plumbing -------------------------------------------------------------------------------
    def _check(self, rc: int):
        if rc != 0:
            raise PimcError(rc, self._lib.pimc_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pimc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def name(self, kind: int, index: int) -> str:
        buf = C.create_string_buffer(256)
        self._check(self._lib.pimc_get_name(self._h, kind, index, buf, 256))
        return buf.value.decode()

    def species_info(self, s: int):
        n, off, lam = C.c_uint32(), C.c_uint32(), C.c_double()
        self._check(self._lib.pimc_species_info(self._h, s, C.byref(n), C.byref(off), C.byref(lam)))
        return n.value, off.value, lam.value

    def set_seed(self, seed: int):
        self._check(self._lib.pimc_set_seed(self._h, seed))

    def set_sweep_grid(self, grid: int):
        self._check(self._lib.pimc_set_sweep_grid(self._h, grid))

    def set_precision(self, bits: int):
        """Sweep precision: 64 (double-float densities) or 32 (FP32 densities and phases)."""
        self._check(self._lib.pimc_set_precision(self._h, bits))

    def set_sweep_wave(self, wave: int):
        """Bisection attempts in flight per round of the sweep (1 = one at a time, 0 = automatic)."""
        self._check(self._lib.pimc_set_sweep_wave(self._h, wave))

    def set_timeout_ns(self, ns: int):
        self._check(self._lib.pimc_set_timeout_ns(self._h, ns))

    def check_wait_limit(self, ns: int):
        """One bounded device wait that nothing completes: returns (status code, device-measured
        wait in ns). The status is PIMC_ERR_TIMEOUT (-4) when the limit works."""
        w = C.c_uint64()
        rc = self._lib.pimc_check_wait_limit(self._h, ns, C.byref(w))
        return rc, w.value

    def synchronize(self):
        self._check(self._lib.pimc_synchronize(self._h))

    def sweep_timing(self, enable: int = -1) -> dict:
        """Per-phase cycles of the sweep kernel's block 0 since the last reset (tracing aid);
        enable=1/0 switches recording on/off and resets the sums."""
        out = np.zeros(len(SWEEP_PHASES), dtype=np.uint64)
        self._check(self._lib.pimc_sweep_timing(self._h, enable, out.ctypes.data_as(_U64P)))
        return dict(zip(SWEEP_PHASES, (int(x) for x in out)))

    # -- path -----------------------------------------------------------------------------------
    @property
    def path_shape(self):
        return (self.n_total, self.n_bead, self.n_d)

    def set_path(self, pos: np.ndarray, which: int = 2):
        a = np.ascontiguousarray(pos, dtype=np.float64)
        if a.shape != self.path_shape:
            raise ValueError(f"path must have shape {self.path_shape}, got {a.shape}")
        self._check(self._lib.pimc_set_path(self._h, which, _dp(a)))

    def get_path(self, which: int = 1) -> np.ndarray:
        a = np.empty(self.path_shape, dtype=np.float64)
        self._check(self._lib.pimc_get_path(self._h, which, _dp(a)))
        return a

    def rho_k(self, species: int) -> np.ndarray:
        a = np.empty((self.n_bead, self.n_k, 2), dtype=np.float64)
        self._check(self._lib.pimc_get_rho_k(self._h, species, _dp(a)))
        return a[..., 0] + 1j * a[..., 1]

    def kvecs(self) -> np.ndarray:
        a = np.empty((self.n_k, self.n_d), dtype=np.float64)
        if self.n_k:
            self._check(self._lib.pimc_get_kvecs(self._h, _dp(a)))
        return a

    # -- actions --------------------------------------------------------------------------------
    @staticmethod
    def _parts(particles):
        sp = np.array([p[0] for p in particles], dtype=np.uint32)
        pi = np.array([p[1] for p in particles], dtype=np.uint32)
        return sp, pi

    def get_action(self, action: int, b0: int, b1: int, particles, level: int = 0, mode: int = 1) -> float:
        sp, pi = self._parts(particles)
        out = C.c_double()
        self._check(self._lib.pimc_get_action(self._h, action, b0, b1, sp.ctypes.data_as(_U32P), pi.ctypes.data_as(_U32P),
                                              len(sp), level, mode, C.byref(out)))
        return out.value

    def get_action_gradient(self, action: int, b0: int, b1: int, particles, level: int = 0, mode: int = 1) -> np.ndarray:
        sp, pi = self._parts(particles)
        out = np.zeros(self.n_d, dtype=np.float64)
        self._check(self._lib.pimc_get_action_gradient(self._h, action, b0, b1, sp.ctypes.data_as(_U32P), pi.ctypes.data_as(_U32P),
                                                       len(sp), level, mode, _dp(out)))
        return out

    def get_action_gradient_exact(self, action: int, b0: int, b1: int, particles, level: int = 0, mode: int = 1) -> np.ndarray:
        sp, p = self._parts(particles)
        out = np.zeros(self.n_d, dtype=np.float64)
        self._check(self._lib.pimc_get_action_gradient_exact(self._h, action, b0, b1, sp.ctypes.data_as(_U32P), p.ctypes.data_as(_U32P),
                                                             len(particles), level, mode, _dp(out)))
        return out

    def total_action(self, action: int = -1, mode: int = 0) -> float:
        """Whole-ring action at level 0 of one action, or of every action (-1)."""
        out = C.c_double()
        self._check(self._lib.pimc_total_action(self._h, action, mode, C.byref(out)))
        return out.value

    def action_gradient_path(self, action: int = -1, mode: int = 0) -> np.ndarray:
        """Exact dS/dR of total_action, shaped like the path (n_total, n_bead, n_d)."""
        out = np.zeros((self.n_total, self.n_bead, self.n_d), dtype=np.float64)
        self._check(self._lib.pimc_action_gradient_path(self._h, action, mode, _dp(out)))
        return out

    def dactiondbeta(self, action: int) -> float:
        out = C.c_double()
        self._check(self._lib.pimc_dactiondbeta(self._h, action, C.byref(out)))
        return out.value

    def potential(self, action: int) -> float:
        out = C.c_double()
        self._check(self._lib.pimc_potential(self._h, action, C.byref(out)))
        return out.value

    def virial_energy(self, action: int, window: float) -> float:
        out = C.c_double()
        self._check(self._lib.pimc_virial_energy(self._h, action, float(window), C.byref(out)))
        return out.value

    # -- moves, observables, run ----------------------------------------------------------------
    def move_attempts(self, move: int, n: int):
        self._check(self._lib.pimc_move_attempts(self._h, move, n))

    def sweep(self, moves, counts, n_rep: int = 1):
        mv = np.ascontiguousarray(moves, dtype=np.uint32)
        ct = np.ascontiguousarray(counts, dtype=np.uint64)
        self._check(self._lib.pimc_sweep(self._h, mv.ctypes.data_as(_U32P), ct.ctypes.data_as(_U64P), len(mv), n_rep))

    def get_perm(self, species: int):
        """Path permutation of a species: perm[p] = particle whose slice-0 bead follows (p, M - 1)."""
        n, _, _ = self.species_info(species)
        out = np.zeros(n, dtype=np.uint32)
        self._check(self._lib.pimc_get_perm(self._h, species, out.ctypes.data_as(_U32P)))
        return out.astype(np.int64)

    def set_perm(self, species: int, perm):
        pi = np.ascontiguousarray(perm, dtype=np.uint32)
        self._check(self._lib.pimc_set_perm(self._h, species, pi.ctypes.data_as(_U32P)))

    def perm_stats(self, move: int, n_part: int):
        """Per cycle length: (attempts, accepts) of a permuting move in the current block."""
        out = np.zeros(2 * n_part, dtype=np.uint64)
        self._check(self._lib.pimc_perm_stats(self._h, move, out.ctypes.data_as(_U64P), out.size))
        return out[:n_part].astype(np.int64), out[n_part:].astype(np.int64)

    def move_stats(self, move: int):
        """(total attempts, attempts in block, accepts in block)."""
        return self.move_counters(move)[:3]

    def move_counters(self, move: int):
        """(total attempts, block attempts, block accepts, total accepts, total level-0 tests)."""
        out = np.zeros(5, dtype=np.uint64)
        self._check(self._lib.pimc_move_stats(self._h, move, out.ctypes.data_as(_U64P)))
        return tuple(int(x) for x in out)

    def observable_accumulate(self, obs: int):
        self._check(self._lib.pimc_observable_accumulate(self._h, obs))

    def observable_block(self, obs: int, cap: int = 1 << 20) -> np.ndarray:
        out = np.zeros(cap, dtype=np.float64)
        n = C.c_size_t()
        self._check(self._lib.pimc_observable_block(self._h, obs, _dp(out), cap, C.byref(n)))
        return out[: n.value].copy()

    def run(self):
        self._check(self._lib.pimc_run(self._h))

    def write_output(self, path) -> None:
        """Write the run's output (the reference's dataset paths) to `path`; read it with
        simpimc_gb300.tables.read_table."""
        self._check(self._lib.pimc_write_output(self._h, os.fsencode(str(path))))

    def blocks(self, obs: int, cap: int = 1 << 20) -> list[np.ndarray]:
        n = C.c_size_t()
        self._check(self._lib.pimc_n_blocks(self._h, obs, C.byref(n)))
        out = []
        buf = np.zeros(cap, dtype=np.float64)
        for b in range(n.value):
            m = C.c_size_t()
            self._check(self._lib.pimc_get_block(self._h, obs, b, _dp(buf), cap, C.byref(m)))
            out.append(buf[: m.value].copy())
        return out


def sweep_chains(sims, moves, counts, n_rep: int = 1):
    """pimc_sweep on many independent chains (Simulation objects of the same input structure on
    one device): schedules on the permutation kernel run as one launch with one CTA per chain."""
    if not sims:
        return
    lib = sims[0]._lib
    hs = (_P * len(sims))(*[s._h for s in sims])
    mv = np.ascontiguousarray(moves, dtype=np.uint32)
    ct = np.ascontiguousarray(counts, dtype=np.uint64)
    sims[0]._check(lib.pimc_sweep_chains(hs, len(sims), mv.ctypes.data_as(_U32P), ct.ctypes.data_as(_U64P), len(mv), n_rep))


class ChainBatch:
    """Many independent chains on one GPU (one XML input per chain; chain i replays the
    single-chain context created with ``chain=i`` up to FP32 rounding)."""

    def __init__(self, xmls, base_dir: str | os.PathLike = ".", device: int = 0):
        self._lib = load_library()
        arr = (C.c_char_p * len(xmls))(*[x.encode() for x in xmls])
        h = _P()
        rc = self._lib.pimc_batch_create(arr, len(xmls), str(base_dir).encode(), device, C.byref(h))
        if rc != 0:
            raise PimcError(rc, self._lib.pimc_batch_last_error(None).decode())
        self._h = h
        self.n_chains = len(xmls)
        self.shapes = [self.chain_info(i)[:3] for i in range(self.n_chains)]

    def _check(self, rc: int):
        if rc != 0:
            raise PimcError(rc, self._lib.pimc_batch_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.pimc_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def chain_info(self, chain: int):
        """(n_part, n_bead, n_level, warps of the chain's pair tile)."""
        out = np.zeros(4, dtype=np.uint32)
        self._check(self._lib.pimc_batch_chain_info(self._h, chain, out.ctypes.data_as(_U32P)))
        return tuple(int(x) for x in out)

    def set_path(self, chain: int, pos: np.ndarray):
        n, m, _ = self.shapes[chain]
        a = np.ascontiguousarray(pos, dtype=np.float64)
        if a.shape != (n, m, 3):
            raise ValueError(f"path shape {a.shape} != {(n, m, 3)}")
        self._check(self._lib.pimc_batch_set_path(self._h, chain, _dp(a)))

    def get_path(self, chain: int) -> np.ndarray:
        n, m, _ = self.shapes[chain]
        out = np.zeros((n, m, 3), dtype=np.float64)
        self._check(self._lib.pimc_batch_get_path(self._h, chain, _dp(out)))
        return out

    def set_paths(self, flat: np.ndarray):
        """Every chain's path at once: the chains' (n_part, n_bead, 3) arrays concatenated (copied
        as they are; pinned host memory moves at full link speed)."""
        a = np.ascontiguousarray(flat, dtype=np.float64).ravel()
        if a.size != sum(n * m * 3 for n, m, _ in self.shapes):
            raise ValueError("flat path size does not match the chains")
        self._check(self._lib.pimc_batch_set_paths(self._h, _dp(a)))

    def get_paths(self, out: np.ndarray | None = None) -> np.ndarray:
        """Every chain's path, concatenated; `out` (float64, contiguous, e.g. pinned) is reused."""
        n = sum(n * m * 3 for n, m, _ in self.shapes)
        if out is None:
            out = np.zeros(n, dtype=np.float64)
        if out.dtype != np.float64 or out.size != n or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a contiguous float64 array of the concatenated path size")
        self._check(self._lib.pimc_batch_get_paths(self._h, _dp(out)))
        return out

    def last_energy(self) -> np.ndarray:
        out = np.zeros((self.n_chains, 4), dtype=np.float64)
        self._check(self._lib.pimc_batch_last_energy(self._h, _dp(out)))
        return out

    def attempts(self, n: int):
        self._check(self._lib.pimc_batch_attempts(self._h, n))

    def sweeps(self, n: int):
        self._check(self._lib.pimc_batch_sweeps(self._h, n))

    def measure(self):
        self._check(self._lib.pimc_batch_measure(self._h))

    def run(self, n_cycles: int, sweeps_per_measure: int = 1):
        self._check(self._lib.pimc_batch_run(self._h, n_cycles, sweeps_per_measure))

    def synchronize(self):
        self._check(self._lib.pimc_batch_sync(self._h))

    def energy(self, chain: int, cap: int = 4096) -> tuple[np.ndarray, int]:
        """(series[m, 4] of {E, kinetic, trap, pair} per measurement, measurements since reset)."""
        out = np.zeros((cap, 4), dtype=np.float64)
        n = C.c_uint64()
        self._check(self._lib.pimc_batch_energy(self._h, chain, _dp(out), cap, C.byref(n)))
        return out[: min(n.value, cap)].copy(), int(n.value)

    def reset_energy(self):
        self._check(self._lib.pimc_batch_reset_energy(self._h))

    def counters(self):
        att = np.zeros(self.n_chains, dtype=np.uint64)
        acc = np.zeros(self.n_chains, dtype=np.uint64)
        self._check(self._lib.pimc_batch_counters(self._h, att.ctypes.data_as(_U64P), acc.ctypes.data_as(_U64P)))
        return att, acc

    @property
    def overlap(self) -> int:
        """Heaviest chains run beside the others in the measurement cycle's graph (0: one stream)."""
        n = C.c_uint32()
        self._check(self._lib.pimc_batch_get_overlap(self._h, C.byref(n)))
        return n.value

    @overlap.setter
    def overlap(self, heavy: int):
        self._check(self._lib.pimc_batch_set_overlap(self._h, heavy))

    @property
    def split(self) -> int:
        """Chains running on two-block clusters (the most expensive ones that qualify)."""
        n = C.c_uint32()
        self._check(self._lib.pimc_batch_get_split(self._h, C.byref(n)))
        return n.value

    @split.setter
    def split(self, n: int):
        self._check(self._lib.pimc_batch_set_split(self._h, n))

    def rounds(self):
        """Scheduling rounds of the bisection sweep kernel per chain (attempts / rounds = concurrency)."""
        r = np.zeros(self.n_chains, dtype=np.uint64)
        self._check(self._lib.pimc_batch_rounds(self._h, r.ctypes.data_as(_U64P)))
        return r

    def hmc_attempts(self, n: int):
        """n hybrid Monte Carlo attempts on every chain whose input has an HMC move."""
        self._check(self._lib.pimc_batch_hmc_attempts(self._h, n))

    def hmc_counters(self):
        att = np.zeros(self.n_chains, dtype=np.uint64)
        acc = np.zeros(self.n_chains, dtype=np.uint64)
        self._check(self._lib.pimc_batch_hmc_counters(self._h, att.ctypes.data_as(_U64P), acc.ctypes.data_as(_U64P)))
        return att, acc

    def set_hmc_per_cycle(self, n: int):
        """HMC attempts in every measurement cycle of run() (after the sweeps)."""
        self._check(self._lib.pimc_batch_set_hmc_per_cycle(self._h, n))

    @property
    def hmc_cluster(self) -> int:
        """Thread blocks per chain (one cluster) of the HMC launch."""
        k = C.c_uint32()
        self._check(self._lib.pimc_batch_get_hmc_cluster(self._h, C.byref(k)))
        return k.value

    @hmc_cluster.setter
    def hmc_cluster(self, k: int):
        self._check(self._lib.pimc_batch_set_hmc_cluster(self._h, k))

    def set_tiles(self, items_per_lane: int, max_warps: int, wave: int = 1):
        self._check(self._lib.pimc_batch_set_tiles(self._h, items_per_lane, max_warps, wave))

    def autotune(self, trial_sweeps: int = 2):
        """(items_per_lane, max_warps, wave, seconds per sweep) of the fastest tile, now set."""
        ipl, mw, wv, sec = C.c_uint32(), C.c_uint32(), C.c_uint32(), C.c_double()
        self._check(self._lib.pimc_batch_autotune(self._h, trial_sweeps, C.byref(ipl), C.byref(mw), C.byref(wv), C.byref(sec)))
        return int(ipl.value), int(mw.value), int(wv.value), float(sec.value)

    def stats(self) -> dict:
        out = np.zeros(4, dtype=np.uint64)
        self._check(self._lib.pimc_batch_stats(self._h, out.ctypes.data_as(_U64P)))
        return {"n_chains": int(out[0]), "bead_moves_per_sweep": int(out[1]), "kernel_launches": int(out[2]),
                "series_cap": int(out[3])}

    def stream(self) -> int:
        s = _P()
        self._check(self._lib.pimc_batch_stream(self._h, C.byref(s)))
        return int(s.value or 0)
