"""pimc_get_action_noalloc against pimc_get_action, through the C interface.

The no-allocation entry point serves callers that cannot let a library call cudaMalloc during a
run: host programs that have given the GPU's memory to their own pool, or code that calls this
library from a place where device allocation is not allowed. It must return the value the normal
entry point returns (tolerance 1e-10 relative, the FP64 action tolerance of the parity tests), on
consecutive calls that share its fixed scratch array, and refuse requests that do not fit.

This file is collected last so that a run stopping at the first failure has already run every
other test; it also passes when run alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from simpimc_gb300 import Simulation
from simpimc_gb300.configs import electron_gas

pytestmark = pytest.mark.gpu

_U32P = C.POINTER(C.c_uint32)
_DP = C.POINTER(C.c_double)


def _bind(lib):
    fn = lib.pimc_get_action_noalloc
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, _U32P, _U32P, C.c_uint32, C.c_uint32, C.c_int, _DP]
    return fn


def _noalloc(fn, sim, action, b0, b1, particles, level, mode):
    sp = np.array([p[0] for p in particles], dtype=np.uint32)
    pi = np.array([p[1] for p in particles], dtype=np.uint32)
    out = C.c_double()
    rc = fn(sim._h, action, b0, b1, sp.ctypes.data_as(_U32P), pi.ctypes.data_as(_U32P), len(sp), level, mode, C.byref(out))
    return rc, out.value


def test_noalloc_matches_get_action(tmp_path, gpu_lib):
    fn = _bind(gpu_lib)
    xml, path = electron_gas(tmp_path, n_part=14, n_bead=16, n_level=2, rs=2.0, k_cut_units=4.0, seed=17)
    sim = Simulation(xml, base_dir=tmp_path)
    sim.set_path(path)
    rng = np.random.default_rng(3)
    new = path.copy()
    for b in range(5, 9):
        new[2, b] += 0.2 * rng.standard_normal(3)
    sim.set_path(new, 1)
    pair_actions = [a for a in range(sim.n_actions) if "BarePairAction" in sim.name(1, a)]
    assert pair_actions
    for a in pair_actions:
        for mode in (0, 1):
            ref = sim.get_action(a, 4, 8, [(0, 2)], 0, mode)
            for _ in range(2):  # two calls in a row share the scratch array
                rc, val = _noalloc(fn, sim, a, 4, 8, [(0, 2)], 0, mode)
                assert rc == 0, sim._lib.pimc_last_error(sim._h)
                assert abs(val - ref) <= 1e-10 * max(1.0, abs(ref)), (a, mode, val, ref)
    sim.close()


def test_noalloc_refuses_oversize(tmp_path, gpu_lib):
    fn = _bind(gpu_lib)
    xml, path = electron_gas(tmp_path, n_part=66, n_bead=128, n_level=4, rs=2.0, k_cut_units=12.0, seed=19)
    sim = Simulation(xml, base_dir=tmp_path)
    sim.set_path(path)
    a = [a for a in range(sim.n_actions) if "BarePairAction" in sim.name(1, a)][0]
    # NEW-mode long-range over the whole path: 128 slices x 3561 k-vectors x 16 B > 4 MiB.
    rc, _ = _noalloc(fn, sim, a, 0, 128, [(0, 1)], 0, 1)
    assert rc == -1
    assert b"no-allocation limit" in sim._lib.pimc_last_error(sim._h)
    # A segment that fits still works and agrees with the allocating entry point.
    ref = sim.get_action(a, 0, 16, [(0, 1)], 0, 1)
    rc, val = _noalloc(fn, sim, a, 0, 16, [(0, 1)], 0, 1)
    assert rc == 0 and abs(val - ref) <= 1e-10 * max(1.0, abs(ref))
    sim.close()
