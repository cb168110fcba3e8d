"""pimc_get_action_noalloc against pimc_get_action, through the C interface.

The no-allocation entry point serves callers that cannot let a library call cudaMalloc during a
run: host programs that have given the GPU's memory to their own pool, or code that calls this
library from a place where device allocation is not allowed. It must return the value the normal
entry point returns (tolerance 1e-10 relative, the FP64 action tolerance of the parity tests), on
consecutive calls that share its fixed scratch array, leave the GPU's free memory unchanged, and
refuse requests that do not fit.

This file is collected last so that a run stopping at the first failure has already run every
other test; it also passes when run alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from simpimc_gb300 import PimcError, Simulation
from simpimc_gb300.configs import electron_gas, trapped_coulomb

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


def _close(val, ref):
    return abs(val - ref) <= 1e-10 * max(1.0, abs(ref))


def _pair_actions(sim):
    return [a for a in range(sim.n_actions) if "PairAction" in sim.name(1, a)]


def _moved(sim, path, particle, slices, seed):
    new = path.copy()
    rng = np.random.default_rng(seed)
    for b in slices:
        new[particle, b] += 0.2 * rng.standard_normal(3)
    sim.set_path(new, 1)


def _check_pairs(fn, sim, cases):
    """Both entry points on every (action, b0, b1, particles, level, mode) case, two no-alloc calls each."""
    for a, b0, b1, parts, level, mode in cases:
        ref = sim.get_action(a, b0, b1, parts, level, mode)
        for _ in range(2):  # two calls in a row share the scratch array
            rc, val = _noalloc(fn, sim, a, b0, b1, parts, level, mode)
            assert rc == 0, sim._lib.pimc_last_error(sim._h)
            assert _close(val, ref), (a, b0, b1, level, mode, val, ref)


def test_noalloc_matches_get_action(tmp_path, gpu_lib):
    fn = _bind(gpu_lib)
    xml, path = electron_gas(tmp_path, n_part=14, n_bead=16, n_level=2, rs=2.0, k_cut_units=4.0, seed=17)
    sim = Simulation(xml, base_dir=tmp_path)
    sim.set_path(path)
    _moved(sim, path, 2, range(5, 9), 3)
    pair_actions = _pair_actions(sim)
    assert pair_actions
    _check_pairs(fn, sim, [(a, 4, 8, [(0, 2)], 0, mode) for a in pair_actions for mode in (0, 1)])
    sim.close()


def test_noalloc_table_actions_above_level_zero(tmp_path, gpu_lib):
    """DavidPairAction reads its table of index `level` (david_pair_action_class.h:63-102), with
    max_level 1 here: levels 0 and 1 in both modes, level 2 is zero on both sides."""
    fn = _bind(gpu_lib)
    xml, path = trapped_coulomb(tmp_path, n_part=6, n_bead=16, n_level=2, seed=5, pair="DavidPairAction", n_order=2,
                                pair_max_level=1)
    sim = Simulation(xml, base_dir=tmp_path)
    sim.set_path(path)
    _moved(sim, path, 3, range(3, 8), 8)
    a = _pair_actions(sim)[0]
    _check_pairs(fn, sim, [(a, 2, 10, [(0, 3)], level, mode) for level in (0, 1, 2) for mode in (0, 1)])
    sim.close()


@pytest.mark.parametrize("pair", ["IlkkaPairAction", "DavidPairAction"])
def test_noalloc_table_long_range(tmp_path, gpu_lib, pair):
    """Tabulated pair actions with an Ewald part: u_long_k in place of tau v_long_k, NEW-mode densities
    formed from the listed particles (ilkka_pair_action_class.h:104-122, david_pair_action_class.h:105-123)."""
    fn = _bind(gpu_lib)
    xml, path = electron_gas(tmp_path, n_part=14, n_bead=16, n_level=2, rs=2.0, k_cut_units=4.0, seed=21, pair=pair, n_order=1)
    sim = Simulation(xml, base_dir=tmp_path)
    sim.set_path(path)
    _moved(sim, path, 9, range(6, 11), 4)
    acts = _pair_actions(sim)
    assert acts
    # particle 9 is a down spin: the cross action sees it as species b
    _check_pairs(fn, sim, [(a, 5, 12, [(1, 9 - 7)], 0, mode) for a in acts for mode in (0, 1)])
    sim.close()


def test_noalloc_leaves_free_memory_unchanged(tmp_path, gpu_lib):
    """After pimc_create, no-alloc calls leave the device's free memory as it was: the scratch array
    and the kernels the call launches were loaded when the context was created."""
    torch = pytest.importorskip("torch")
    fn = _bind(gpu_lib)
    xml, path = electron_gas(tmp_path, n_part=14, n_bead=16, n_level=2, rs=2.0, k_cut_units=4.0, seed=29)
    sim = Simulation(xml, base_dir=tmp_path)
    sim.set_path(path)
    _moved(sim, path, 4, range(2, 7), 6)
    a = _pair_actions(sim)[0]
    refs = [sim.get_action(a, 1, 9, [(0, 4)], 0, mode) for mode in (0, 1)]
    torch.cuda.mem_get_info(0)  # torch's own first-use set-up, before the reading that counts
    free0, _ = torch.cuda.mem_get_info(0)
    vals = []
    for _ in range(2):
        for mode in (0, 1):
            rc, v = _noalloc(fn, sim, a, 1, 9, [(0, 4)], 0, mode)
            assert rc == 0, sim._lib.pimc_last_error(sim._h)
            vals.append(v)
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0, (free0, free1)
    for i, v in enumerate(vals):
        assert _close(v, refs[i % 2]), (i, v, refs[i % 2])
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
    assert rc == 0 and _close(val, ref)
    sim.close()


def test_noalloc_refuses_ranges_past_one_wrap(tmp_path, gpu_lib):
    """M = 10 at level 2 from b0 = 9 to b1 = 19: the last link's far slice is 21 >= 2M, beyond the one
    wrap the reference's bead_loop makes (species_class.h:101). Both entry points refuse it."""
    fn = _bind(gpu_lib)
    xml, path = trapped_coulomb(tmp_path, n_part=4, n_bead=10, n_level=2, seed=3, pair="DavidPairAction", n_order=1,
                                pair_max_level=2)
    sim = Simulation(xml, base_dir=tmp_path)
    sim.set_path(path)
    a = _pair_actions(sim)[0]
    rc, _ = _noalloc(fn, sim, a, 9, 19, [(0, 1)], 2, 0)
    assert rc == -1
    assert b"one wrap" in sim._lib.pimc_last_error(sim._h)
    with pytest.raises(PimcError, match="one wrap"):
        sim.get_action(a, 9, 19, [(0, 1)], 2, 0)
    with pytest.raises(PimcError, match="one wrap"):
        sim.get_action_gradient(a, 9, 19, [(0, 1)], 2, 0)
    # a range whose links end inside one wrap still agrees
    _check_pairs(fn, sim, [(a, 9, 17, [(0, 1)], 2, 0), (a, 6, 16, [(0, 1)], 1, 1)])
    sim.close()
