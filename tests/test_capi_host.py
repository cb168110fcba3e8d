"""Host-side checks of the C interface: the library builds and loads, exports every entry point
that include/simpimc_gb300.h declares, and rejects bad input before any device work."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "simpimc_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pimc_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from simpimc_gb300 import build as B
    B.build()
    return C.CDLL(str(B.LIB))


def test_header_declares_the_interface():
    names = declared_functions()
    for want in ("pimc_create", "pimc_destroy", "pimc_get_action", "pimc_get_action_gradient", "pimc_dactiondbeta",
                 "pimc_potential", "pimc_virial_energy", "pimc_sweep", "pimc_move_attempts", "pimc_observable_accumulate",
                 "pimc_observable_block", "pimc_run", "pimc_get_action_noalloc"):
        assert want in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_interface():
    import simpimc_gb300
    declared = set(declared_functions())
    bound = set(simpimc_gb300.SIGNATURES)
    # pimc_get_action_noalloc is bound by its own test through ctypes directly.
    assert declared - bound <= {"pimc_get_action_noalloc"}, declared - bound


def test_malformed_input_is_an_error_code(lib):
    lib.pimc_create.restype = C.c_int
    lib.pimc_create.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_uint32, C.POINTER(C.c_void_p)]
    lib.pimc_last_error.restype = C.c_char_p
    lib.pimc_last_error.argtypes = [C.c_void_p]
    h = C.c_void_p()
    assert lib.pimc_create(b"<Input><System", b".", 0, 0, C.byref(h)) == -2
    assert b"XML parse error" in lib.pimc_last_error(None)
    assert not h.value
    assert lib.pimc_create(None, b".", 0, 0, C.byref(h)) == -1
    # concurrent-attempt count outside 0..8 is rejected before the context is touched
    lib.pimc_set_sweep_wave.restype = C.c_int
    lib.pimc_set_sweep_wave.argtypes = [C.c_void_p, C.c_int]
    assert lib.pimc_set_sweep_wave(None, 9) == -1
    # the many-chain sweep and the permutation calls check their pointers before any device work
    lib.pimc_sweep_chains.restype = C.c_int
    lib.pimc_sweep_chains.argtypes = [C.POINTER(C.c_void_p), C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint64]
    assert lib.pimc_sweep_chains(None, 1, None, None, 0, 1) == -1
    arr = (C.c_void_p * 2)(None, None)
    assert lib.pimc_sweep_chains(arr, 0, None, None, 0, 1) == -1
    assert lib.pimc_sweep_chains(arr, 2, None, None, 0, 1) == -1
    for name in ("pimc_get_perm", "pimc_set_perm"):
        fn = getattr(lib, name)
        fn.restype = C.c_int
        fn.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p]
        assert fn(None, 0, None) == -1
    lib.pimc_perm_stats.restype = C.c_int
    lib.pimc_perm_stats.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_size_t]
    assert lib.pimc_perm_stats(None, 0, None, 0) == -1
    assert lib.pimc_set_sweep_wave(None, -1) == -1


def test_binding_fails_loudly_without_library(tmp_path):
    import simpimc_gb300
    with pytest.raises(RuntimeError, match="not built"):
        simpimc_gb300.load_library(tmp_path / "missing.so")


@pytest.mark.parametrize("edit,code", [
    (('n_images="0"', 'n_images="2"'), -6),                           # Kinetic with periodic images
    (('type="Bisect"', 'type="Bisect" adaptive="1" target_ratio="0.5"'), -6),
    (('n_level="2"', 'n_level="6"'), -6),                              # segment beyond 32 beads
    (('n_bead="8"', 'n_bead="2"'), -2),                                # segment longer than the path
    (('is_coulomb="1"', 'is_coulomb="0"'), -6),
])
def test_batch_rejects_inputs_before_device_work(lib, tmp_path, edit, code):
    """Chain inputs are parsed before any CUDA call, so these errors are reported without a GPU."""
    import simpimc_gb300
    from simpimc_gb300.configs import trapped_coulomb
    xml, _ = trapped_coulomb(tmp_path, n_part=4, n_bead=8, n_level=2, seed=1)
    bad = xml.replace(*edit)
    assert bad != xml
    with pytest.raises(simpimc_gb300.PimcError) as e:
        simpimc_gb300.ChainBatch([xml, bad], base_dir=tmp_path)
    assert e.value.code == code, str(e.value)
