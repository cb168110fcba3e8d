"""Failure paths of the library, each made on the host or by a bounded wait; none faults, traps or
hangs the GPU.

The reference reports every failure by printing and exiting (actions.h:32-33). Here each call returns
a status code and the context stays usable:
- a device wait that nothing completes gives up at its time limit (PIMC_ERR_TIMEOUT);
- a non-finite action difference inside the sweep (a coordinate whose square overflows the sweep's
  double-float representation) sets the device error word, and the call returns PIMC_ERR_NONFINITE;
- non-finite coordinates are refused at upload, single chain and batched;
- a missing pair-action table is refused at creation (PIMC_ERR_INPUT).
"""
import numpy as np
import pytest

from simpimc_gb300 import ChainBatch, PimcError, Simulation
from simpimc_gb300.configs import electron_gas, trapped_coulomb

pytestmark = pytest.mark.gpu

ERR_ARG, ERR_INPUT, ERR_TIMEOUT, ERR_NONFINITE = -1, -2, -4, -5


def test_wait_limit_gives_up_and_context_recovers(tmp_path, gpu_lib, oracle_mod):
    xml, path = electron_gas(tmp_path, n_part=14, n_bead=16, n_level=2, rs=2.0, k_cut_units=4.0, seed=31)
    g = Simulation(xml, base_dir=tmp_path)
    g.set_path(path)
    limit = 2_000_000  # 2 ms
    rc, waited = g.check_wait_limit(limit)
    assert rc == ERR_TIMEOUT
    assert b"timed out" in g._lib.pimc_last_error(g._h)
    assert limit <= waited < limit + 500_000_000, waited
    rc, _ = g.check_wait_limit(20_000_000_000)  # above the 10 s bound of the check
    assert rc == ERR_ARG
    # the path was not touched: the context still replays the oracle
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    c.set_path(path)
    g.sweep([0, 1], [7, 7], n_rep=4)
    for _ in range(4):
        c.move_attempts(0, 7)
        c.move_attempts(1, 7)
    for m in range(2):
        assert g.move_stats(m) == c.move_stats(m)
    assert np.max(np.abs(g.get_path(1) - c.get_path(1))) < 1e-9
    g.close()
    c.close()


def test_sweep_reports_nonfinite_action_difference(tmp_path, gpu_lib):
    """The sweep keeps positions as double-float pairs of FP32 numbers, so squares of coordinates and
    displacements above ~3e38 overflow there (in FP64 they would not). One bead at 1e20 makes every
    attempt whose segment reaches it form a non-finite action difference; the sweep stops and the
    call returns PIMC_ERR_NONFINITE instead of accepting or rejecting on it."""
    xml, path = trapped_coulomb(tmp_path, n_part=4, n_bead=16, n_level=2, seed=13)
    path = np.array(path)
    path[0, 6, 0] = 1.0e20
    g = Simulation(xml, base_dir=tmp_path)
    g.set_path(path)
    with pytest.raises(PimcError) as e:
        g.move_attempts(0, 2000)
    assert e.value.code == ERR_NONFINITE, e.value
    # a finite start makes the same context usable again
    _, good = trapped_coulomb(tmp_path, n_part=4, n_bead=16, n_level=2, seed=13)
    g.set_path(good)
    g.move_attempts(0, 200)
    assert np.all(np.isfinite(g.get_path(1)))
    g.close()


def test_nonfinite_coordinates_refused(tmp_path, gpu_lib):
    xml, path = trapped_coulomb(tmp_path, n_part=4, n_bead=16, n_level=2, seed=17)
    g = Simulation(xml, base_dir=tmp_path)
    g.set_path(path)
    bad = np.array(path)
    bad[2, 5, 1] = np.nan
    with pytest.raises(PimcError) as e:
        g.set_path(bad)
    assert e.value.code == ERR_NONFINITE
    assert np.array_equal(g.get_path(0), np.asarray(path))  # nothing was uploaded
    g.close()

    items = [trapped_coulomb(tmp_path, n_part=n, n_bead=m, n_level=2, seed=50 + n) for n, m in ((5, 16), (9, 32))]
    b = ChainBatch([x for x, _ in items], base_dir=tmp_path)
    flat = np.concatenate([np.asarray(p, dtype=np.float32).astype(np.float64).ravel() for _, p in items])
    b.set_paths(flat)
    bad = flat.copy()
    bad[-7] = np.inf
    with pytest.raises(PimcError) as e:
        b.set_paths(bad)
    assert e.value.code == ERR_ARG
    b.set_paths(flat)  # the batch accepts a finite upload afterwards and runs
    b.attempts(20)
    assert np.all(np.isfinite(b.get_paths()))
    b.close()


def test_missing_table_refused_at_create(tmp_path, gpu_lib):
    xml, _ = trapped_coulomb(tmp_path, n_part=4, n_bead=16, n_level=2, seed=1)
    xml = xml.replace('file="coulomb_open.pat"', 'file="no_such_table.pat"')
    with pytest.raises(PimcError) as e:
        Simulation(xml, base_dir=tmp_path)
    assert e.value.code == ERR_INPUT
    assert "no_such_table" in str(e.value)
