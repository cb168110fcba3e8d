"""FP32 sweep mode (FP32 per-slice densities, bead phases and Ewald differences with compensated
sums; double-float positions, pair links and acceptance) against the FP64 oracle.

Tolerances: the draws are shared, so accept counts match the oracle exactly and positions to
1e-9 (no decision lies within the FP32 error of its threshold for these seeds); densities after
the run within 2e-5 absolute per component (FP32 phases and sums of up to 33 unit phases);
estimator values within 1e-5 relative (FP32-accurate densities fed to the FP64 estimators).
"""
import numpy as np
import pytest

from simpimc_gb300 import Simulation
from simpimc_gb300.configs import electron_gas

pytestmark = pytest.mark.gpu


def test_fp32_mode_replays_oracle(tmp_path, gpu_lib, oracle_mod):
    xml, path = electron_gas(tmp_path, n_part=14, n_bead=16, n_level=2, rs=2.0, k_cut_units=4.0, seed=9)
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_precision(32)
    g.set_path(path)
    c.set_path(path)
    g.sweep([0, 1], [7, 7], n_rep=20)
    for _ in range(20):
        c.move_attempts(0, 7)
        c.move_attempts(1, 7)
    for m in range(2):
        assert g.move_stats(m) == c.move_stats(m)
    assert np.max(np.abs(g.get_path(1) - c.get_path(1))) < 1e-9
    for s in range(2):
        assert np.max(np.abs(g.rho_k(s) - c.rho_k(s))) < 2e-5
    for a in range(g.n_actions):
        gd, cd = g.dactiondbeta(a), c.dactiondbeta(a)
        assert abs(gd - cd) <= 1e-5 * max(1.0, abs(cd)), (a, gd, cd)
    g.close()
    c.close()


def test_precision_switch_keeps_the_chain(tmp_path, gpu_lib, oracle_mod):
    """Switching precision between sweep calls continues the same Markov chain."""
    xml, path = electron_gas(tmp_path, n_part=10, n_bead=16, n_level=2, rs=2.0, k_cut_units=4.0, seed=15)
    g = Simulation(xml, base_dir=tmp_path)
    c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    g.set_path(path)
    c.set_path(path)
    for bits in (32, 64, 32):
        g.set_precision(bits)
        g.sweep([0, 1], [5, 5], n_rep=6)
        for _ in range(6):
            c.move_attempts(0, 5)
            c.move_attempts(1, 5)
    for m in range(2):
        assert g.move_stats(m) == c.move_stats(m)
    assert np.max(np.abs(g.get_path(1) - c.get_path(1))) < 1e-9
    g.close()
    c.close()
