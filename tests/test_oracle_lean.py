"""The oracle's lean-density mode against its default mode (CPU).

The reference stores every bead's charge density and its copy (bead_class.h:20-21). The oracle's
lean mode keeps only the per-slice densities and recomputes a bead's density from its position
where the reference reads the stored one; the GPU parity tests at sizes where the stored densities
do not fit in host memory (N = 1024, M = 512, K = 25398) use it. Because a stored density always
equals CalcRhoK of that copy's position, the two modes must agree bit for bit: trajectories,
densities, action derivatives and estimator blocks.
"""
import numpy as np
import pytest

from simpimc_gb300.configs import electron_gas


@pytest.mark.parametrize("pair", ["BarePairAction", "IlkkaPairAction"])
def test_lean_densities_are_bit_identical(tmp_path, oracle_mod, pair):
    xml, path = electron_gas(tmp_path, n_part=14, n_bead=16, n_level=2, rs=2.0, k_cut_units=4.0, seed=3, pair=pair,
                             structure_factor=True)
    path = path + 0.3 * np.random.default_rng(1).standard_normal(path.shape)
    res = []
    for lean in (False, True):
        o = oracle_mod.OracleSim(xml, base_dir=tmp_path, lean_densities=lean)
        o.set_path(path)
        for _ in range(25):
            o.move_attempts(0, 7)
            o.move_attempts(1, 7)
        grads = [o.get_action_gradient(a, 3, 4, [(0, 2)], 0, 0) for a in range(o.n_actions)]
        vals = [o.get_action(a, 2, 10, [(1, 3)], 0, 1) for a in range(o.n_actions)]
        d = [o.dactiondbeta(a) for a in range(o.n_actions)]
        blocks = []
        for obs in range(o.n_observables):
            o.observable_accumulate(obs)
            blocks.append(np.asarray(o.observable_block(obs)))
        res.append(dict(path=o.get_path(1), rho0=o.rho_k(0), rho1=o.rho_k(1), grads=grads, vals=vals, d=d, blocks=blocks,
                        stats=[o.move_stats(m) for m in range(2)]))
        o.close()
    a, b = res
    assert a["stats"] == b["stats"]
    for key in ("path", "rho0", "rho1"):
        assert np.array_equal(a[key], b[key]), key
    assert a["d"] == b["d"] and a["vals"] == b["vals"]
    for ga, gb in zip(a["grads"], b["grads"]):
        assert np.array_equal(ga, gb)
    for x, y in zip(a["blocks"], b["blocks"]):
        assert np.array_equal(x, y)
