"""New device buffers are ready before the context's non-blocking stream uses them.

A context allocates some scratch buffers on first use (the attempt schedule of a concurrent sweep,
particle and pair lists, partial sums) and zero-fills them. The fill runs on the legacy default
stream; the context's stream is non-blocking, so the fill must complete before the buffer is handed
out, or a copy enqueued right after the allocation can be overwritten by it. This test keeps the
legacy default stream busy (PyTorch's default stream) while a fresh context runs its first
concurrent sweep and several action evaluations, then replays the oracle: identical accept counts,
positions and densities within 1e-9, action values within 1e-10 relative.
"""
import numpy as np
import pytest

from simpimc_gb300 import Simulation
from simpimc_gb300.configs import electron_gas

pytestmark = pytest.mark.gpu


def test_first_use_buffers_survive_busy_default_stream(tmp_path, gpu_lib, oracle_mod):
    torch = pytest.importorskip("torch")
    x = torch.ones(32 * 1024 * 1024, device="cuda")
    for rep in range(3):
        xml, path = electron_gas(tmp_path, n_part=14, n_bead=64, n_level=3, rs=2.0, k_cut_units=4.0, seed=41 + rep)
        g = Simulation(xml, base_dir=tmp_path)
        c = oracle_mod.OracleSim(xml, base_dir=tmp_path)
        g.set_sweep_wave(2)
        g.set_path(path)
        c.set_path(path)
        for _ in range(40):  # tens of ms of work queued on the default stream
            x.mul_(1.0000001)
        g.sweep([0, 1], [7, 7], n_rep=12)
        for _ in range(12):
            c.move_attempts(0, 7)
            c.move_attempts(1, 7)
        for m in range(2):
            assert g.move_stats(m) == c.move_stats(m), (rep, m, g.move_stats(m), c.move_stats(m))
        assert np.max(np.abs(g.get_path(1) - c.get_path(1))) < 1e-9
        for s in range(2):
            assert np.max(np.abs(g.rho_k(s) - c.rho_k(s))) < 1e-9
        for _ in range(40):
            x.mul_(1.0000001)
        for a in range(g.n_actions):
            gv, cv = g.get_action(a, 5, 13, [(0, 3), (1, 2)], 0, 1), c.get_action(a, 5, 13, [(0, 3), (1, 2)], 0, 1)
            assert abs(gv - cv) <= 1e-10 * max(1.0, abs(cv)), (rep, a, gv, cv)
        g.close()
        c.close()
    torch.cuda.synchronize()
