"""Whole runs on the GPU against exactly known energies, gated at two standard errors.

* 64 batched chains of 8 trapped particles without Coulomb (24 independent oscillators each,
  beta = 2, M = 32), advanced by bisection sweeps and the whole-path HMC move in FP32: the mean
  thermal energy over the chains against 24 x the exact energy of the discretised action.
* 4 free particles in a periodic box of side L = 3 (beta = 2, lambda = 1/2, M = 16, kinetic
  images), single-chain sweep kernel: the thermal energy against 3 N <lambda k^2> over the
  box's k lattice, 0.0533 per degree of freedom here against the classical 0.25.

The standard errors come from independent chains (first case) and from blocks of 200
measurements (second); seeds are fixed, so each check is one deterministic run.
"""
import math

import numpy as np
import pytest

from exact_energies import blocked_error, exact_sho_energy, free_particle_energy_1d
from simpimc_gb300 import ChainBatch, Simulation
from simpimc_gb300.configs import trapped_coulomb

pytestmark = pytest.mark.gpu


def test_batched_trap_energy_matches_exact_oscillators(tmp_path, gpu_lib):
    n_chains, n, m, beta = 64, 8, 32, 2.0
    items = [trapped_coulomb(tmp_path, n_part=n, n_bead=m, n_level=3, beta=beta, seed=7000 + c, coulomb=False, hmc=(0.03, 10),
                             write_table=(c == 0)) for c in range(n_chains)]
    b = ChainBatch([x for x, _ in items], base_dir=tmp_path)
    for c, (_, p) in enumerate(items):
        b.set_path(c, p)
    b.set_hmc_per_cycle(1)
    b.run(300, 1)  # equilibration
    b.reset_energy()
    b.run(1500, 1)
    means = np.array([b.energy(c, cap=1500)[0][:, 0].mean() for c in range(n_chains)])
    hatt, hacc = b.hmc_counters()
    b.close()
    exact = 3 * n * exact_sho_energy(beta, m, 1.0)
    err = means.std(ddof=1) / math.sqrt(n_chains)
    assert 0 < int(hacc.sum()) < int(hatt.sum())  # HMC moved the chains
    assert abs(means.mean() - exact) < 2 * err, (means.mean(), exact, err)
    assert err < 0.01 * exact  # the gate resolves the energy to 1 %


def _free_box_xml(n_part, n_bead, beta, L, n_level, n_images, seed):
    return f"""<Input>
  <RNG seed="{seed}" />
  <IO output_prefix="free" />
  <Parallel procs_per_group="1" />
  <System n_d="3" n_bead="{n_bead}" beta="{beta}" L="{L!r}" pbc="1" k_cut="0" />
  <Particles>
    <Species name="e" n_part="{n_part}" lambda="0.5" fermi="0" init_type="File" file_name="init.xyz" all_beads="1" />
  </Particles>
  <Actions>
    <Action name="Kinetic" type="Kinetic" n_images="{n_images}" species="e" />
  </Actions>
  <Moves>
    <Move name="BisectE" type="Bisect" species="e" n_level="{n_level}" n_images="{n_images}" />
  </Moves>
  <Observables>
    <Observable name="Energy" type="Energy" />
  </Observables>
  <Algorithm />
</Input>
"""


def test_free_particles_in_a_box_match_the_lattice_sum(tmp_path, gpu_lib):
    n, m, beta, L, lvl = 4, 16, 2.0, 3.0, 3
    xml = _free_box_xml(n, m, beta, L, lvl, 2, seed=8101)
    rng = np.random.default_rng(8101)
    path = np.repeat(rng.uniform(-L / 2, L / 2, size=(n, 1, 3)), m, axis=1)
    (tmp_path / "init.xyz").write_text("")
    s = Simulation(xml, base_dir=tmp_path)
    s.set_path(path)
    per_sweep = n * (m // (1 << lvl))
    s.sweep([0], [per_sweep], 500)  # equilibration
    s.observable_block(0)
    vals = []
    for _ in range(8000):
        s.sweep([0], [per_sweep], 1)
        s.observable_accumulate(0)
        vals.append(s.observable_block(0)[0])
    s.close()
    vals = np.asarray(vals)
    exact = 3 * n * free_particle_energy_1d(beta, L)
    err = blocked_error(vals, n_blocks=40)
    assert abs(vals.mean() - exact) < 2 * err, (vals.mean(), exact, err)
    classical = 3 * n / (2 * beta)
    assert abs(vals.mean() - classical) > 10 * err  # the box's quantisation is resolved


def test_free_particles_replay_the_oracle(tmp_path, gpu_lib, oracle_mod):
    """Attempts without a grid phase (no pair action) on the single-chain sweep kernel: every block
    runs them and commits the same beads, after a grid barrier that keeps a fast block's commit from
    a slow block's reads. The oracle's accept count and path, on the same draws."""
    n, m, beta, L, lvl = 4, 16, 2.0, 3.0, 3
    xml = _free_box_xml(n, m, beta, L, lvl, 2, seed=8102)
    rng = np.random.default_rng(8102)
    path = np.repeat(rng.uniform(-L / 2, L / 2, size=(n, 1, 3)), m, axis=1)
    (tmp_path / "init.xyz").write_text("")
    s = Simulation(xml, base_dir=tmp_path)
    o = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    s.set_path(path)
    o.set_path(path)
    per_sweep = n * (m // (1 << lvl))
    s.sweep([0], [per_sweep], 300)
    o.move_attempts(0, 300 * per_sweep)
    assert s.move_counters(0)[3] == o.move_stats(0)[2], (s.move_counters(0), o.move_stats(0))
    assert np.max(np.abs(s.get_path(1) - o.get_path())) < 1e-9
    s.close()
    o.close()
