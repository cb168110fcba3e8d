"""CPU tests that pin the oracle (the FP64 restatement of the reference hot path) to known answers.

The reference ships no unit tests, fixtures or golden vectors for this path, so the oracle is pinned
through answers that do not depend on it:
  * Philox4x32-10 known-answer vectors (Random123 KAT) for the move's random stream;
  * the exact energy of the discretised harmonic oscillator (the reference's inputs/sho case and
    the trapped-particle configuration with the Coulomb term off) against the oracle's Monte Carlo
    thermal estimator;
  * an independent brute-force Ewald sum for the Coulomb pair action's potential;
  * the free-particle image sum behind the kinetic action's spline;
  * bit identity of the exactly specified binary32 random transforms between the oracle and the
    product header compiled for the host.
"""
import math
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from exact_energies import blocked_error, exact_sho_energy
from simpimc_gb300.configs import electron_gas, trapped_coulomb
from simpimc_gb300.tables import coulomb_table, lattice_k_magnitudes


def test_philox_kat():
    # Random123 kat_vectors for philox4x32 (10 rounds).
    cases = [
        ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
        ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
        ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
         (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
    ]
    for ctr, key, want in cases:
        assert tuple(int(x) for x in oracle.philox(ctr, key)) == want


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs a host C++ compiler")
def test_random_transforms_bit_identical(tmp_path):
    exe = tmp_path / "draws"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "tests/host/draws_main.cc", "-o", str(exe)], check=True)
    for seed, chain, move, attempt, n_level in [(1, 0, 0, 0, 3), (20261203, 7, 1, 123456789, 4), (99, 2, 3, 2**40 + 5, 5)]:
        out = subprocess.run([str(exe), str(seed), str(chain), str(move), str(attempt), "66", "128", str(n_level)],
                             check=True, capture_output=True, text=True).stdout.split("\n")
        pb, z, lu = oracle.bisect_draws(seed, chain, move, attempt, 66, 128, n_level)
        assert [int(x) for x in out[0].split()] == [int(pb[0]), int(pb[1])]
        zb = z.view(np.uint32)
        for i in range((1 << n_level) - 1):
            assert [int(x, 16) for x in out[1 + i].split()] == [int(v) for v in zb[i]]
        lb = lu.view(np.uint32)
        for li in range(n_level):
            assert int(out[1 + (1 << n_level) - 1 + li], 16) == int(lb[li])


def test_normals_statistics():
    zs = np.concatenate([oracle.bisect_draws(5, 0, 0, a, 8, 32, 5)[1].ravel() for a in range(400)])
    assert abs(zs.mean()) < 0.02 and abs(zs.std() - 1.0) < 0.02
    assert abs(np.mean(zs ** 4) - 3.0) < 0.15


def run_energy_series(o, n_sweeps, attempts_per_sweep, n_warm):
    o.move_attempts(0, n_warm * attempts_per_sweep)
    o.observable_block(0)
    vals = []
    for _ in range(n_sweeps):
        o.move_attempts(0, attempts_per_sweep)
        o.observable_accumulate(0)
        vals.append(o.observable_block(0)[0])
    return np.array(vals)


def test_sho_reference_case_exact_energy():
    # The reference's inputs/sho case (1-D, beta = 10, M = 32, omega = 1, bisection level 2).
    xml = """<Input><RNG seed="3"/><System n_d="1" n_bead="32" beta="10.0" pbc="0"/>
      <Particles><Species name="e" n_part="1" lambda="0.5" init_type="Random"/></Particles>
      <Actions><Action name="Kinetic" type="Kinetic" n_images="0" species="e"/>
        <Action name="HarmonicTrap" type="HarmonicTrap" species="e" omega="1." max_level="0"/></Actions>
      <Moves><Move name="BisectE" type="Bisect" species="e" n_level="2"/></Moves>
      <Observables><Observable name="Energy" type="Energy"/></Observables><Algorithm/></Input>"""
    o = oracle.OracleSim(xml)
    o.set_path(np.zeros((1, 32, 1)))
    e = run_energy_series(o, 40000, 8, 200)
    exact = exact_sho_energy(10.0, 32, 1.0)
    err = blocked_error(e)
    assert abs(e.mean() - exact) < 4 * err, (e.mean(), exact, err)
    assert abs(exact - 0.5 / math.tanh(5.0)) < 0.01  # Trotter error of the discretisation


def test_trap_without_coulomb_exact_energy(tmp_path):
    # The 8-particle trapped configuration with the Coulomb term off: 3N independent oscillators.
    xml, path = trapped_coulomb(tmp_path, n_part=8, n_bead=32, beta=2.0, n_level=3, seed=11, coulomb=False)
    o = oracle.OracleSim(xml, base_dir=tmp_path)
    o.set_path(path)
    e = run_energy_series(o, 3000, 32, 100)
    exact = 24 * exact_sho_energy(2.0, 32, 1.0)
    err = blocked_error(e)
    assert abs(e.mean() - exact) < 4 * err, (e.mean(), exact, err)
    assert abs(24 * 0.5 / math.tanh(1.0) - 15.7565) < 1e-3


def brute_force_ewald(pos, L, alpha=None, nmax_r=2, nmax_k=12):
    """Coulomb energy of unit charges in a periodic cube with a neutralising background (standard
    Ewald with its own splitting parameter and generous cut-offs, independent of the tables)."""
    N = len(pos)
    V = L ** 3
    alpha = 6.0 / L if alpha is None else alpha
    from math import erfc
    e_real = 0.0
    rng = range(-nmax_r, nmax_r + 1)
    for i in range(N):
        for j in range(N):
            for nx in rng:
                for ny in rng:
                    for nz in rng:
                        if i == j and nx == ny == nz == 0:
                            continue
                        d = pos[i] - pos[j] + L * np.array([nx, ny, nz])
                        r = np.linalg.norm(d)
                        e_real += 0.5 * erfc(alpha * r) / r
    ks = 2 * np.pi / L * np.array([(a, b, c) for a in range(-nmax_k, nmax_k + 1) for b in range(-nmax_k, nmax_k + 1)
                                   for c in range(-nmax_k, nmax_k + 1) if (a, b, c) != (0, 0, 0)])
    k2 = np.sum(ks ** 2, axis=1)
    sk = np.exp(1j * pos @ ks.T).sum(axis=0)
    e_k = 2 * np.pi / V * np.sum(np.exp(-k2 / (4 * alpha ** 2)) / k2 * np.abs(sk) ** 2)
    return e_real + e_k - alpha / math.sqrt(math.pi) * N - math.pi * N ** 2 / (2 * V * alpha ** 2)


def test_ewald_potential_matches_brute_force(tmp_path):
    # Classical configuration (all beads of a particle at one point): Potential()/M of the three
    # Coulomb actions is the periodic Coulomb energy of the 14 electrons.
    xml, path = electron_gas(tmp_path, n_part=14, n_bead=4, n_level=1, rs=2.0, k_cut_units=8.0, seed=2)
    o = oracle.OracleSim(xml, base_dir=tmp_path)
    o.set_path(path)
    L = (4 * math.pi * 14 / 3) ** (1 / 3) * 2.0
    v = sum(o.potential(a) for a in (2, 3, 4)) / 4
    exact = brute_force_ewald(path[:, 0, :], L)
    assert abs(v - exact) < 2e-6 * abs(exact), (v, exact)


def test_kinetic_image_spline_known_answer(tmp_path):
    # Periodic box smaller than the thermal wavelength, so images matter: the kinetic action of a
    # link equals -log of the image sum of the free propagator (free_spline_class.h:40-63).
    L, lam, beta, M = 2.0, 0.5, 4.0, 4
    tau = beta / M
    xml = f"""<Input><RNG seed="1"/><System n_d="3" n_bead="{M}" beta="{beta}" L="{L}" pbc="1"/>
      <Particles><Species name="e" n_part="1" lambda="{lam}" init_type="Random"/></Particles>
      <Actions><Action name="Kinetic" type="Kinetic" n_images="4" species="e"/></Actions>
      <Moves/><Observables/><Algorithm/></Input>"""
    o = oracle.OracleSim(xml)
    rng = np.random.default_rng(4)
    path = rng.uniform(-L / 2, L / 2, size=(1, M, 3))
    o.set_path(path)
    got = o.get_action(0, 0, 1, [(0, 0)], 0, 1)
    dr = path[0, 0] - path[0, 1]
    dr -= L * np.rint(dr / L)
    want = 0.0
    for x in dr:
        s = sum(math.exp(-((x + n * L) ** 2 - x ** 2) / (4 * lam * tau)) for n in range(-4, 5))
        want += x * x / (4 * lam * tau) - math.log(s)
    assert abs(got - want) < 1e-7, (got, want)


def test_kspace_size_of_electron_gas(tmp_path):
    # |k| < 12 (2 pi / L) in the 66-electron box: 3561 stored half-space vectors (7122 with -k).
    xml, _ = electron_gas(tmp_path, n_part=66, n_bead=4, n_level=1, rs=2.0, k_cut_units=12.0)
    o = oracle.OracleSim(xml, base_dir=tmp_path)
    assert o.n_k == 3561
    ks = o.kvecs()
    mags = np.linalg.norm(ks, axis=1)
    L = (4 * math.pi * 66 / 3) ** (1 / 3) * 2.0
    assert np.all(mags < 12 * 2 * math.pi / L)
    table = lattice_k_magnitudes(L, 12 * 2 * math.pi / L)
    assert np.all(np.min(np.abs(mags[:, None] - table[None, :]), axis=1) < 1e-9)


def test_oracle_rejects_bad_input(tmp_path):
    with pytest.raises(RuntimeError, match="XML parse error"):
        oracle.OracleSim("<Input><System n_d='3'></Input>")
    with pytest.raises(RuntimeError, match="missing required attribute"):
        oracle.OracleSim("<Input><System n_d='3' n_bead='4'/><Particles/></Input>")
    xml = """<Input><System n_d="3" n_bead="4" beta="1" L="5" pbc="1"/>
      <Particles><Species name="e" n_part="2" lambda="0.5"/></Particles>
      <Actions><Action name="C" type="BarePairAction" file="missing.pat" species_a="e" species_b="e"/></Actions></Input>"""
    with pytest.raises(RuntimeError, match="cannot open pair-action table"):
        oracle.OracleSim(xml, base_dir=tmp_path)


def test_table_round_trip(tmp_path):
    ds = coulomb_table(tmp_path / "t.pat", L=10.0, k_cut=3.0)
    text = (tmp_path / "t.pat").read_text().split()
    i = text.index("v/diag/v_long_k_0")
    assert float(text[i + 2]) == ds["v/diag/v_long_k_0"]


def _fd_check(o, path, coords, h=1e-5):
    g = o.action_gradient_path()
    out = []
    for i in coords:
        pp = path.copy()
        pp[i] += h
        o.set_path(pp)
        sp = o.total_action()
        pp[i] -= 2 * h
        o.set_path(pp)
        sm = o.total_action()
        out.append((g[i], (sp - sm) / (2 * h)))
    o.set_path(path)
    return out


def test_oracle_exact_gradient_matches_central_differences(oracle_mod, tmp_path):
    """The oracle's analytic dS/dR (kinetic, trap, pair, Ewald) against central differences of
    its whole-ring action, h = 1e-5: agreement within the O(h^2) truncation."""
    from simpimc_gb300.configs import electron_gas, trapped_coulomb
    rng = np.random.default_rng(11)
    xml, path = trapped_coulomb(tmp_path, n_part=4, n_bead=8, n_level=2, seed=3)
    o = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    o.set_path(path)
    coords = [tuple(int(x) for x in (rng.integers(4), rng.integers(8), rng.integers(3))) for _ in range(6)]
    for g, fd in _fd_check(o, path, coords):
        assert abs(g - fd) <= 1e-6 * max(1.0, abs(g)), (g, fd)
    xml, path = electron_gas(tmp_path, n_part=8, n_bead=8, n_level=2, rs=2.0, k_cut_units=3.0, seed=5)
    L = (4 * np.pi * 8 / 3) ** (1 / 3) * 2.0
    path = rng.uniform(-L / 2, L / 2, size=path.shape)
    o = oracle_mod.OracleSim(xml, base_dir=tmp_path)
    o.set_path(path)
    coords = [tuple(int(x) for x in (rng.integers(8), rng.integers(8), rng.integers(3))) for _ in range(6)]
    for g, fd in _fd_check(o, path, coords):
        assert abs(g - fd) <= 1e-6 * max(1.0, abs(g)), (g, fd)


def test_oracle_hmc_energy_error_shrinks_with_step(oracle_mod, tmp_path):
    """Leapfrog is second order: the mean |dH| of an HMC trajectory of fixed length falls by ~4x
    when the step halves, so acceptance approaches 1."""
    from simpimc_gb300.configs import trapped_coulomb
    xml, path = trapped_coulomb(tmp_path, n_part=3, n_bead=8, n_level=2, seed=9)
    rates = []
    for step, n in ((0.02, 10), (0.01, 20)):
        x = xml.replace('<Move name="Bisect" type="Bisect" species="e" n_level="2" />',
                        f'<Move name="HMC" type="HMC" step_size="{step}" n_steps="{n}" />')
        o = oracle_mod.OracleSim(x, base_dir=tmp_path)
        o.set_path(path)
        o.move_attempts(0, 40)
        rates.append(o.move_stats(0)[2] / 40)
    assert rates[1] >= rates[0] and rates[1] > 0.5, rates
