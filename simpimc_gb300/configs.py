"""XML inputs, pair-action tables and seeded initial paths for the benchmark systems.

Each builder returns ``(xml_text, initial_path)``; tables are written into ``workdir``. The
systems follow the reference's input format (inputs/*.xml): <System>, <Particles>, <Actions>,
<Moves>, <Observables>, <Algorithm>.

* ``trapped_coulomb``: N distinguishable unit-mass particles in an isotropic 3-D harmonic trap
  with bare Coulomb repulsion (primitive action tau*V), open boundaries; beads i.i.d. N(0, 1).
* ``electron_gas``: N Boltzmannon electrons (half up, half down) in a periodic cube at density
  r_s, Coulomb split into a short-range primitive part and an Ewald long-range k-sum; beads
  uniform in the box.

* ``trapped_bosons``: N bosons (or sign-weighted fermions) in the same trap, with a permuting
  bisection (PermBisectIterative or PermBisectTable) beside the plain one; optional Coulomb.

The first two take ``pair="IlkkaPairAction"`` or ``pair="DavidPairAction"`` (with ``n_order``) to use the
off-diagonal pair action of a synthetic ``tables.ilkka_table`` / ``tables.david_table`` instead of
the primitive BarePairAction.
"""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np

from .tables import coulomb_table, david_table, ilkka_table


def _open_pair_xml(workdir, species, pair, n_bead, beta, n_order, pair_max_level, write_table):
    """The Coulomb pair action of an open-boundary species (its table written into `workdir`)."""
    if pair == "DavidPairAction":
        tab = workdir / f"david_open_{n_bead}_{beta}_{n_order}_{pair_max_level}.pat"
        if write_table or not tab.exists():
            david_table(tab, tau=beta / n_bead, n_order=n_order, lam=0.5, z_ab=1.0, L=0.0, n_tau=pair_max_level + 1)
        return (f'<Action name="Coulomb" type="DavidPairAction" file="{tab.name}" n_order="{n_order}" species_a="{species}" '
                f'species_b="{species}" max_level="{pair_max_level}" use_long_range="0" />')
    if pair == "IlkkaPairAction":
        tab = workdir / f"ilkka_open_{n_bead}_{beta}.pat"
        if write_table or not tab.exists():
            ilkka_table(tab, tau=beta / n_bead, lam=0.5, z_ab=1.0, L=0.0)
        return (f'<Action name="Coulomb" type="IlkkaPairAction" file="{tab.name}" species_a="{species}" species_b="{species}" '
                f'max_level="{pair_max_level}" use_long_range="0" />')
    tab = workdir / "coulomb_open.pat"
    if write_table or not tab.exists():
        coulomb_table(tab, z_ab=1.0, L=0.0)
    return (f'<Action name="Coulomb" type="BarePairAction" file="{tab.name}" is_coulomb="1" species_a="{species}" '
            f'species_b="{species}" max_level="{pair_max_level}" use_long_range="0" />')


def trapped_coulomb(workdir, *, n_part=8, beta=2.0, n_bead=32, omega=1.0, n_level=3, seed=1234, coulomb=True,
                    n_step_inner=100, n_step_outer=10, gr_bins=200, gr_rmax=5.0, virial=False, path_seed=None,
                    write_table=True, pair="BarePairAction", n_order=2, pair_max_level=0, adaptive=False, target_ratio=0.5,
                    hmc=None, trap_max_level=0, path_dump=0):
    workdir = Path(workdir)
    workdir.mkdir(parents=True, exist_ok=True)
    pair_xml = _open_pair_xml(workdir, "e", pair, n_bead, beta, n_order, pair_max_level, write_table)
    pair = pair_xml if coulomb else ""
    energy = ('<Observable name="Energy" type="Energy" use_virial_estimator="1" />' if virial
              else '<Observable name="Energy" type="Energy" />')
    adapt = f' adaptive="1" target_ratio="{target_ratio!r}"' if adaptive else ""
    # path_dump = skip: a PathDump observable (every skip-th Write dumps the path) after the others
    dump_xml = f'\n    <Observable name="path_dump" type="PathDump" skip="{path_dump}" />' if path_dump else ""
    # hmc = (step_size, n_steps): the library's whole-path hybrid Monte Carlo move besides Bisect
    hmc_xml = (f'\n    <Move name="HMC" type="HMC" species="e" step_size="{hmc[0]!r}" n_steps="{int(hmc[1])}" />' if hmc else "")
    xml = f"""<Input>
  <RNG seed="{seed}" />
  <IO output_prefix="trap" />
  <Parallel procs_per_group="1" />
  <System n_d="3" n_bead="{n_bead}" beta="{beta}" pbc="0" />
  <Particles>
    <Species name="e" n_part="{n_part}" lambda="0.5" fermi="0" init_type="File" file_name="init.xyz" all_beads="1" />
  </Particles>
  <Actions>
    <Action name="Kinetic" type="Kinetic" n_images="0" species="e" />
    <Action name="Trap" type="HarmonicTrap" species="e" omega="{omega}" max_level="{trap_max_level}" />
    {pair}
  </Actions>
  <Moves>
    <Move name="Bisect" type="Bisect" species="e" n_level="{n_level}"{adapt} />{hmc_xml}
  </Moves>
  <Observables>
    {energy}
    <Observable name="gr" type="PairCorrelation" species_a="e" species_b="e" r_min="0." r_max="{gr_rmax}" n_r="{gr_bins}" />{dump_xml}
  </Observables>
  <Algorithm>
    <Loop n_step="{n_step_outer}">
      <Loop n_step="{n_step_inner}">
        <Move name="Bisect" />
        <Observable name="Energy" />
        <Observable name="gr" />
      </Loop>
      <Write />
    </Loop>
  </Algorithm>
</Input>
"""
    rng = np.random.default_rng(seed if path_seed is None else path_seed)
    path = rng.standard_normal((n_part, n_bead, 3))
    return xml, path


def electron_gas(workdir, *, n_part=66, rs=2.0, beta=8.0, n_bead=128, k_cut_units=12.0, n_level=4, seed=4321,
                 n_step_inner=10, n_step_outer=4, path_seed=None, structure_factor=False, pair="BarePairAction", n_order=2,
                 pair_max_level=0, n_images=0, perm=None, measure_all=False, virial=False):
    """Two-spin electron gas in a periodic box with Ewald sums; `perm` (PermBisectIterative or
    PermBisectTable over every up particle) adds a permuting move of the up spins; `measure_all`
    accumulates g(r) (and S(k)) in the Algorithm besides the energy; `virial` measures the energy
    with the virial estimator."""
    workdir = Path(workdir)
    workdir.mkdir(parents=True, exist_ok=True)
    L = (4.0 * math.pi * n_part / 3.0) ** (1.0 / 3.0) * rs
    k_cut = k_cut_units * 2.0 * math.pi / L
    if pair == "DavidPairAction":
        tab = workdir / f"david_ewald_{n_part}_{rs}_{n_bead}_{beta}_{n_order}.pat"
        david_table(tab, tau=beta / n_bead, n_order=n_order, lam=0.5, z_ab=1.0, L=L, k_cut=k_cut, n_tau=pair_max_level + 1)
        extra = f' n_order="{n_order}"'
    elif pair == "IlkkaPairAction":
        tab = workdir / f"ilkka_ewald_{n_part}_{rs}_{n_bead}_{beta}.pat"
        ilkka_table(tab, tau=beta / n_bead, lam=0.5, z_ab=1.0, L=L, k_cut=k_cut)
        extra = ""
    else:
        tab = workdir / f"coulomb_ewald_{n_part}_{rs}.pat"
        coulomb_table(tab, z_ab=1.0, L=L, k_cut=k_cut)
        extra = ' is_coulomb="1"'

    n_up = n_part // 2
    n_dn = n_part - n_up
    img = f' n_images="{n_images}"' if n_images else ""
    sk = ('<Observable name="sk" type="StructureFactor" species_a="eU" species_b="eU" />' if structure_factor else "")
    perm_move = perm_event = more_events = ""
    energy_opt = ' use_virial_estimator="1"' if virial else ""
    if measure_all:
        more_events = '\n        <Observable name="gr" />' + ('\n        <Observable name="sk" />' if structure_factor else "")
    if perm:
        table = f' n_perm_part="{n_up}"' if perm == "PermBisectTable" else ""
        perm_move = f'\n    <Move name="PermU" type="{perm}" species="eU" n_level="{n_level}"{table}{img} />'
        perm_event = '\n        <Move name="PermU" />'
    xml = f"""<Input>
  <RNG seed="{seed}" />
  <IO output_prefix="egas" />
  <Parallel procs_per_group="1" />
  <System n_d="3" n_bead="{n_bead}" beta="{beta}" L="{L!r}" pbc="1" k_cut="{k_cut!r}" />
  <Particles>
    <Species name="eU" n_part="{n_up}" lambda="0.5" fermi="0" init_type="File" file_name="init.xyz" all_beads="1" />
    <Species name="eD" n_part="{n_dn}" lambda="0.5" fermi="0" init_type="File" file_name="init.xyz" all_beads="1" />
  </Particles>
  <Actions>
    <Action name="KineticU" type="Kinetic" n_images="{n_images}" species="eU" />
    <Action name="KineticD" type="Kinetic" n_images="{n_images}" species="eD" />
    <Action name="CoulombUU" type="{pair}" file="{tab.name}"{extra} species_a="eU" species_b="eU" max_level="{pair_max_level}" use_long_range="1" />
    <Action name="CoulombDD" type="{pair}" file="{tab.name}"{extra} species_a="eD" species_b="eD" max_level="{pair_max_level}" use_long_range="1" />
    <Action name="CoulombUD" type="{pair}" file="{tab.name}"{extra} species_a="eU" species_b="eD" max_level="{pair_max_level}" use_long_range="1" />
  </Actions>
  <Moves>
    <Move name="BisectU" type="Bisect" species="eU" n_level="{n_level}"{img} />
    <Move name="BisectD" type="Bisect" species="eD" n_level="{n_level}"{img} />{perm_move}
  </Moves>
  <Observables>
    <Observable name="Energy" type="Energy"{energy_opt} />
    <Observable name="gr" type="PairCorrelation" species_a="eU" species_b="eD" n_r="100" />
    {sk}
  </Observables>
  <Algorithm>
    <Loop n_step="{n_step_outer}">
      <Loop n_step="{n_step_inner}">
        <Move name="BisectU" />
        <Move name="BisectD" />{perm_event}
        <Observable name="Energy" />{more_events}
      </Loop>
      <Write />
    </Loop>
  </Algorithm>
</Input>
"""
    # Classical start as the reference's init_type="Random" (species_class.h:262-272): one uniform
    # point in the box per particle, shared by all of its beads.
    rng = np.random.default_rng(seed if path_seed is None else path_seed)
    path = np.repeat(rng.uniform(-L / 2, L / 2, size=(n_part, 1, 3)), n_bead, axis=1)
    return xml, path


def two_species_trap(workdir, *, n_a=3, n_b=3, lambda_a=0.5, lambda_b=0.25, z_ab=0.5, beta=2.0, n_bead=32, omega=1.0, n_level=3,
                     seed=1234, n_step_inner=40, n_step_outer=3):
    """Two distinguishable species of different masses (lambda = hbar^2 / 2m) in one harmonic trap, with
    bare Coulomb actions within and between them (charge product z_ab across species) and a Bisect
    move per species."""
    workdir = Path(workdir)
    workdir.mkdir(parents=True, exist_ok=True)
    coulomb_table(workdir / "coulomb_open.pat", z_ab=1.0, L=0.0)
    coulomb_table(workdir / "coulomb_open_ab.pat", z_ab=z_ab, L=0.0)
    xml = f"""<Input>
  <RNG seed="{seed}" />
  <IO output_prefix="trap2" />
  <Parallel procs_per_group="1" />
  <System n_d="3" n_bead="{n_bead}" beta="{beta}" pbc="0" />
  <Particles>
    <Species name="a" n_part="{n_a}" lambda="{lambda_a!r}" fermi="0" init_type="File" file_name="init.xyz" all_beads="1" />
    <Species name="b" n_part="{n_b}" lambda="{lambda_b!r}" fermi="0" init_type="File" file_name="init.xyz" all_beads="1" />
  </Particles>
  <Actions>
    <Action name="KineticA" type="Kinetic" n_images="0" species="a" />
    <Action name="KineticB" type="Kinetic" n_images="0" species="b" />
    <Action name="TrapA" type="HarmonicTrap" species="a" omega="{omega}" max_level="0" />
    <Action name="TrapB" type="HarmonicTrap" species="b" omega="{omega}" max_level="0" />
    <Action name="CoulombAA" type="BarePairAction" file="coulomb_open.pat" is_coulomb="1" species_a="a" species_b="a" max_level="0" use_long_range="0" />
    <Action name="CoulombBB" type="BarePairAction" file="coulomb_open.pat" is_coulomb="1" species_a="b" species_b="b" max_level="0" use_long_range="0" />
    <Action name="CoulombAB" type="BarePairAction" file="coulomb_open_ab.pat" is_coulomb="0" species_a="a" species_b="b" max_level="0" use_long_range="0" />
  </Actions>
  <Moves>
    <Move name="BisectA" type="Bisect" species="a" n_level="{n_level}" />
    <Move name="BisectB" type="Bisect" species="b" n_level="{n_level}" />
  </Moves>
  <Observables>
    <Observable name="Energy" type="Energy" />
    <Observable name="gr" type="PairCorrelation" species_a="a" species_b="b" r_min="0." r_max="5.0" n_r="100" />
  </Observables>
  <Algorithm>
    <Loop n_step="{n_step_outer}">
      <Loop n_step="{n_step_inner}">
        <Move name="BisectA" />
        <Move name="BisectB" />
        <Observable name="Energy" />
        <Observable name="gr" />
      </Loop>
      <Write />
    </Loop>
  </Algorithm>
</Input>
"""
    rng = np.random.default_rng(seed)
    path = rng.standard_normal((n_a + n_b, n_bead, 3))
    return xml, path


def batched_trap_chains(workdir, *, n_chains=256, seed0=1000, n_range=(16, 128), bead_choices=(32, 64, 128),
                        n_level=3, beta=2.0, omega=1.0, chain_seed0=None, hmc=None):
    """Independent trapped Coulomb chains with uneven sizes: chain c has seed ``chain_seed0 + c``
    (``chain_seed0`` defaults to ``seed0``), N drawn uniformly from ``n_range`` (inclusive) and M
    from ``bead_choices`` by a generator seeded with ``seed0``; beads i.i.d. N(0, 1) from the
    chain's seed; ``hmc = (step_size, n_steps)`` adds the HMC move to every chain. Returns a list of
    ``(xml_text, initial_path)``."""
    cs0 = seed0 if chain_seed0 is None else chain_seed0
    rng = np.random.default_rng(seed0)
    ns = rng.integers(n_range[0], n_range[1] + 1, size=n_chains)
    ms = rng.choice(np.asarray(bead_choices), size=n_chains)
    out = []
    for c in range(n_chains):
        out.append(trapped_coulomb(workdir, n_part=int(ns[c]), n_bead=int(ms[c]), n_level=n_level, beta=beta,
                                   omega=omega, seed=cs0 + c, write_table=(c == 0), hmc=hmc))
    return out


def sweep_schedule(sim_or_counts, n_bisect_beads: int, n_bead: int):
    """One sweep: N_s * ceil(M / 2^l) attempts of each species' bisection move, in move order."""
    counts = [n * math.ceil(n_bead / n_bisect_beads) for n in sim_or_counts]
    return list(range(len(counts))), counts


def trapped_bosons(workdir, *, n_part=3, beta=2.0, n_bead=16, omega=1.0, n_level=2, seed=1234, coulomb=False,
                   perm="PermBisectIterative", n_perm_part=2, fermi=False, n_step_inner=100, n_step_outer=10,
                   path_seed=None, perm_level=None, sector_max=0, pair="BarePairAction", n_order=2, pair_max_level=0, path_dump=0):
    """Identical particles with exchange: the permuting move's species carries the path
    permutation. Observables: Energy (thermal), Permutation (cycle histogram and sectors), Sign.
    With coulomb, `pair` chooses the Coulomb pair action as in trapped_coulomb."""
    workdir = Path(workdir)
    workdir.mkdir(parents=True, exist_ok=True)
    pair_xml = _open_pair_xml(workdir, "b", pair, n_bead, beta, n_order, pair_max_level, True) if coulomb else ""
    extra = f' n_perm_part="{n_perm_part}"' if perm == "PermBisectTable" else ""
    perm_level = n_level if perm_level is None else perm_level
    dump_xml = f'\n    <Observable name="path_dump" type="PathDump" skip="{path_dump}" />' if path_dump else ""
    xml = f"""<Input>
  <RNG seed="{seed}" />
  <IO output_prefix="bosons" />
  <Parallel procs_per_group="1" />
  <System n_d="3" n_bead="{n_bead}" beta="{beta}" pbc="0" />
  <Particles>
    <Species name="b" n_part="{n_part}" lambda="0.5" fermi="{int(fermi)}" init_type="File" file_name="init.xyz" all_beads="1" />
  </Particles>
  <Actions>
    <Action name="Kinetic" type="Kinetic" n_images="0" species="b" />
    <Action name="Trap" type="HarmonicTrap" species="b" omega="{omega}" max_level="0" />
    {pair_xml}
  </Actions>
  <Moves>
    <Move name="Bisect" type="Bisect" species="b" n_level="{n_level}" />
    <Move name="Perm" type="{perm}" species="b" n_level="{perm_level}"{extra} />
  </Moves>
  <Observables>
    <Observable name="Energy" type="Energy" />
    <Observable name="Permutation" type="Permutation" species="b"{f' sector_max="{sector_max}"' if sector_max else ""} />
    <Observable name="Sign" type="Sign" />{dump_xml}
  </Observables>
  <Algorithm>
    <Loop n_step="{n_step_outer}">
      <Loop n_step="{n_step_inner}">
        <Move name="Bisect" />
        <Move name="Perm" />
        <Observable name="Energy" />
        <Observable name="Permutation" />
        <Observable name="Sign" />
      </Loop>
      <Write />
    </Loop>
  </Algorithm>
</Input>
"""
    rng = np.random.default_rng(seed if path_seed is None else path_seed)
    path = rng.standard_normal((n_part, n_bead, 3))
    return xml, path
