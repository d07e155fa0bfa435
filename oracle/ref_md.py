"""Lennard-Jones user script for the reference code generator (test oracle input).

Run by oracle/ref_build.py with the reference's `src/` on PYTHONPATH; it writes
`<name>.cpp` into the working directory.  The physics is the reference's own LJ
example (examples/md.py:5-17): the same pair kernel, the same velocity-Verlet
half kicks, the same schedule knobs.  Sizes and options come from the JSON in
the PAIRS_ORACLE_CFG environment variable so one script serves every parity
configuration.  Test infrastructure only.
"""
import json
import os

import pairs


def lennard_jones(i, j):
    sr2 = 1.0 / squared_distance(i, j)
    sr6 = sr2 * sr2 * sr2 * sigma6[i, j]
    apply(force, delta(i, j) * (48.0 * sr6 * (sr6 - 0.5) * sr2 * epsilon[i, j]))


def initial_integrate(i):
    linear_velocity[i] += (dt * 0.5) * force[i] / mass[i]
    position[i] += dt * linear_velocity[i]


def final_integrate(i):
    linear_velocity[i] += (dt * 0.5) * force[i] / mass[i]


cfg = json.loads(os.environ["PAIRS_ORACLE_CFG"])
name = cfg["name"]
ntypes = cfg.get("ntypes", 1)
eps = cfg.get("epsilon", [1.0] * (ntypes * ntypes))
sig6 = cfg.get("sigma6", [1.0] * (ntypes * ntypes))

psim = pairs.simulation(name, [pairs.point_mass()], timesteps=cfg["timesteps"],
                        double_prec=True, particle_capacity=cfg.get("particle_capacity", 800000),
                        neighbor_capacity=cfg.get("neighbor_capacity", 100))
psim.target(pairs.target_cpu())
psim.add_position('position')
psim.add_property('mass', pairs.real(), 1.0)
psim.add_property('linear_velocity', pairs.vector())
psim.add_property('force', pairs.vector(), volatile=True)
psim.add_feature('type', ntypes)
psim.add_feature_property('type', 'epsilon', pairs.real(), eps)
psim.add_feature_property('type', 'sigma6', pairs.real(), sig6)

if "input" in cfg:
    lo, hi = cfg["domain"]
    psim.set_domain([lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]])
    psim.read_particle_data(cfg["input"], ['uid', 'type', 'flags', 'mass', 'position', 'linear_velocity'],
                            pairs.point_mass())
else:
    n = cfg["n"]
    psim.copper_fcc_lattice(n[0], n[1], n[2], cfg.get("rho", 0.8442), cfg.get("temp", 1.44), ntypes)

psim.set_domain_partitioner(pairs.regular_domain_partitioner())
psim.compute_thermo(cfg.get("thermo_every", 100))
psim.reneighbor_every(cfg.get("reneighbor_every", 20))
if cfg.get("half", False):
    psim.compute_half()
psim.build_neighbor_lists(cfg.get("cutoff", 2.5) + cfg.get("skin", 0.3))
psim.compute(initial_integrate, symbols={'dt': cfg.get("dt", 0.005)}, pre_step=True, skip_first=True)
psim.compute(lennard_jones, cfg.get("cutoff", 2.5))
psim.compute(final_integrate, symbols={'dt': cfg.get("dt", 0.005)}, skip_first=True)
psim.generate()
