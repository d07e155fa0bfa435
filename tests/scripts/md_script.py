"""A user script written against the reference's API (the LJ program of
examples/md.py), used unchanged with pairs_gb300 in place of pairs."""


def lennard_jones(i, j):
    sr2 = 1.0 / squared_distance(i, j)
    sr6 = sr2 * sr2 * sr2 * sigma6[i, j]
    apply(force, delta(i, j) * (48.0 * sr6 * (sr6 - 0.5) * sr2 * epsilon[i, j]))


def initial_integrate(i):
    linear_velocity[i] += (dt * 0.5) * force[i] / mass[i]
    position[i] += dt * linear_velocity[i]


def final_integrate(i):
    linear_velocity[i] += (dt * 0.5) * force[i] / mass[i]


def build(pairs, nx=4, ntypes=1, timesteps=100, half=False, input_file=None, **opts):
    dt, cutoff_radius, skin = 0.005, 2.5, 0.3
    psim = pairs.simulation("md", [pairs.point_mass()], timesteps=timesteps, double_prec=True, **opts)
    psim.target(pairs.target_gpu())
    psim.add_position('position')
    psim.add_property('mass', pairs.real(), 1.0)
    psim.add_property('linear_velocity', pairs.vector())
    psim.add_property('force', pairs.vector(), volatile=True)
    psim.add_feature('type', ntypes)
    psim.add_feature_property('type', 'epsilon', pairs.real(), [1.0] * (ntypes * ntypes))
    psim.add_feature_property('type', 'sigma6', pairs.real(), [1.0] * (ntypes * ntypes))
    if input_file is None:
        psim.copper_fcc_lattice(nx, nx, nx, 0.8442, 1.44, ntypes)
    else:
        a = (4.0 / 0.8442) ** (1.0 / 3.0)
        psim.set_domain([0.0, 0.0, 0.0, nx * a, nx * a, nx * a])
        psim.read_particle_data(input_file, ['uid', 'type', 'flags', 'mass', 'position', 'linear_velocity'],
                                pairs.point_mass())
    psim.set_domain_partitioner(pairs.regular_domain_partitioner())
    psim.compute_thermo(100)
    psim.reneighbor_every(20)
    if half:
        psim.compute_half()
    psim.build_neighbor_lists(cutoff_radius + skin)
    psim.compute(initial_integrate, symbols={'dt': dt}, pre_step=True, skip_first=True)
    psim.compute(lennard_jones, cutoff_radius)
    psim.compute(final_integrate, symbols={'dt': dt}, skip_first=True)
    psim.generate()
    return psim
