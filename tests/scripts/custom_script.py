"""A user script with kernels outside the LJ / velocity-Verlet templates, written
against the reference's API and used with pairs_gb300 in place of pairs.  Its
kernels are those of oracle/ref_custom.py, the script fed to the reference's own
generator for the golden fixtures custom6 / custom6_half (program "capped") and
custom_wca (program "wca")."""


def capped_lj(i, j):
    rsq = squared_distance(i, j)
    sr2 = 1.0 / rsq
    sr6 = sr2 * sr2 * sr2 * sigma6[i, j]
    r = sqrt(rsq)
    flj = 48.0 * sr6 * (sr6 - 0.5) * sr2 * epsilon[i, j] - fshift / r
    fmag = min(flj, fcap)
    apply(force, delta(i, j) * fmag)


def initial_integrate(i):
    linear_velocity[i] += (dt * 0.5) * force[i] / mass[i]
    position[i] += dt * linear_velocity[i]


def damped_final_integrate(i):
    linear_velocity[i] += (dt * 0.5) * force[i] / mass[i]
    speed2 = squared_length(linear_velocity[i])
    if speed2 > vmax2:
        linear_velocity[i] = linear_velocity[i] * damping
    else:
        linear_velocity[i] = linear_velocity[i] * 1.0
    kinetic[i] = 0.5 * mass[i] * speed2


def wca_soft(i, j):
    d = delta(i, j)
    rsq = squared_distance(i, j)
    skip_when(rsq > wca_rc2)
    r = sqrt(rsq)
    sr2 = 1.0 / rsq
    sr6 = sr2 * sr2 * sr2
    fwca = 48.0 * sr6 * (sr6 - 0.5) * sr2
    fsoft = max(ksoft * (sigma_s - r), 0.0) / r
    apply(force, d * (fwca + fsoft))


def clamped_final_integrate(i):
    linear_velocity[i] += (dt * 0.5) * force[i] / mass[i]
    v2 = dot(linear_velocity[i], linear_velocity[i])
    scale = select(v2 > vmax2, vscale, 1.0)
    linear_velocity[i] = linear_velocity[i] * scale
    steps_done[i] += 1
    accel[i] = normalized(force[i]) * length(force[i]) / mass[i]


def build(pairs, cfg, **opts):
    ntypes = cfg.get("ntypes", 1)
    sym = cfg["symbols"]
    psim = pairs.simulation("custom", [pairs.point_mass()], timesteps=cfg["timesteps"], double_prec=True, **opts)
    psim.target(pairs.target_gpu())
    psim.add_position('position')
    psim.add_property('mass', pairs.real(), 1.0)
    psim.add_property('linear_velocity', pairs.vector())
    psim.add_property('force', pairs.vector(), volatile=True)
    psim.add_property('kinetic', pairs.real(), 0.0)
    psim.add_property('steps_done', pairs.int32(), 0)
    psim.add_property('accel', pairs.vector())
    psim.add_feature('type', ntypes)
    psim.add_feature_property('type', 'epsilon', pairs.real(), cfg.get("epsilon", [1.0] * (ntypes * ntypes)))
    psim.add_feature_property('type', 'sigma6', pairs.real(), cfg.get("sigma6", [1.0] * (ntypes * ntypes)))
    n = cfg["n"]
    psim.copper_fcc_lattice(n[0], n[1], n[2], cfg.get("rho", 0.8442), cfg.get("temp", 1.44), ntypes)
    psim.set_domain_partitioner(pairs.regular_domain_partitioner())
    psim.compute_thermo(cfg.get("thermo_every", 100))
    psim.reneighbor_every(cfg.get("reneighbor_every", 20))
    if cfg.get("half", False):
        psim.compute_half()
    psim.build_neighbor_lists(cfg.get("cutoff", 2.5) + cfg.get("skin", 0.3))
    psim.compute(initial_integrate, symbols={'dt': sym["dt"]}, pre_step=True, skip_first=True)
    if cfg.get("program", "capped") == "capped":
        psim.compute(capped_lj, cfg.get("cutoff", 2.5), symbols={'fshift': sym["fshift"], 'fcap': sym["fcap"]})
        psim.compute(damped_final_integrate, symbols={'dt': sym["dt"], 'vmax2': sym["vmax2"],
                                                      'damping': sym["damping"]}, skip_first=True)
    else:
        psim.compute(wca_soft, cfg.get("cutoff", 2.5), symbols={'wca_rc2': sym["wca_rc2"], 'ksoft': sym["ksoft"],
                                                                 'sigma_s': sym["sigma_s"]})
        psim.compute(clamped_final_integrate, symbols={'dt': sym["dt"], 'vmax2': sym["vmax2"],
                                                       'vscale': sym["vscale"]}, skip_first=True)
    return psim
