"""Simulation: the reference's user-facing API (src/pairs/sim/simulation.py:37-452)
on top of the GB300 engine.

A user script written for the reference (declare properties and features, set up
particles, register compute kernels, call generate()) runs unchanged up to
generate(); run() -- the one addition -- executes the time loop on the GPU.  Where
the reference compiles a generated program, generate() here recognises each
compute() kernel (pairs_gb300.kernels), checks that the program is one this build
implements (the LJ point-mass program of examples/md.py, the DEM sphere program of
examples/dem.py) and prepares the plan.  CPU targets are refused: there is no CPU
fallback.
"""
import math
import os

import numpy as np

from . import kernels as K
from . import lattice
from .types import DomainPartitioners, Shapes, Target, Types


class Property:
    def __init__(self, name, ptype, value, volatile, layout=None):
        self.name, self.type, self.value, self.volatile, self.layout = name, ptype, value, volatile, layout


class FeatureProperty:
    def __init__(self, feature, name, ptype, data):
        self.feature, self.name, self.type, self.data = feature, name, ptype, list(data)


class Simulation:
    def __init__(self, ref, shapes, dims=3, timesteps=100, double_prec=False, use_contact_history=False,
                 particle_capacity=800000, neighbor_capacity=100, debug=False, precision=None,
                 ghost_sync="reference", rebuild_policy="fixed", device="cuda"):
        self.ref = ref
        self._shapes = list(shapes)
        self.dims = dims
        self.ntimesteps = timesteps
        self._double_prec = double_prec
        self._use_contact_history = use_contact_history
        self.particle_capacity = particle_capacity
        self.neighbor_capacity = neighbor_capacity
        self.debug = debug
        # GB300 knobs: FP64 everywhere for double_prec=True (the reference's meaning),
        # else the mixed path (FP32 force on fixed-point or compensated positions, FP64
        # integration).
        self.precision = precision or ("fp64" if double_prec else "mixed")
        self.ghost_sync = ghost_sync if self.precision == "fp64" else "exact"
        self.rebuild_policy = rebuild_policy
        self.device = device
        self.properties = {}
        self.features = {}
        self.feature_properties = {}
        self.contact_properties = {}
        self.position_prop = None
        self.grid = None
        self._pbc = [True] * dims
        self._partitioner = None
        self.reneighbor_frequency = 1
        self._compute_half = False
        self._compute_thermo = 0
        self._target = None
        self.vtk_file, self.vtk_frequency = None, 0
        self.setups = []           # ('fcc', args) | ('read', args) | ('dem_sc_grid', args)
        self.setup_functions = []
        self.pre_step_functions = []
        self.functions = []
        self.cell_spacing = None
        self.neighbor_spacing = None
        self.plan = None
        self.engine = None
        self.thermo_lines = []
        for name, t, v in (("uid", Types.Int32, 0), ("shape", Types.Int32, 0), ("flags", Types.Int32, 0)):
            self.properties[name] = Property(name, t, v, False)

    # ------------------------------------------------------------------ declarations
    def set_domain_partitioner(self, partitioner):
        if partitioner not in (DomainPartitioners.Regular, DomainPartitioners.RegularXY):
            raise Exception("Invalid domain partitioner.")
        self._partitioner = partitioner      # one GPU, one domain: accepted, no split

    def partitioner(self):
        return self._partitioner

    def compute_half(self):
        self._compute_half = True

    def use_double_precision(self):
        return self._double_prec

    def get_shape_id(self, shape):
        return self._shapes[shape]

    def max_shapes(self):
        return len(self._shapes)

    def ndims(self):
        return self.dims

    def pbc(self, pbc_config):
        assert len(pbc_config) == self.dims, "PBC must be specified for each dimension."
        self._pbc = list(pbc_config)

    def add_property(self, prop_name, prop_type, value=0.0, volatile=False):
        assert self.property(prop_name) is None, f"Property already defined: {prop_name}"
        self.properties[prop_name] = Property(prop_name, prop_type, value, volatile)
        return self.properties[prop_name]

    def add_position(self, prop_name, value=(0.0, 0.0, 0.0), volatile=False, layout=None):
        assert self.property(prop_name) is None, f"Property already defined: {prop_name}"
        self.position_prop = Property(prop_name, Types.Vector, list(value), volatile, layout)
        self.properties[prop_name] = self.position_prop
        return self.position_prop

    def add_feature(self, feature_name, nkinds):
        assert feature_name not in self.features, f"Feature already defined: {feature_name}"
        self.features[feature_name] = nkinds
        self.properties[feature_name] = Property(feature_name, Types.Int32, 0, False)
        return feature_name

    def add_feature_property(self, feature_name, prop_name, prop_type, prop_data):
        assert feature_name in self.features, f"Feature not found: {feature_name}"
        assert self.property(prop_name) is None, f"Property already defined: {prop_name}"
        nk = self.features[feature_name]
        assert len(prop_data) == nk * nk, f"{prop_name}: expected {nk * nk} values"
        self.feature_properties[prop_name] = FeatureProperty(feature_name, prop_name, prop_type, prop_data)
        return self.feature_properties[prop_name]

    def add_contact_property(self, prop_name, prop_type, prop_default, layout=None):
        assert self.property(prop_name) is None, f"Property already defined: {prop_name}"
        self.contact_properties[prop_name] = Property(prop_name, prop_type, prop_default, False, layout)
        return self.contact_properties[prop_name]

    def property(self, prop_name):
        return self.properties.get(prop_name) or self.feature_properties.get(prop_name) or \
            self.contact_properties.get(prop_name)

    def position(self):
        return self.position_prop

    def feature_property(self, name):
        return self.feature_properties.get(name)

    def contact_property(self, name):
        return self.contact_properties.get(name)

    def set_domain(self, grid):
        self.grid = (list(map(float, grid[0:3])), list(map(float, grid[3:6])))

    def reneighbor_every(self, frequency):
        self.reneighbor_frequency = frequency

    def read_particle_data(self, filename, prop_names, shape_id):
        for p in prop_names:
            assert self.property(p) is not None, f"read_particle_data: unknown property {p}"
        self.setups.append(("read", (filename, list(prop_names), shape_id)))

    def copper_fcc_lattice(self, nx, ny, nz, rho, temperature, ntypes):
        a = pow((4.0 / rho), (1.0 / 3.0))            # sim/copper_fcc_lattice.py:19-23
        self.set_domain([0.0, 0.0, 0.0, nx * a, ny * a, nz * a])
        self.setups.append(("fcc", (nx, ny, nz, rho, temperature, ntypes)))

    def dem_sc_grid(self, xmax, ymax, zmax, spacing, diameter, min_diameter, max_diameter, initial_velocity,
                    particle_density, ntypes):
        self.setups.append(("dem_sc_grid", (xmax, ymax, zmax, spacing, diameter, min_diameter, max_diameter,
                                            initial_velocity, particle_density, ntypes)))

    def build_cell_lists(self, spacing, store_neighbors_per_cell=False):
        self.cell_spacing = spacing

    def build_neighbor_lists(self, spacing):
        self.cell_spacing = spacing
        self.neighbor_spacing = spacing

    def compute(self, func, cutoff_radius=None, symbols={}, pre_step=False, skip_first=False):
        entry = dict(func=func, cutoff=cutoff_radius, symbols=dict(symbols), pre_step=pre_step,
                     skip_first=skip_first)
        (self.pre_step_functions if pre_step else self.functions).append(entry)

    def setup(self, func, symbols={}):
        self.setup_functions.append(dict(func=func, symbols=dict(symbols)))

    def vtk_output(self, filename, frequency=0):
        self.vtk_file, self.vtk_frequency = filename, frequency

    def target(self, target):
        if not isinstance(target, Target):
            raise TypeError("target must come from pairs_gb300.target_gpu()")
        if not target.is_gpu():
            raise NotImplementedError(
                "this build runs the particle path on the GPU only (no CPU fallback); use target_gpu()")
        self._target = target

    def compute_thermo(self, every=0):
        self._compute_thermo = every

    def enable_profiler(self):
        pass

    # ------------------------------------------------------------------ generate / run
    def generate(self):
        """Recognise the kernels and build the execution plan (no code is generated)."""
        assert self._target is not None, "Target not specified!"
        assert self.position_prop is not None, "position property not declared"
        kinds = [s[0] for s in self.setups]
        if self._shapes == [Shapes.PointMass]:
            try:
                self.plan = self._plan_lj()
            except NotImplementedError as why:
                # not the LJ / velocity-Verlet program: generated kernels (codegen.py)
                self.plan = dict(program="generic", reason=str(why))
        elif Shapes.Sphere in self._shapes:
            from .dem import plan_dem
            self.plan = plan_dem(self)
        else:
            raise NotImplementedError(f"shape set {self._shapes} is not implemented")
        self.plan["setups"] = kinds
        return self.plan

    def _symbol(self, entry, match, name):
        sym = match.symbol(name)
        if sym not in entry["symbols"]:
            raise ValueError(f"{entry['func'].__name__}: symbol {sym!r} missing from symbols")
        return float(entry["symbols"][sym])

    def _plan_lj(self):
        pos = self.position_prop.name
        pair = initial = final = None
        for e in self.pre_step_functions + self.functions:
            m = K.recognize(e["func"], families=("lj_pair", "vv_initial", "vv_final"))
            if m.family == "lj_pair":
                if e["cutoff"] is None:
                    raise ValueError("the LJ pair kernel needs a cutoff radius")
                pair = (e, m)
            elif m.family == "vv_initial":
                if not (e["pre_step"] and e["skip_first"]):
                    raise NotImplementedError("initial integration must be pre_step=True, skip_first=True")
                if m.prop("position") != pos:
                    raise ValueError("initial integration must advance the position property")
                initial = (e, m)
            else:
                if e["pre_step"] or not e["skip_first"]:
                    raise NotImplementedError("final integration must be a skip_first step kernel")
                final = (e, m)
        if pair is None or initial is None or final is None:
            raise NotImplementedError("the LJ program needs the pair kernel and both velocity-Verlet halves")
        e, m = pair
        force = m.prop("force")
        for prop in ("sigma6", "epsilon"):
            if m.prop(prop) not in self.feature_properties:
                raise ValueError(f"{m.prop(prop)} must be a feature property")
        feat = self.feature_properties[m.prop("epsilon")].feature
        if self.feature_properties[m.prop("sigma6")].feature != feat:
            raise ValueError("sigma6 and epsilon must belong to one feature")
        for ent, mm in (initial, final):
            if mm.prop("force") != force:
                raise ValueError("integration must read the force the pair kernel applies")
        dt = self._symbol(*initial, "dt")
        if self._symbol(*final, "dt") != dt:
            raise ValueError("both integration halves must use the same dt")
        if self.neighbor_spacing is None:
            raise NotImplementedError("the LJ program needs build_neighbor_lists(cutoff + skin)")
        cutoff = float(e["cutoff"])
        return dict(program="lj", cutoff=cutoff, skin=float(self.neighbor_spacing) - cutoff, dt=dt,
                    feature=feat, ntypes=self.features[feat],
                    epsilon=list(self.feature_properties[m.prop("epsilon")].data),
                    sigma6=list(self.feature_properties[m.prop("sigma6")].data),
                    velocity=initial[1].prop("velocity"), mass=initial[1].prop("mass"), force=force)

    def _initial_state(self):
        for kind, args in self.setups:
            if kind == "fcc":
                nx, ny, nz, rho, temp, ntypes = args
                st = lattice.copper_fcc_lattice(nx, ny, nz, rho, temp, ntypes)
                return st
            if kind == "read":
                from .io import read_particle_data
                return read_particle_data(self, *args)
        raise NotImplementedError("no particle setup (copper_fcc_lattice / read_particle_data) given")

    def build_engine(self):
        if self.plan is None:
            self.generate()
        if self.plan["program"] == "generic":
            from .generic import GenericEngine
            if self.precision != "fp64":
                raise NotImplementedError("generated kernels run in FP64: use double_prec=True")
            setups = [dict(e, setup=True, cutoff=None) for e in self.setup_functions]
            return GenericEngine(self, self._initial_state(), self.pre_step_functions + self.functions, setups,
                                 device=self.device)
        if self.plan["program"] != "lj":
            from .dem import build_dem_engine
            return build_dem_engine(self)
        from .engine import LJEngine
        p = self.plan
        st = self._initial_state()
        lo, hi = self.grid
        box_lo, box_hi = np.array(lo), np.array(hi)
        st = dict(st, box=box_hi - box_lo)
        return LJEngine(st, lo=box_lo, hi=box_hi, periodic=self._pbc, cutoff=p["cutoff"], skin=p["skin"],
                        dt=p["dt"], ntypes=p["ntypes"], epsilon=p["epsilon"], sigma6=p["sigma6"],
                        precision=self.precision, half=self._compute_half, sync=self.ghost_sync,
                        every=self.reneighbor_frequency, neighbor_capacity=self.neighbor_capacity,
                        policy=self.rebuild_policy, device=self.device)

    def run(self, timesteps=None, verbose=True):
        """Execute the time loop: timesteps + 1 iterations, like the generated main()
        (sim/timestep.py:13), printing "T<TAB>P" at the thermo cadence."""
        self.engine = self.build_engine()
        eng = self.engine
        nsteps = (self.ntimesteps if timesteps is None else timesteps) + 1
        if self.plan["program"] == "dem":
            return self._run_dem(eng, nsteps)
        every = self._compute_thermo
        for _ in range(nsteps):
            ts = eng.ts
            eng.step()
            if every and (ts == 0 or (ts + 1) % every == 0):
                t, p = eng.compute_thermo()
                line = "%g\t%g" % (t, p)
                self.thermo_lines.append(line)
                if verbose:
                    print(line)
            if self.vtk_file is not None and (self.vtk_frequency == 0 or ts % self.vtk_frequency == 0):
                from .io import write_vtk
                write_vtk(self, eng, ts)
        return eng

    def _run_dem(self, eng, nsteps):
        """DEM time loop: the engine advances in chunks between VTK frames.  The frame of
        step ts is written after that step, at the end of the time-step body
        (sim/simulation.py:422-423)."""
        from .io import write_vtk
        vtk = self.vtk_file is not None
        freq = self.vtk_frequency if vtk else 0
        while eng.ts < nsteps:
            if not vtk:
                end = nsteps
            elif freq == 0:
                end = eng.ts + 1
            else:
                end = min(nsteps, -(-eng.ts // freq) * freq + 1)   # just past the next frame step
            eng.run(end - eng.ts)
            ts = eng.ts - 1
            if vtk and (freq == 0 or ts % freq == 0):
                write_vtk(self, eng, ts)
        return eng
