"""Engine for point-mass programs whose kernels are lowered by codegen.py.

It runs the reference's time step (sim/simulation.py:387-417) with one generated
CUDA kernel per compute() function:

    pre-step kernels           (skip_first ones not at ts == 0)
    rebuild, every N steps     wrap + bin + sort (pg_bin_particles, the user
                               properties permuted alongside), Verlet list
    reset volatile properties  (sim/properties.py:61-70)
    step kernels               (skip_first ones not at ts == 0)
    thermo                     at its cadence (pg_compute_thermo)

setup() kernels run once before the first step.  State is FP64.  The rebuild is the
reference's fixed schedule ((ts + 1) % every == 0 or ts == 0, sim/timestep.py:47).
Periodic images of a pair kernel's partner come from the list's image codes; with
ghost_sync "reference" an image shifted in k > 1 dimensions takes its position from
min(k - 1, steps since the build) steps back, as the reference's ghost refresh.
"""
import ctypes as C
import math

import numpy as np
import torch

from . import _capi as A
from . import codegen
from .engine import _box_quantum, set_fixed_point_units

INT32_MAX = 2 ** 31 - 1


class GenArgs(C.Structure):
    _fields_ = [("box", A.PgBox), ("p", A.PgParticles), ("list", A.PgNeighborList), ("half", C.c_int32),
                ("sync_ref", C.c_int32), ("feat_n", C.c_int32 * codegen.MAX_FEATURES),
                ("feat", C.c_void_p * codegen.MAX_FEATURES), ("prop", C.c_void_p * codegen.MAX_PROPS)]


class GenericEngine:
    def __init__(self, sim, state, entries, setups=(), device="cuda"):
        A.load()
        if not torch.cuda.is_available():
            raise A.PairsError("a CUDA device is required: the particle path runs only on the GPU")
        self.sim = sim
        self.dev = torch.device(device)
        self.modules, self.layout, self.source = codegen.lower_program(sim, list(setups) + list(entries))
        self.so_path = codegen.compile_source(self.source)
        self.lib = C.CDLL(self.so_path)
        self.fns = {}
        for m in self.modules:
            fn = getattr(self.lib, "run_" + m.name)
            fn.argtypes = [C.POINTER(GenArgs), C.c_void_p]
            fn.restype = C.c_int
            self.fns[m.name] = fn
        if sim.neighbor_spacing is None and any(m.pair for m in self.modules):
            raise NotImplementedError("pair kernels need build_neighbor_lists(cutoff + skin)")
        for m in self.modules:
            if m.pair and sim.neighbor_spacing is not None and m.cutoff > sim.neighbor_spacing:
                raise ValueError(f"{m.name}: cutoff {m.cutoff} exceeds the neighbour list radius")
        written = set().union(*[m.written for m in self.modules]) if self.modules else set()
        self.sync_ref = sim.ghost_sync == "reference"
        if self.sync_ref:
            for m in self.modules:
                moving = (m.read_j & written) - {self.layout.position}
                if moving:
                    raise NotImplementedError(
                        f"{m.name} reads {sorted(moving)} of the partner, which kernels change: the reference's "
                        "lagged ghost copies of those are not reproduced; use ghost_sync='exact'")

        pos = np.asarray(state["pos"], dtype=np.float64)
        n = len(pos)
        self.n = n
        self.cap = cap = max(n, 1)
        lo, hi = (np.asarray(x, dtype=np.float64) for x in sim.grid)
        self.ts = 0
        self.since_build = 0
        self.nbuilds = 0
        self.every = sim.reneighbor_frequency
        self.r_list = float(sim.neighbor_spacing) if sim.neighbor_spacing is not None else 0.0

        # ---- box
        self.box = A.PgBox()
        q = _box_quantum(lo, hi)
        for d in range(3):
            self.box.lo[d], self.box.hi[d] = lo[d], hi[d]
            self.box.len[d] = hi[d] - lo[d]
            self.box.periodic[d] = int(bool(sim._pbc[d]))
            lh = round(self.box.len[d] / q) * q
            self.box.len_hi[d] = lh
            self.box.len_lo[d] = self.box.len[d] - lh
        self.box.quantum = q
        set_fixed_point_units(self.box)

        # ---- particles: FP64 state plus hi/lo for the list build's FP32 screen
        f64, f32, i32 = torch.float64, torch.float32, torch.int32
        z = lambda shape, dt: torch.zeros(shape, dtype=dt, device=self.dev)
        t = self.t = {}
        for name in ("pos", "vel", "pos_ref"):
            t[name] = z((cap, 4), f64)
        t["mass"] = z((cap,), f64)
        for name in ("type", "uid", "flags"):
            t[name] = z((cap,), i32)
        for name in ("pos_hi", "pos_lo", "ref_hi", "ref_lo"):
            t[name] = z((cap, 4), f32)
        if self.sync_ref:
            t["pos_prev1"] = z((cap, 4), f64)
            t["pos_prev2"] = z((cap, 4), f64)
        # user properties by slot, filled with their declared defaults
        self.user = []
        for name in self.layout.slots:
            prop = sim.properties[name]
            kind = codegen.prop_kind(prop.type)
            if kind == codegen.VEC:
                buf = z((cap, 4), f64)
                v = prop.value if isinstance(prop.value, (list, tuple)) else [prop.value] * 3
                for d in range(3):
                    buf[:n, d] = float(v[d])
            elif kind == codegen.REAL:
                buf = z((cap,), f64)
                buf[:n] = float(prop.value or 0.0)
            else:
                buf = z((cap,), i32)
                buf[:n] = int(prop.value or 0)
            self.user.append((name, buf, 32 if kind == codegen.VEC else (8 if kind == codegen.REAL else 4)))
        self.scratch = z((cap * 32,), torch.uint8)
        hp = torch.zeros((n, 4), dtype=f64)
        hp[:, :3] = torch.from_numpy(pos)
        t["pos"][:n].copy_(hp)
        if state.get("vel") is not None:
            hv = torch.zeros((n, 4), dtype=f64)
            hv[:, :3] = torch.from_numpy(np.asarray(state["vel"], dtype=np.float64))
            t["vel"][:n].copy_(hv)
        mass = state.get("mass")
        if mass is not None:
            t["mass"][:n].copy_(torch.from_numpy(np.asarray(mass, dtype=np.float64)))
        else:
            t["mass"][:n] = float(sim.properties["mass"].value if "mass" in sim.properties else 1.0)
        if state.get("type") is not None:
            t["type"][:n].copy_(torch.from_numpy(np.asarray(state["type"], dtype=np.int32)))
        uid = state.get("uid")
        uid = np.arange(n, dtype=np.int32) if uid is None else np.asarray(uid, dtype=np.int32)
        t["uid"][:n].copy_(torch.from_numpy(uid))
        if state.get("flags") is not None:
            t["flags"][:n].copy_(torch.from_numpy(np.asarray(state["flags"], dtype=np.int32)))
        self.p = A.PgParticles()
        self.p.n, self.p.capacity, self.p.hilo_stride = n, cap, 1
        for name in ("pos", "pos_prev1", "pos_prev2", "vel", "pos_hi", "pos_lo", "pos_ref", "ref_hi", "ref_lo",
                     "mass", "type", "uid", "flags"):
            setattr(self.p, name, t[name].data_ptr() if name in t else None)

        # ---- cells and list
        self.cells = A.PgCells()
        self.cells.reach = 1
        ncells = 1
        for d in range(3):
            L = self.box.len[d]
            dims = max(1, int(math.floor(L / self.r_list))) if self.r_list > 0 else 1
            self.cells.dims[d] = dims
            self.cells.cell_len[d] = L / dims
            ncells *= dims
        self.cells.ncells = ncells
        t["cell_start"] = z((ncells + 2,), i32)
        t["cell_count"] = z((ncells + 1,), i32)
        t["particle_cell"] = z((cap,), i32)
        self.cells.cell_start = t["cell_start"].data_ptr()
        self.cells.cell_count = t["cell_count"].data_ptr()
        self.cells.particle_cell = t["particle_cell"].data_ptr()
        self.list = A.PgNeighborList()
        self.list.stride = cap
        self.list.half = int(bool(sim._compute_half))
        self._alloc_list(int(sim.neighbor_capacity))

        # ---- status, workspace, argument block
        init = A.PgStatus()
        init.guard_tripped = INT32_MAX
        t["status_init"] = torch.tensor(np.frombuffer(bytes(init), dtype=np.int32).copy(), device=self.dev)
        t["status"] = t["status_init"].clone()
        self.status_ptr = C.c_void_p(t["status"].data_ptr())
        wsb = A.load().pg_workspace_bytes(cap, ncells)
        t["ws"] = torch.empty((int(wsb),), dtype=torch.uint8, device=self.dev)
        self.ws = A.PgWorkspace(t["ws"].data_ptr(), int(wsb))
        t["thermo"] = z((3,), f64)
        self.feat_tensors = []
        self.args = GenArgs()
        for name, (slot, feature) in self.layout.features.items():
            fp = sim.feature_properties[name]
            ft = torch.tensor([float(x) for x in fp.data], dtype=f64, device=self.dev)
            self.feat_tensors.append(ft)
            self.args.feat[slot] = ft.data_ptr()
            self.args.feat_n[slot] = sim.features[feature]
        self.args.half = self.list.half
        self.args.sync_ref = int(self.sync_ref)
        self.stream = torch.cuda.current_stream(self.dev)
        self.sh = C.c_void_p(self.stream.cuda_stream)
        self._bind_user()
        for m in self.modules:
            if m.setup:
                self._launch(m)

    # ------------------------------------------------------------------ buffers
    def _alloc_list(self, max_nb):
        self.list.max_neighbors = max_nb
        self.t["nbr"] = torch.zeros((max_nb, self.cap), dtype=torch.int32, device=self.dev)
        self.t["count"] = torch.zeros((self.cap,), dtype=torch.int32, device=self.dev)
        self.list.nbr = self.t["nbr"].data_ptr()
        self.list.nbr16 = None
        self.list.count = self.t["count"].data_ptr()

    def _bind_user(self):
        for k, (_, buf, _) in enumerate(self.user):
            self.args.prop[k] = buf.data_ptr()

    def _launch(self, m):
        self.args.box = self.box
        self.args.p = self.p
        self.args.list = self.list
        rc = self.fns[m.name](C.byref(self.args), self.sh)
        if rc != 0:
            raise A.PairsError(f"generated kernel {m.name} failed to launch ({rc})")

    # ------------------------------------------------------------------ modules
    def rebuild(self):
        by = C.byref
        lib = A.load()
        st = self.t["status"]
        st[0:3].zero_()
        A.call("pg_bin_particles", by(self.box), by(self.p), by(self.cells), self.ws, self.status_ptr, self.sh)
        if self.user:
            perm = lib.pg_bin_permutation(self.n, self.cells.ncells, self.ws)
            for _, buf, nb in self.user:
                A.call("pg_permute", self.n, C.c_void_p(perm), C.c_void_p(buf.data_ptr()),
                       C.c_void_p(self.scratch.data_ptr()), nb, self.sh)
                buf.reshape(-1).view(torch.uint8)[: self.n * nb].copy_(self.scratch[: self.n * nb])
        while True:
            st[0] = 0
            st[2] = 0
            A.call("pg_build_neighbor_lists", by(self.box), by(self.p), by(self.cells), by(self.list),
                   self.r_list * self.r_list, self.status_ptr, self.sh)
            s = A.PgStatus.from_buffer_copy(st.cpu().numpy().tobytes())
            if s.nonfinite:
                raise A.PairsError("non-finite particle position met while binning")
            if s.overflow & 2:
                self._alloc_list(int(s.max_neighbors * 1.2) + 8)
                continue
            break
        self.list.steps_since_build = 0
        self.since_build = 0
        self.nbuilds += 1

    def _reset_volatile(self):
        for name, prop in self.sim.properties.items():
            if not prop.volatile:
                continue
            for uname, buf, _ in self.user:
                if uname == name:
                    buf.zero_()
            if name == "linear_velocity" and self.layout.props[name][1] == "a.p.vel":
                self.t["vel"].zero_()
            if name == "mass" and self.layout.props[name][1] == "a.p.mass":
                self.t["mass"].zero_()

    def _rotate_ring(self):
        t = self.t
        t["pos_prev2"], t["pos_prev1"], t["pos"] = t["pos_prev1"], t["pos"], t["pos_prev2"]
        t["pos"].copy_(t["pos_prev1"])
        for name in ("pos", "pos_prev1", "pos_prev2"):
            setattr(self.p, name, t[name].data_ptr())

    def step(self):
        """One iteration of the reference's time loop."""
        ts = self.ts
        if self.sync_ref and ts > 0:
            self._rotate_ring()
        for m in self.modules:
            if m.pre_step and not m.setup and not (m.skip_first and ts == 0):
                self._launch(m)
        if ts == 0 or (ts + 1) % self.every == 0:
            self.rebuild()
        else:
            self.since_build += 1
            self.list.steps_since_build = self.since_build
        self._reset_volatile()
        for m in self.modules:
            if not m.pre_step and not m.setup and not (m.skip_first and ts == 0):
                self._launch(m)
        self.ts += 1

    def run(self, nsteps):
        for _ in range(nsteps):
            self.step()

    def compute_thermo(self):
        if "linear_velocity" not in self.layout.props or self.layout.props["linear_velocity"][1] != "a.p.vel" or \
                "mass" not in self.layout.props:
            raise NotImplementedError("thermo needs the linear_velocity (vector) and mass (real) properties")
        A.call("pg_compute_thermo", C.byref(self.box), C.byref(self.p), C.c_void_p(self.t["thermo"].data_ptr()),
               self.ws, self.sh)
        out = self.t["thermo"].cpu().numpy()
        return float(out[0]), float(out[1])

    # ------------------------------------------------------------------ readback
    def _order(self):
        uid = self.t["uid"][: self.n].cpu().numpy()
        return np.argsort(uid, kind="stable")

    def property(self, name):
        """A property's values in uid order (n x 3 for vectors)."""
        order = self._order()
        n = self.n
        kind, base = self.layout.props[name]
        if base == "a.p.pos":
            arr = self.t["pos"][:n, :3]
        elif base == "a.p.vel":
            arr = self.t["vel"][:n, :3]
        elif base == "a.p.mass":
            arr = self.t["mass"][:n]
        elif base == "a.p.type":
            arr = self.t["type"][:n]
        elif base in ("a.p.uid", "a.p.flags"):
            arr = self.t[base.split(".")[-1]][:n]
        else:
            buf = next(b for uname, b, _ in self.user if uname == name)
            arr = buf[:n, :3] if kind == codegen.VEC else buf[:n]
        return arr.cpu().numpy()[order]

    def masses(self):
        return self.t["mass"][: self.n].cpu().numpy()[self._order()]

    def flags(self):
        return self.t["flags"][: self.n].cpu().numpy()[self._order()]

    def state(self):
        """Positions, velocities and the first applied vector property (the force)."""
        force = next((m.applied[0] for m in self.modules if m.pair and m.applied), None)
        vel = self.property("linear_velocity") if "linear_velocity" in self.layout.props else None
        return self.property(self.layout.position), vel, (self.property(force) if force else None)
