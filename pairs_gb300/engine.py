"""Device state and time stepping of the LJ particle path on one GPU.

`LJEngine` owns every buffer as a torch tensor (the C library allocates nothing)
and runs the reference's time-step order (sim/simulation.py:387-417,
sim/timestep.py:36-61) through the C ABI:

    ts > 0:   initial_integrate            (pre_step, skip_first)
    rebuild:  bin particles (wrap + cell sort) + build Verlet list
    always:   LJ force
    ts > 0:   final_integrate              (skip_first)
    cadence:  thermo

A rebuild happens when the schedule asks for it ((ts+1) % every == 0 or ts == 0 for
the reference's fixed schedule) and also whenever the FP64 displacement guard saw a
particle move more than skin/2 since the last build (policy "guard").  Capacity
overflow follows the reference's resize protocol: the kernel reports the size it
needed, the host grows the buffer and re-runs the build
(transformations/modules.py:159-205).
"""
import ctypes as C
import math

import numpy as np
import torch

from . import _capi as A

INT32_MAX = 2 ** 31 - 1
BARRIER_TIMEOUT = 16                # pg_status.overflow bit 4 (pg_lj_steps)


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _box_quantum(lo, hi):
    span = max(max(abs(lo[d]), abs(hi[d])) + (hi[d] - lo[d]) for d in range(3))
    return 2.0 ** (math.ceil(math.log2(span)) - 22)


def set_fixed_point_units(box):
    """Fixed-point position units of a box (pg_box.fx_scale / fx_unit): 2^32 units
    per box length on every axis."""
    for d in range(3):
        box.fx_scale[d] = 2.0 ** 32 / box.len[d]
        box.fx_unit[d] = float(np.float32(box.len[d] / 2.0 ** 32))


class LJEngine:
    """One periodic (or walled) box of point masses with Lennard-Jones forces."""

    def __init__(self, state, *, lo=None, hi=None, periodic=(True, True, True), cutoff=2.5, skin=0.3,
                 dt=0.005, ntypes=1, epsilon=None, sigma6=None, precision="fp64", half=False,
                 sync="exact", every=20, neighbor_capacity=100, policy="fixed", device="cuda",
                 capacity=None, fused=True, tiles=None, tile_tpa=2, tile_atoms=224, cell_reach=1,
                 cell_reach_x=None, fixed_point=None, graphs=True, persistent=None, pair_lists=None):
        A.load()
        if not torch.cuda.is_available():
            raise A.PairsError("a CUDA device is required: the particle path runs only on the GPU")
        self.dev = torch.device(device)
        self.precision = {"fp64": A.PG_FP64, "mixed": A.PG_MIXED}[precision]
        self.sync = {"exact": A.PG_SYNC_EXACT, "reference": A.PG_SYNC_REFERENCE}[sync]
        if self.sync == A.PG_SYNC_REFERENCE and self.precision != A.PG_FP64:
            raise ValueError("reference image sync is defined for the FP64 path only")
        if policy not in ("fixed", "guard", "fixed+guard", "learned", "ema") and not str(policy).startswith("interval:"):
            raise ValueError(f"unknown rebuild policy {policy!r}")
        if (policy in ("learned", "ema") or str(policy).startswith("interval:")) and sync == "reference":
            raise ValueError("speculative rebuild policies need exact image sync")
        self.policy = policy
        self.fused = fused
        self.graphs = bool(graphs)
        self._graphs = {}
        self._deferred = []             # schedule bookkeeping run once the next chunk is queued
        self.graph_replays = 0
        self.graph_kernels = 0          # kernels run by graph replays
        self.graph_captured = 0         # kernels the library counted while capturing
        pos = np.asarray(state["pos"], dtype=np.float64)
        n = len(pos)
        box = np.asarray(state["box"], dtype=np.float64)
        lo = np.zeros(3) if lo is None else np.asarray(lo, dtype=np.float64)
        hi = lo + box if hi is None else np.asarray(hi, dtype=np.float64)
        self.n = n
        self.cap = int(capacity or n)
        self.cutoff, self.skin, self.dt, self.every = cutoff, skin, dt, every
        self.r_list = cutoff + skin
        self.r_list2 = self.r_list * self.r_list
        self.half_skin2 = (0.5 * skin) ** 2
        self.ts = 0
        self._pending_final = False
        self.since_build = 0
        self.nbuilds = 0
        self.host_syncs = 0
        self.rewinds = 0
        self.skipped_steps = 0
        self.thermo_log = []
        self.schedule = None
        self.next_rebuild = 0
        self._cycle_start = 0

        # ---- box
        self.box = A.PgBox()
        q = _box_quantum(lo, hi)
        for d in range(3):
            self.box.lo[d], self.box.hi[d] = lo[d], hi[d]
            self.box.len[d] = hi[d] - lo[d]
            self.box.periodic[d] = int(bool(periodic[d]))
            lh = round(self.box.len[d] / q) * q
            self.box.len_hi[d] = lh
            self.box.len_lo[d] = self.box.len[d] - lh
        self.box.quantum = q
        set_fixed_point_units(self.box)

        # ---- particles
        f64, f32, i32 = torch.float64, torch.float32, torch.int32
        cap = self.cap
        z = lambda shape, dt: torch.zeros(shape, dtype=dt, device=self.dev)
        self.t = {}
        t = self.t
        t["pos"] = z((cap, 4), f64)
        t["vel"] = z((cap, 4), f64)
        t["pos_ref"] = z((cap, 4), f64)
        t["mass"] = z((cap,), f64)
        t["type"] = z((cap,), i32)
        t["uid"] = z((cap,), i32)
        t["flags"] = z((cap,), i32)
        if self.precision == A.PG_FP64:
            t["force"] = z((cap, 4), f64)
        else:
            t["force32"] = z((cap, 4), f32)
        if self.sync == A.PG_SYNC_REFERENCE:
            t["pos_prev1"] = z((cap, 4), f64)
            t["pos_prev2"] = z((cap, 4), f64)
        hp = torch.zeros((n, 4), dtype=f64)
        hp[:, :3] = torch.from_numpy(pos)
        t["pos"][:n].copy_(hp)
        hv = torch.zeros((n, 4), dtype=f64)
        hv[:, :3] = torch.from_numpy(np.asarray(state["vel"], dtype=np.float64))
        t["vel"][:n].copy_(hv)
        t["mass"][:n].copy_(torch.from_numpy(np.asarray(state["mass"], dtype=np.float64)))
        t["type"][:n].copy_(torch.from_numpy(np.asarray(state["type"], dtype=np.int32)))
        uid = state.get("uid")
        uid = np.arange(n, dtype=np.int32) if uid is None else np.asarray(uid, dtype=np.int32)
        t["uid"][:n].copy_(torch.from_numpy(uid))
        if state.get("flags") is not None:
            t["flags"][:n].copy_(torch.from_numpy(np.asarray(state["flags"], dtype=np.int32)))
        self.p = A.PgParticles()
        self.p.n, self.p.capacity = n, cap
        self.p.hilo_stride = 1
        self._bind_particles()

        # ---- cells of at least r_list and the 27-cell stencil (cell_reach=2: half-width
        # cells and 125 cells, 40% fewer candidates but measured slower at 1M atoms,
        # 1.06 vs 0.84 ms per build, from the per-cell overhead of 2.3-atom cells)
        self.cells = A.PgCells()
        reach = int(cell_reach)
        if reach not in (1, 2) or (reach == 2 and (tiles or any(periodic[d] and self.box.len[d] <= 2 * self.r_list
                                                                 for d in range(3)))):
            raise ValueError("cell_reach 2 needs global lists and periodic boxes longer than 2 (cutoff + skin)")
        # half lists: cells half as wide in x (reach 2 along x, 5 x 3 x 3 cells) by
        # default where the box allows it.  A half list keeps the partners above a
        # particle in x; with narrower x slabs the build scans 13.5 cell volumes per
        # particle instead of 18.
        long_x = not periodic[0] or self.box.len[0] > 2 * self.r_list
        if cell_reach_x is None:
            reach_x = 2 if half and not tiles and reach == 1 and long_x else reach
        else:
            reach_x = int(cell_reach_x)
            if reach_x not in (1, 2) or (reach_x == 2 and (tiles or not long_x)):
                raise ValueError("cell_reach_x 2 needs global lists and a box longer than 2 (cutoff + skin) in x")
        self.cells.reach = reach
        self.cells.reach_x = reach_x
        self.reach_axes = (reach_x, reach, reach)
        ncells = 1
        for d in range(3):
            L = self.box.len[d]
            dims = max(1, int(math.floor(L * self.reach_axes[d] / self.r_list)))
            self.cells.dims[d] = dims
            self.cells.cell_len[d] = L / dims
            ncells *= dims
        self.cells.ncells = ncells

        # ---- FP32 position layout (the mixed path's forces, the list build's screen).
        # Fixed point (one int4 per particle, periodic images without shifts) where
        # the box allows it: every axis periodic with at least 2 reach + 2 cells (a
        # candidate then lies less than half a box away); compensated hi/lo float4
        # pairs otherwise, and for tile lists.
        fx_ok = (not tiles and all(periodic) and
                 all(self.cells.dims[d] >= 2 * self.reach_axes[d] + 2 for d in range(3)))
        if fixed_point and not fx_ok:
            raise ValueError("fixed-point positions need global lists and a periodic box "
                             "of at least 2 reach + 2 cells per axis")
        self.fixed_point = fx_ok if fixed_point is None else bool(fixed_point)
        if self.fixed_point:
            t["pos_fx"] = z((cap, 4), i32)
            t["ref_fx"] = z((cap, 4), i32)
        else:
            # hi and lo as two float4 arrays (an interleaved 32-byte record per particle,
            # hilo_stride 2, measured slower for the partner gathers: 257 vs 233 us)
            t["pos_hi"] = z((cap, 4), f32)
            t["pos_lo"] = z((cap, 4), f32)
            t["ref_hi"] = z((cap, 4), f32)
            t["ref_lo"] = z((cap, 4), f32)
        self._bind_particles()
        t["cell_start"] = z((ncells + 2,), i32)
        t["cell_count"] = z((ncells + 1,), i32)
        t["particle_cell"] = z((cap,), i32)
        self.cells.cell_start = t["cell_start"].data_ptr()
        self.cells.cell_count = t["cell_count"].data_ptr()
        self.cells.particle_cell = t["particle_cell"].data_ptr()

        # ---- neighbour list: 16-bit tile lists on the mixed path with full lists
        # (shared-memory neighbourhoods), 32-bit global lists otherwise
        self.list = A.PgNeighborList()
        self.list.stride = cap
        self.list.half = int(bool(half))
        # pair-cluster half lists (one list per two particles of a cell, pairlist.cu) on
        # the mixed path with fixed-point positions; the per-particle half list's pair
        # set, a partner gathered once and one reaction for both members
        pc_ok = (self.precision == A.PG_MIXED and self.fixed_point and bool(half) and not tiles
                 and not persistent)
        if pair_lists and not pc_ok:
            raise ValueError("pair-cluster lists need the mixed path, fixed-point positions and half lists, "
                             "without tiles or persistent steps")
        self.pair_lists = pc_ok if pair_lists is None else bool(pair_lists)
        if self.pair_lists:
            self.list.stride = int(A.load().pg_pair_slots(cap, ncells))
            t["pair_table"] = torch.full((self.list.stride,), -1, dtype=torch.int32, device=self.dev)
            self.list.pair_table = t["pair_table"].data_ptr()
        # tile lists are opt-in: on GB300 the global-list kernels, which gather partners
        # through L1, measured faster (1M atoms, full lists: 0.31 ms global vs 0.94 ms
        # tiles at 2 threads per atom)
        self.tiles = False if tiles is None else bool(tiles)
        if self.tiles:
            if self.precision != A.PG_MIXED or half:
                raise ValueError("tile lists are implemented for the mixed-precision path with full lists")
            if tile_tpa not in (1, 2, 4):
                raise ValueError("tile_tpa must be 1, 2 or 4")
            mean = max(n / ncells, 1.0)
            self.list.tile_tpa = int(tile_tpa)
            # tiles of equal height: the column's cells split into ceil(dims_z / tz) tiles
            dz = self.cells.dims[2]
            ntz = max(1, int(round(dz / max(1.0, tile_atoms / mean))))
            self._set_tile_z(-(-dz // ntz))
        self._alloc_list(int(neighbor_capacity))

        # ---- LJ parameters
        self.lj = A.PgLJParams()
        self.lj.ntypes = ntypes
        self.lj.cutoff2 = cutoff * cutoff
        eps = np.ones(ntypes * ntypes) if epsilon is None else np.asarray(epsilon, dtype=np.float64)
        sig6 = np.ones(ntypes * ntypes) if sigma6 is None else np.asarray(sigma6, dtype=np.float64)
        for k in range(ntypes * ntypes):
            self.lj.epsilon[k], self.lj.sigma6[k] = eps[k], sig6[k]

        # ---- status, workspace, small outputs
        init = A.PgStatus()
        init.guard_tripped = INT32_MAX
        t["status_init"] = torch.tensor(np.frombuffer(bytes(init), dtype=np.int32).copy(), device=self.dev)
        t["status"] = t["status_init"].clone()
        self.status_ptr = C.c_void_p(t["status"].data_ptr())
        self.status_host = torch.zeros_like(t["status"], device="cpu").pin_memory()
        self.status_event = torch.cuda.Event()
        wsb = A.load().pg_workspace_bytes(cap, ncells)
        t["ws"] = torch.empty((int(wsb),), dtype=torch.uint8, device=self.dev)
        self.ws = A.PgWorkspace(t["ws"].data_ptr(), int(wsb))
        t["thermo"] = z((3,), f64)
        t["energy"] = z((2,), f64)
        self.stream = torch.cuda.current_stream(self.dev)
        self.sh = C.c_void_p(self.stream.cuda_stream)
        A.call("pg_split_positions", C.byref(self.box), C.byref(self.p), self.sh)
        # plain steps between rebuild points as one persistent launch (pg_lj_steps) in the
        # graph chunks: mixed precision on fixed-point positions with global lists.
        # Opt-in: at 1M atoms the chunk graph of separate kernels measured 0.345 ms/step
        # against 0.397 for the persistent launch (three grid barriers per step, and far
        # fewer loads in flight in its grid-stride phases than in a 1M-thread launch)
        can_persist = self.precision == A.PG_MIXED and self.fixed_point and not self.tiles and not self.pair_lists
        if persistent and not can_persist:
            raise ValueError("persistent steps need the mixed path with fixed-point positions and global lists")
        self.persistent = bool(persistent) and can_persist
        if self.persistent:
            # queries the device once (outside any stream capture)
            A.call("pg_lj_steps", C.byref(self.box), C.byref(self.p), C.byref(self.list), C.byref(self.lj), self.dt,
                   self.half_skin2, 0, 0, self.status_ptr, self.ws, 0.0, self.sh)
        if self.speculative:
            self.p.guard = t["status"].data_ptr() + 4 * 4         # &status->guard_tripped
        if policy == "learned":
            from .schedule import LearnedSchedule
            self.schedule = LearnedSchedule(self)
        elif policy == "ema":
            from .schedule import EMASchedule
            self.schedule = EMASchedule(self)

    @property
    def speculative(self):
        return self.policy in ("learned", "ema") or str(self.policy).startswith("interval:")

    # ------------------------------------------------------------------ buffers

    def _bind_particles(self):
        t, p = self.t, self.p
        for name in ("pos", "pos_prev1", "pos_prev2", "vel", "force", "force32", "pos_hi", "pos_lo",
                     "pos_ref", "ref_hi", "ref_lo", "pos_fx", "ref_fx", "mass", "type", "uid", "flags"):
            setattr(p, name, t[name].data_ptr() if name in t else None)

    # shared memory per tile block: 32 B per staged particle, below the 227 KB a
    # block may use; the build flags neighbourhoods larger than this
    SMEM_LIMIT = 220 * 1024
    TILE_LIMIT = SMEM_LIMIT // 32

    def _set_tile_z(self, tz):
        self.list.tile_z = int(tz)
        ntz = -(-self.cells.dims[2] // self.list.tile_z)
        ntiles = self.cells.dims[0] * self.cells.dims[1] * ntz
        self.t["tile_table"] = torch.zeros((ntiles * A.TILE_RECORD_WORDS,), dtype=torch.int32, device=self.dev)
        self.list.tile_table = self.t["tile_table"].data_ptr()
        self.list.tile_capacity = self.TILE_LIMIT

    def _alloc_list(self, max_nb):
        self._graphs = {}                   # captured graphs hold the old list's address
        self.list.max_neighbors = max_nb
        self.t.pop("nbr", None)
        self.t.pop("nbr16", None)
        if self.tiles:
            self.t["nbr16"] = torch.zeros((max_nb, self.cap), dtype=torch.int16, device=self.dev)
            self.list.nbr16 = self.t["nbr16"].data_ptr()
            self.list.nbr = None
        else:
            self.t["nbr"] = torch.zeros((max_nb, self.list.stride), dtype=torch.int32, device=self.dev)
            self.list.nbr = self.t["nbr"].data_ptr()
            self.list.nbr16 = None
        self.t["count"] = torch.zeros((self.list.stride,), dtype=torch.int32, device=self.dev)
        self.list.count = self.t["count"].data_ptr()

    def _rotate_ring(self):
        t = self.t
        t["pos_prev2"], t["pos_prev1"], t["pos"] = t["pos_prev1"], t["pos"], t["pos_prev2"]
        self._bind_particles()

    def read_status(self):
        self.host_syncs += 1
        s = self.t["status"].cpu().numpy()
        return A.PgStatus.from_buffer_copy(s.tobytes())

    def _snapshot_status(self):
        """Queue a copy of the status to pinned host memory (read by _wait_status)."""
        self.status_host.copy_(self.t["status"], non_blocking=True)
        self.status_event.record(self.stream)

    def _wait_status(self):
        self.status_event.synchronize()
        self.host_syncs += 1
        return A.PgStatus.from_buffer_copy(self.status_host.numpy().tobytes())

    def reset_status(self):
        self.t["status"].copy_(self.t["status_init"])

    # ------------------------------------------------------------------ modules

    def rebuild(self, pre_bin=None, then=None, post_bin=None):
        """Bin + sort + Verlet build, growing the list until it fits.  Returns the
        step at which the guard had tripped before this build (INT32_MAX if none).
        pre_bin, if given, queues work on the state before the particles are
        re-sorted.  post_bin, if given, queues work on the binned state beside the list
        build (the learned schedule's features and prediction, on its own stream) and
        returns an event that later work on the engine's stream waits for, or None.
        then, if given, queues the work that uses the new list (the force pass) before
        the host waits for the build's status, so the host's bookkeeping overlaps it;
        it is queued again if the build has to be repeated."""
        by = C.byref
        if pre_bin is not None:
            pre_bin()
        st_dev = self.t["status"]
        st_dev[0:1].bitwise_and_(BARRIER_TIMEOUT)       # overflow (a barrier timeout stays to be seen)
        st_dev[1:3].zero_()                             # max_cell_count, max_neighbors
        A.call("pg_bin_particles", by(self.box), by(self.p), by(self.cells), self.ws, self.status_ptr, self.sh)
        side = post_bin() if post_bin is not None else None
        guard = None
        first = True
        while True:
            if not first:
                st_dev[0:1].bitwise_and_(BARRIER_TIMEOUT)
                st_dev[2] = 0
            first = False
            if self.tiles:
                st_dev[6] = 0                           # max_tile_staged
                self.list.tile_capacity = self.TILE_LIMIT
            A.call("pg_build_neighbor_lists", by(self.box), by(self.p), by(self.cells), by(self.list),
                   self.r_list2, self.status_ptr, self.sh)
            self._snapshot_status()
            st_dev[4] = INT32_MAX                       # guard reset, after the snapshot
            early = then is not None and not self.tiles
            if early:
                self.list.steps_since_build = 0
                if side is not None:
                    self.stream.wait_event(side)
                then()
            st = self._wait_status()
            guard = self._guard_abs(st.guard_tripped) if guard is None else guard
            if st.nonfinite:
                raise A.PairsError("non-finite particle position met while binning")
            if st.overflow & BARRIER_TIMEOUT:
                raise A.PairsError("a grid barrier of the persistent steps ran out of time: the state is unfinished")
            if st.overflow & 4:
                # a tile neighbourhood is larger than a block's shared memory: make
                # tiles shorter, or give up tiles for this system
                if self.list.tile_z > 1:
                    self._set_tile_z(max(1, self.list.tile_z // 2))
                else:
                    self.tiles = False
                    self._alloc_list(self.list.max_neighbors)
                continue
            if st.overflow & 2:
                self._alloc_list(int(st.max_neighbors * 1.2) + 8)
                continue
            break
        if self.tiles:
            # each force block stages exactly the largest neighbourhood of this build
            self.list.tile_capacity = max(1, int(st.max_tile_staged))
        self.list.steps_since_build = 0
        self.since_build = 0
        self.nbuilds += 1
        if side is not None:
            self.stream.wait_event(side)
        if then is not None and not early:
            then()
        return guard

    def force(self, energy=False):
        e = C.c_void_p(self.t["energy"].data_ptr()) if energy else None
        A.call("pg_lj_force", C.byref(self.box), C.byref(self.p), C.byref(self.cells), C.byref(self.list),
               C.byref(self.lj),
               self.precision, self.sync, e, self.ws, self.sh)

    def advance(self, kicks):
        """Initial half step of this time step, preceded by the deferred final half
        step of the previous one when kicks == 2 (one fused pass)."""
        by = C.byref
        if self.precision == A.PG_MIXED:
            A.call("pg_integrate_mixed", by(self.box), by(self.p), self.dt, kicks, 1, self.half_skin2,
                   self.device_step(self.ts), self.status_ptr, self.sh)
            return
        if self.sync == A.PG_SYNC_REFERENCE:
            self._rotate_ring()
        name = "pg_final_initial_integrate" if kicks == 2 else "pg_initial_integrate"
        A.call(name, by(self.box), by(self.p), self.dt, self.precision, self.half_skin2, self.device_step(self.ts),
               self.sync, self.status_ptr, self.sh)

    def flush(self):
        """Apply a deferred final half step (velocities at full step)."""
        if not self._pending_final:
            return
        self._pending_final = False
        self.p.step = self.device_step(max(self.ts - 1, 0))
        by = C.byref
        if self.precision == A.PG_MIXED:
            A.call("pg_integrate_mixed", by(self.box), by(self.p), self.dt, 1, 0, self.half_skin2,
                   self.device_step(self.ts), self.status_ptr, self.sh)
        else:
            A.call("pg_final_integrate", by(self.box), by(self.p), self.dt, self.precision, self.sh)

    def compute_thermo(self):
        self.settle()
        self.flush()
        A.call("pg_compute_thermo", C.byref(self.box), C.byref(self.p), C.c_void_p(self.t["thermo"].data_ptr()),
               self.ws, self.sh)
        out = self.t["thermo"].cpu().numpy()
        return float(out[0]), float(out[1])

    def potential_energy(self):
        """(PE, virial sum r.F) of the current positions (FP64 sums)."""
        self.settle()
        if self.nbuilds == 0:
            self.rebuild()
        self.p.step = self.device_step(self.ts - 1 if self.ts > 0 else 0)
        self.force(energy=True)
        e = self.t["energy"].cpu().numpy()
        return float(e[0]), float(e[1])

    # ------------------------------------------------------------------ schedule

    def device_step(self, ts):
        """Step number the kernels see for time step ts: counted from the start of the
        current rebuild cycle, so that a captured chunk of steps replays unchanged in
        any cycle.  The guard word holds such numbers too."""
        return ts - self._cycle_start

    def _guard_abs(self, g):
        return g if g == INT32_MAX else g + self._cycle_start

    def guard_step(self):
        """Step at which the guard tripped since the last build (INT32_MAX if none)."""
        self.host_syncs += 1
        return self._guard_abs(int(self.t["status"][4].item()))

    def guard_tripped(self):
        return self.guard_step() != INT32_MAX

    def needs_rebuild(self, ts):
        fixed = ((ts + 1) % self.every == 0) or ts == 0
        if self.policy == "fixed":
            return fixed
        if self.policy == "guard":
            return ts == 0 or self.guard_tripped()
        return fixed or self.guard_tripped()

    def _rewind(self, s):
        """The guard tripped at step s < ts: every pass after advance(s) was skipped on
        the device; continue from step s (positions x(s), forces still to compute)."""
        self.skipped_steps += self.ts - s
        self.rewinds += 1
        self.ts = s
        self._pending_final = False
        self.thermo_log = [e for e in self.thermo_log if e[0] < s]

    def _speculative_rebuild_point(self, ts):
        """Rebuild point of the learned / interval policies at step ts (after the
        advance of ts).  The list is rebuilt from the current positions; if the
        guard had tripped at s < ts, the device froze at step s, so those positions
        are x(s) and the build is the one step s needed: rewind to s."""
        if ts != 0 and ts != self.next_rebuild:
            return False
        s = self.rebuild(post_bin=self._schedule_hook(), then=self.force)
        tripped_at = None
        if ts > 0 and s <= ts:
            tripped_at = s
            if s < ts:
                self._rewind(s)
        self._cycle_start = self.ts
        self._after_rebuild_schedule(self.ts, tripped_at)
        return True

    def _schedule_hook(self):
        """The learned schedule's work at a list build (features of the binned state,
        and the prediction once trained, beside the list build), or None."""
        sch = self.schedule
        if sch is None:
            return None
        return lambda: sch.sample_after_bin(predict=sch.trained)

    def _after_rebuild_schedule(self, ts, tripped_at):
        """Close the finished cycle and choose the next rebuild step."""
        sch = self.schedule
        if self.policy.startswith("interval:"):
            self.next_rebuild = ts + max(1, int(self.policy.split(":")[1]))
            return
        if self.policy == "learned" and sch.trained and sch._next is not None:
            # the new cycle's prediction came back with the rebuild's status: choose the
            # next rebuild now, and leave the cycle bookkeeping (labels, calibration, the
            # periodic training step) until the next chunk is queued on the GPU
            raw, r = sch.raw_prediction()
            self.next_rebuild = ts + max(1, int(math.floor(r * sch.margin)))
            end = ts + 1 if tripped_at is None else None

            def bookkeeping():
                if ts > 0:
                    sch.close_cycle(tripped_at, end)
                sch.open_cycle(ts)
                sch.note_prediction(raw)
                sch.history.append((ts, r))

            self._deferred.append(bookkeeping)
            return
        if ts > 0:
            sch.close_cycle(tripped_at, ts + 1 if tripped_at is None else None)
        predicted = sch.trained and sch._next is not None
        sch.open_cycle(ts)                          # the sample taken at this build
        if not sch.trained:
            # warm-up: exact guard every step, samples along the cycle
            if sch.cycles >= sch.warmup_cycles:
                sch.train()
        if sch.trained:
            if predicted:
                r = sch.predicted()                 # read back with the rebuild's status
            else:
                r, slot = sch.predicted_steps()
                if slot is not None:
                    sch.pending.append((slot, ts))
            sch.history.append((ts, r))
            self.next_rebuild = ts + max(1, int(math.floor(r * sch.margin)))

    def _flush_deferred(self):
        while self._deferred:
            self._deferred.pop(0)()

    def step(self, thermo_every=0):
        """One iteration of the reference's time loop.  The final half step of a time
        step is deferred and fused with the next step's initial half step."""
        self._flush_deferred()
        ts = self.ts
        self.p.step = self.device_step(ts)
        if ts > 0:
            self.advance(2 if self._pending_final else 1)
            self._pending_final = False
        if self.speculative and (self.schedule is None or self.schedule.trained):
            self._post_advance(False, None, thermo_every, built=self._speculative_rebuild_point(ts))
            return
        elif self.speculative:
            # learned policy warm-up: exact guard read every step
            g = ts == 0 or self.guard_tripped()
            rebuild, tripped_at = g, (ts if g and ts > 0 else None)
            if not rebuild and self.schedule.pending and \
                    (ts - self._cycle_start) % 2 == 0 and len(self.schedule.pending) < self.schedule.samples_per_cycle:
                self.schedule.record(ts)
        else:
            rebuild, tripped_at = self.needs_rebuild(ts), None
        self._post_advance(rebuild, tripped_at, thermo_every)

    def _post_advance(self, rebuild, tripped_at, thermo_every=0, built=False):
        """Second half of a time step (after the integration pass): rebuild if asked,
        force, defer the final half step, thermo."""
        ts = self.ts
        self.p.step = self.device_step(ts)
        if built:
            pass                                        # the rebuild queued the force pass
        elif rebuild:
            self.rebuild(post_bin=self._schedule_hook() if self.speculative else None, then=self.force)
            self._cycle_start = ts
            if self.speculative:
                self._after_rebuild_schedule(ts, tripped_at)
        else:
            self.since_build += 1
            self.list.steps_since_build = self.since_build
            self.force()
        if ts > 0:
            self._pending_final = True
            if not self.fused:
                self.flush()
        if thermo_every and (ts == 0 or (ts + 1) % thermo_every == 0):
            self.thermo_log.append((ts,) + self.compute_thermo())
        self.ts += 1

    def settle(self):
        """Speculative policies: make sure no guard trip is pending, so the state is
        the exact one at the current step (redo steps from a trip if needed)."""
        self._flush_deferred()
        if not self.speculative or self.ts == 0:
            return
        target = self.ts
        for _ in range(10000):
            s = self.guard_step()
            if s >= target:
                return
            self._rewind(s)
            self._post_advance(True, s)
            while self.ts < target:
                self.step()
        raise A.PairsError("settle(): guard kept tripping")

    def run(self, nsteps, thermo_every=0):
        """Advance until nsteps more time steps are done (a speculative policy may
        step back to a guard trip and redo steps).  Under a trained speculative policy
        the plain steps between two rebuild points replay as one captured CUDA graph."""
        target = self.ts + nsteps
        while self.ts < target:
            k = self._plain_run(target, thermo_every)
            if k >= 2:
                self._replay_plain(k)
            else:
                self.step(thermo_every)
        self._flush_deferred()

    # ------------------------------------------------------------------ CUDA graphs

    def _plain_run(self, target, thermo_every):
        """Number of plain steps (no rebuild point, no thermo, no host read) that can
        run from the current step, or 0."""
        if not (self.graphs and self.speculative and self.fused and not self.tiles):
            return 0
        if self.schedule is not None and not self.schedule.trained:
            return 0
        if thermo_every or not self._pending_final or self.ts <= self._cycle_start:
            return 0
        return max(0, min(self.next_rebuild, target) - self.ts)

    def _plain_launches(self, r0, k, stream_handle):
        """The kernels of k plain steps with device steps r0 .. r0 + k - 1: the fused
        final + initial half kicks with the drift and the guard, then the force pass."""
        saved = self.sh
        self.sh = stream_handle
        try:
            if self.persistent:
                self.p.step = r0 + k - 1
                A.call("pg_lj_steps", C.byref(self.box), C.byref(self.p), C.byref(self.list), C.byref(self.lj),
                       self.dt, self.half_skin2, r0, k, self.status_ptr, self.ws, 0.0, self.sh)
                return
            for r in range(r0, r0 + k):
                self.p.step = r
                if self.precision == A.PG_MIXED:
                    A.call("pg_integrate_mixed", C.byref(self.box), C.byref(self.p), self.dt, 2, 1, self.half_skin2,
                           r, self.status_ptr, self.sh)
                else:
                    A.call("pg_final_initial_integrate", C.byref(self.box), C.byref(self.p), self.dt, self.precision,
                           self.half_skin2, r, self.sync, self.status_ptr, self.sh)
                self.force()
        finally:
            self.sh = saved

    def _replay_plain(self, k):
        """Run k plain steps as one graph replay.  The graph of a (first device step,
        length) pair is captured on first use; it holds the buffers' addresses, so a
        list regrow drops every graph.  Its kernels read the guard word like any other
        launch, so steps after a trip are skipped on the device as before."""
        r0 = self.device_step(self.ts)
        entry = self._graphs.get((r0, k))
        if entry is None:
            g = torch.cuda.CUDAGraph()
            cap = torch.cuda.Stream(device=self.dev)
            cap.wait_stream(self.stream)
            lib = A.load()
            l0 = lib.pg_kernel_launches()
            with torch.cuda.graph(g, stream=cap):
                self._plain_launches(r0, k, C.c_void_p(cap.cuda_stream))
            # kernels per replay (the library counts launches when they are issued)
            entry = (g, lib.pg_kernel_launches() - l0)
            self.graph_captured += entry[1]         # counted at capture, run by the replays
            self.stream.wait_stream(cap)
            self._graphs[(r0, k)] = entry
        with torch.cuda.stream(self.stream):
            entry[0].replay()
        self._flush_deferred()                      # host bookkeeping while the chunk runs
        self.graph_replays += 1
        self.graph_kernels += entry[1]
        self.since_build += k
        self.list.steps_since_build = self.since_build
        self.p.step = r0 + k - 1
        self.ts += k

    def upload(self, pos, vel, mass=None, type=None, uid=None):
        """Replace the particle state with host arrays (n x 4 or n x 3 FP64 pos/vel,
        in any order; pinned memory makes the copies asynchronous).  The next step is
        a fresh first step (force only, rebuild)."""
        n = self.n
        t = self.t
        for key, src in (("pos", pos), ("vel", vel)):
            if src.shape[1] == 4:
                t[key][:n].copy_(src, non_blocking=True)
            else:
                t[key][:n, :3].copy_(src, non_blocking=True)
        for key, src in (("mass", mass), ("type", type), ("uid", uid)):
            if src is not None:
                t[key][:n].copy_(src, non_blocking=True)
        self.ts = 0
        self._cycle_start = 0
        self._pending_final = False

    # ------------------------------------------------------------------ readback

    def state(self):
        """Positions, velocities, forces as numpy arrays in uid order."""
        self.settle()
        self.flush()
        n = self.n
        uid = self.t["uid"][:n].cpu().numpy()
        order = np.argsort(uid, kind="stable")
        pos = self.t["pos"][:n, :3].cpu().numpy()[order]
        vel = self.t["vel"][:n, :3].cpu().numpy()[order]
        if self.precision == A.PG_FP64:
            frc = self.t["force"][:n, :3].cpu().numpy()[order]
        else:
            frc = self.t["force32"][:n, :3].cpu().numpy().astype(np.float64)[order]
        return pos, vel, frc

    def vtk_fields(self):
        """Device tensors (pos n x 4, mass, flags, uid) of the state at the current
        step, for the device VTK writer."""
        self.settle()
        self.flush()
        n, t = self.n, self.t
        return t["pos"][:n], t["mass"][:n], t["flags"][:n], t["uid"][:n]

    def _uid_order(self):
        uid = self.t["uid"][: self.n].cpu().numpy()
        return np.argsort(uid, kind="stable")

    def masses(self):
        return self.t["mass"][: self.n].cpu().numpy()[self._uid_order()]

    def flags(self):
        return self.t["flags"][: self.n].cpu().numpy()[self._uid_order()]

    def _tile_slot_tables(self):
        """Host restatement of the tile layout (tile.cu tile_layout): for every particle
        the global index and image code of each shared-memory slot of its tile."""
        dims = [self.cells.dims[d] for d in range(3)]
        per = [bool(self.box.periodic[d]) for d in range(3)]
        start = self.t["cell_start"].cpu().numpy()
        count = self.t["cell_count"].cpu().numpy()
        tz = self.list.tile_z
        ntz = (dims[2] + tz - 1) // tz
        dx, dy, dz = dims
        enc = lambda s: 1 if s > 0 else (2 if s < 0 else 0)
        tables = {}
        for cx in range(dx):
            for cy in range(dy):
                for zt in range(ntz):
                    z0, z1 = zt * tz, min(zt * tz + tz, dz)
                    segs = []
                    for pas in (0, 1):
                        for ox in (-1, 0, 1):
                            nx, sx = cx + ox, 0
                            if nx < 0 or nx >= dx:
                                if not per[0]:
                                    continue
                                sx = -1 if nx < 0 else 1
                                nx %= dx
                            for oy in (-1, 0, 1):
                                ny, sy = cy + oy, 0
                                if ny < 0 or ny >= dy:
                                    if not per[1]:
                                        continue
                                    sy = -1 if ny < 0 else 1
                                    ny %= dy
                                cell0 = (nx * dy + ny) * dz
                                parts = [(max(z0 - 1, 0), min(z1, dz - 1), 0)]
                                if z0 - 1 < 0 and per[2]:
                                    parts.append((dz - 1, dz - 1, -1))
                                if z1 >= dz and per[2]:
                                    parts.append((0, 0, 1))
                                for za, zb, sz in parts:
                                    code = enc(sx) | (enc(sy) << 2) | (enc(sz) << 4)
                                    if (code == 0) != (pas == 0):
                                        continue
                                    b = start[cell0 + za]
                                    e = start[cell0 + zb] + count[cell0 + zb]
                                    segs.append((b, e - b, code))
                    gj = np.concatenate([np.arange(b, b + c) for b, c, _ in segs]) if segs else np.zeros(0, int)
                    gc = np.concatenate([np.full(c, code) for b, c, code in segs]) if segs else np.zeros(0, int)
                    c_first = (cx * dy + cy) * dz
                    ib = start[c_first + z0]
                    ie = start[c_first + z1 - 1] + count[c_first + z1 - 1]
                    for i in range(ib, ie):
                        tables[i] = (gj, gc)
        return tables

    def _cluster_rows(self):
        """Valid entries of a pair-cluster list as a (rows, slots) mask, and the count
        per slot."""
        cnt = self.t["count"][: self.list.stride]
        k = torch.arange(self.list.max_neighbors, device=self.dev)[:, None]
        return k < cnt[None, :], cnt

    def _cluster_pairs(self):
        """Pair-cluster entries as (uid_i, uid_j, sx, sy, sz) rows, i the member that
        stores the pair; the image is the partner's nearest to i at the last rebuild."""
        stride = self.list.stride
        table = self.t["pair_table"][:stride].cpu().numpy().astype(np.int64)
        valid, _ = self._cluster_rows()
        nbr = self.t["nbr"][:, :stride].cpu().numpy().astype(np.uint32)
        uid = self.t["uid"][: self.n].cpu().numpy()
        ref = self.t["pos_ref"][: self.n, :3].cpu().numpy()
        sel = valid.cpu().numpy().nonzero()
        e = nbr[sel]
        slot = sel[1]
        first = table[slot] & ((1 << 30) - 1)
        j = (e & ((1 << 30) - 1)).astype(np.int64)
        rows = []
        for member, bit in ((0, 1 << 30), (1, 1 << 31)):
            m = (e & np.uint32(bit)) != 0
            i = first[m] + member
            d = ref[i] - ref[j[m]]
            half = 0.5 * np.array([self.box.len[k] for k in range(3)])
            img = np.where(d > half, 1, np.where(d < -half, -1, 0))
            rows.append(np.concatenate([uid[i][:, None], uid[j[m]][:, None], img], axis=1))
        return np.concatenate(rows).astype(np.int32)

    def list_counts(self):
        """Stored entries per list row owner (a particle, or a pair-cluster slot) as a
        numpy array."""
        if not self.pair_lists:
            return self.t["count"][: self.n].cpu().numpy()
        return self.t["count"][: self.list.stride].cpu().numpy()

    def list_size(self):
        """(pairs, entries) of the current Verlet list: a per-particle list stores one
        pair per entry, a pair-cluster entry one or two (its member bits)."""
        if not self.pair_lists:
            entries = int(self.t["count"][: self.list.stride].sum().item())
            return entries, entries
        valid, cnt = self._cluster_rows()
        entries = int(cnt.sum().item())
        nbr = self.t["nbr"][:, : self.list.stride]
        e = nbr.to(torch.int64) & 0xFFFFFFFF
        bits = ((e >> 30) & 1) + ((e >> 31) & 1)
        return int(bits[valid].sum().item()), entries

    def pairs(self):
        """Verlet entries as (uid_i, uid_j, sx, sy, sz) rows (list order per particle)."""
        if self.pair_lists:
            return self._cluster_pairs()
        n = self.n
        cnt = self.t["count"][:n].cpu().numpy()
        if self.tiles:
            tab = self._tile_slot_tables()
            slots = self.t["nbr16"][:, :n].cpu().numpy().astype(np.int64) & 0xFFFF
            uid = self.t["uid"][:n].cpu().numpy()
            rows = []
            dec = lambda c: np.where(c == 1, 1, np.where(c == 2, -1, 0))
            for i in range(n):
                k = cnt[i]
                if k == 0:
                    continue
                gj, gc = tab[i]
                sl = slots[:k, i]
                j, code = gj[sl], gc[sl]
                rows.append(np.stack([np.full(k, uid[i]), uid[j], dec(code & 3), dec((code >> 2) & 3),
                                      dec((code >> 4) & 3)], axis=1))
            return np.concatenate(rows).astype(np.int32) if rows else np.zeros((0, 5), np.int32)
        nbr = self.t["nbr"][:, :n].cpu().numpy().astype(np.uint32)
        uid = self.t["uid"][:n].cpu().numpy()
        rows = []
        kk = np.arange(nbr.shape[0])[:, None]
        mask = kk < cnt[None, :]
        e = nbr[mask.nonzero()]
        ii = np.broadcast_to(np.arange(n)[None, :], nbr.shape)[mask.nonzero()]
        j = (e & ((1 << A.NBR_INDEX_BITS) - 1)).astype(np.int64)
        code = e >> A.NBR_INDEX_BITS
        dec = lambda c: np.where(c == 1, 1, np.where(c == 2, -1, 0))
        rows = np.stack([uid[ii], uid[j], dec(code & 3), dec((code >> 2) & 3), dec((code >> 4) & 3)], axis=1)
        return rows.astype(np.int32)

    def cell_occupancy(self):
        return self.t["cell_count"][: self.cells.ncells].cpu().numpy()
