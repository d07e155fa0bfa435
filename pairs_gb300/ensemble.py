"""Batched ensembles: many independent periodic LJ replicas on one GPU.

`Ensemble` concatenates the replicas' particles into one set of device arrays (a
replica table gives each its slice, box, cell grid and FP32 position grid) and runs
the mixed-precision LJ time step of `LJEngine` for all of them with one launch per
phase (pg_ensemble_*).  Between list rebuilds the steps run speculatively in chunks
captured once as a CUDA graph: a chunk of K steps is 2K kernel nodes (integrate,
force), replayed without host work; the FP64 displacement guard freezes every later
pass on the device once any replica's atom moved more than skin/2, the host then
rebuilds the replicas that need it and continues from the step after the trip.

Partial rebuilds (`partial=True`, the default with the guard policy): at a trip only the
replicas with an atom displaced by more than `select` x skin/2 since their own last build
are binned and listed again (pg_ensemble_select, pg_ensemble.rebuild); the others keep
their particle order, cells and lists.  A replica's guard reference is its own last
build, so every replica rebuilds on its own cycle; `select` below 1 rebuilds replicas
close to their trip along with the tripped ones, saving host round trips.

`autotune()` picks the threads per atom of the force kernel, its block size, the
cell size (27 cells of >= r_list, or 125 cells of >= r_list/2) and the list layout
(per-particle full or half lists, or pair-cluster half lists) by timing the candidates
on the ensemble itself.
"""
import ctypes as C
import math

import numpy as np
import torch

from . import _capi as A
from .engine import _box_quantum

INT32_MAX = 2 ** 31 - 1


def replica_grid(box, r_list, reach, pair_lists=False, index=0):
    """Cell grid of one replica: (dims, reach_x, reach) with cells of >= r_list /
    reach_x along x and >= r_list / reach along y and z.  reach 1, 2, 3 name the layouts
    (1, 1), (2, 2) and (2, 1); reach 0 takes the first of (1, 1), (2, 1), (2, 2) whose grid
    has 2 reach + 1 cells per axis (every stencil cell visited once), else (2, 2).
    Pair-cluster lists need that grid: a replica without it raises ValueError."""
    modes = {1: [(1, 1)], 2: [(2, 2)], 3: [(2, 1)], 0: [(1, 1), (2, 1), (2, 2)]}[reach]
    for rx, rr in modes:
        dims = [max(1, int(math.floor(box[d] * (rx if d == 0 else rr) / r_list))) for d in range(3)]
        if all(dims[d] >= 2 * (rx if d == 0 else rr) + 1 for d in range(3)):
            return dims, rx, rr
    if pair_lists:
        need = tuple(2 * (rx if d == 0 else rr) + 1 for d in range(3))
        raise ValueError(f"replica {index}: pair-cluster lists need {need} cells per axis at reach "
                         f"{reach}, the box gives {tuple(dims)}")
    return dims, rx, rr


class Ensemble:
    def __init__(self, replicas, *, cutoff=2.5, skin=0.3, dt=0.005, epsilon=1.0, sigma6=1.0, tpa=1, block=256,
                 reach=1, neighbor_capacity=None, policy="guard", chunk=None, graphs=True, fixed_point=None,
                 half=True, pair_lists=False, persistent=False, partial=True, select=0.6, device="cuda"):
        A.load()
        if not torch.cuda.is_available():
            raise A.PairsError("a CUDA device is required: the particle path runs only on the GPU")
        if policy not in ("guard", "every"):
            raise ValueError(f"unknown ensemble rebuild policy {policy!r}")
        self.dev = torch.device(device)
        self.policy = policy
        self.graphs = graphs and policy == "guard"
        # persistent: a chunk's plain steps as one cooperative launch (pg_ensemble_steps)
        # instead of two kernel nodes per step; needs fixed-point positions
        self.persistent = bool(persistent) and policy == "guard"
        # partial rebuilds: the replicas whose displacement reached select * skin/2
        if not 0.0 < select < 0.95:
            raise ValueError("select must lie in (0, 0.95): the tripped replicas must be selected")
        self.partial = bool(partial) and policy == "guard"
        self.select2 = (select * 0.5 * skin) ** 2
        self.cutoff, self.skin, self.dt = cutoff, skin, dt
        self.r_list = cutoff + skin
        self.r_list2 = self.r_list * self.r_list
        self.half_skin2 = (0.5 * skin) ** 2
        self.nrep = len(replicas)
        sizes = [len(r["pos"]) for r in replicas]
        self.sizes = np.array(sizes, dtype=np.int64)
        self.first = np.concatenate([[0], np.cumsum(self.sizes)[:-1]]).astype(np.int64)
        self.n = int(self.sizes.sum())
        self.boxes = np.array([np.asarray(r["box"], dtype=np.float64) for r in replicas])
        for L in self.boxes:
            if min(L) <= 2.0 * self.r_list:
                raise ValueError("every replica box must be longer than 2 (cutoff + skin)")
        # fixed-point positions (2^32 units per replica box) for the force pass and the
        # guard: a listed pair stays below half a box while every box exceeds
        # 2 (r_list + skin) (the guard bounds each displacement by skin/2); the list
        # build keeps the compensated hi/lo screen, split again at every binning
        fx_ok = all(min(L) > 2.0 * (self.r_list + skin) for L in self.boxes)
        if fixed_point and not fx_ok:
            raise ValueError("fixed-point positions need every replica box longer than 2 (cutoff + 2 skin)")
        self.fixed_point = fx_ok if fixed_point is None else bool(fixed_point)
        if self.persistent and not self.fixed_point:
            raise ValueError("persistent ensemble steps need fixed-point positions")
        self.pair_lists = False
        self.ts = 0
        self.nbuilds = 0
        self.rebuilt_atoms = 0                 # atoms binned and listed again, over all builds
        self.host_syncs = 0
        self.chunk = chunk
        self._cycle = 6
        self._build_ts = 0
        self._graphs = {}
        self.graph_kernels = 0                 # kernels run by graph replays
        self.graph_captured = 0                # kernels the library counted while capturing
        self.stream = torch.cuda.Stream(device=self.dev)
        self.sh = C.c_void_p(self.stream.cuda_stream)

        f64, f32, i32 = torch.float64, torch.float32, torch.int32
        n = self.n
        z = lambda shape, dt: torch.zeros(shape, dtype=dt, device=self.dev)
        t = self.t = {}
        for name in ("pos", "vel", "pos_ref"):
            t[name] = z((n, 4), f64)
        for name in ("pos_hi", "pos_lo", "ref_hi", "ref_lo", "force32"):
            t[name] = z((n, 4), f32)
        if self.fixed_point:
            t["pos_fx"] = z((n, 4), i32)
            t["ref_fx"] = z((n, 4), i32)
        t["mass"] = z((n,), f64)
        t["type"] = z((n,), i32)
        t["uid"] = z((n,), i32)
        t["replica_of"] = z((n,), i32)
        hp = np.zeros((n, 4))
        hv = np.zeros((n, 4))
        hp[:, :3] = np.concatenate([np.asarray(r["pos"], dtype=np.float64) for r in replicas])
        hv[:, :3] = np.concatenate([np.asarray(r["vel"], dtype=np.float64) for r in replicas])
        t["pos"].copy_(torch.from_numpy(hp))
        t["vel"].copy_(torch.from_numpy(hv))
        t["mass"].copy_(torch.from_numpy(np.concatenate([np.asarray(r["mass"], dtype=np.float64) for r in replicas])))
        t["uid"].copy_(torch.from_numpy(np.arange(n, dtype=np.int32)))
        t["replica_of"].copy_(torch.from_numpy(np.repeat(np.arange(self.nrep, dtype=np.int32), self.sizes)))

        self.p = A.PgParticles()
        self.p.n = self.p.capacity = n
        for name in ("pos", "vel", "pos_ref", "pos_hi", "pos_lo", "ref_hi", "ref_lo", "force32", "mass", "type",
                     "uid", "pos_fx", "ref_fx"):
            setattr(self.p, name, t[name].data_ptr() if name in t else None)
        self.p.guard = None

        self.lj = A.PgLJParams()
        self.lj.ntypes = 1
        self.lj.cutoff2 = cutoff * cutoff
        self.lj.epsilon[0], self.lj.sigma6[0] = epsilon, sigma6

        init = A.PgStatus()
        init.guard_tripped = INT32_MAX
        # the status record, then the per-replica rebuild flags (one read gets both)
        words = np.frombuffer(bytes(init), dtype=np.int32)
        t["status"] = torch.tensor(np.concatenate([words, np.ones(self.nrep, np.int32)]), device=self.dev)
        self.status_ptr = C.c_void_p(t["status"].data_ptr())
        self.nstatus = len(words)
        self.flags_ptr = C.c_void_p(t["status"].data_ptr() + 4 * self.nstatus)
        # the build's status is copied to pinned memory behind the build, so that the
        # force pass is queued before the host waits for it
        self.status_host = torch.empty(len(words) + self.nrep, dtype=torch.int32).pin_memory()
        self.status_event = torch.cuda.Event()
        t["thermo"] = z((2 * self.nrep,), f64)
        self.e = A.PgEnsemble()
        self.e.nreplicas = self.nrep
        self.e.replica_of = t["replica_of"].data_ptr()
        # cubic boxes: the pair-cluster build screens in each replica's fixed-point units
        self.e.cubic = int(all(L[0] == L[1] == L[2] for L in self.boxes))
        self.list = A.PgNeighborList()
        self.list.stride = n
        # half lists (each interior pair once, the reaction by a vector atomic): at 512
        # replicas the build takes 3.84 ms instead of 4.60 and the step 1.87 ms instead of
        # 2.12.  The atomics make the summation order of the forces nondeterministic; full
        # lists (half=False) give bit-reproducible runs
        self.half = bool(half)
        self.list.half = int(self.half)
        self.e.half = int(self.half)
        # a liquid at rho <= 0.9 has about 4/3 pi 2.8^3 rho ~ 83 partners within r_list
        self._max_nb = int(neighbor_capacity or 112)
        self.configure(tpa, block, reach, pair_lists=pair_lists)
        with torch.cuda.stream(self.stream):
            self.rebuild(then=lambda: self._force(0))    # step 0: forces only (the reference's skip_first)
        self.ts = 1
        self._pending = False                  # no final half kick is owed for step 0

    # ------------------------------------------------------------------ layout

    def configure(self, tpa, block, reach, half=None, pair_lists=None):
        """Set the force kernel's threads per atom / block size, the cell size and, if
        given, the list layout (half or full; per-particle or pair-cluster rows); takes
        effect at the next rebuild.  reach 1: cells of >= r_list (27-cell stencil); 2:
        cells of >= r_list / 2 (125 cells); 3: cells of >= r_list / 2 along x and >= r_list
        along y and z (5 x 3 x 3 cells); 0: per replica the first of 1, 3, 2 whose grid
        has 2 reach + 1 cells per axis (else 2).

        Pair-cluster lists (pair_lists=True): one row per two consecutive particles of a
        cell, each entry a partner and which of the two members it pairs with; half lists
        on fixed-point positions, one thread per row in the force pass (tpa and block do
        not apply).  Every replica grid needs 2 reach + 1 cells per axis."""
        if half is not None:
            self.half = bool(half)
            self.list.half = int(self.half)
            self.e.half = int(self.half)
        if pair_lists is not None:
            self.pair_lists = bool(pair_lists)
        if self.pair_lists:
            if not (self.half and self.fixed_point):
                raise ValueError("pair-cluster lists are half lists on fixed-point positions")
            if self.persistent:
                raise ValueError("persistent ensemble steps run per-particle lists")
        self.tpa, self.block, self.reach = int(tpa), int(block), int(reach)
        self.e.tpa, self.e.block = self.tpa, self.block
        # the hi/lo layouts feed only the per-particle build's screen: pair-cluster lists
        # on fixed-point positions read none, and the binning then writes none
        for name in ("pos_hi", "pos_lo"):
            setattr(self.p, name, None if self.pair_lists else self.t[name].data_ptr())
        reps = (A.PgReplica * self.nrep)()
        cell0 = 0
        for r in range(self.nrep):
            R = reps[r]
            L = self.boxes[r]
            R.first, R.n = int(self.first[r]), int(self.sizes[r])
            R.cell0 = cell0
            dims, rx, rr = replica_grid(L, self.r_list, self.reach, self.pair_lists, r)
            nc = 1
            for d in range(3):
                R.dims[d] = dims[d]
                R.lo[d] = 0.0
                R.len[d] = L[d]
                R.cell_len[d] = L[d] / dims[d]
                R.inv_cell_len[d] = 1.0 / R.cell_len[d]
                nc *= dims[d]
            R.ncells = nc
            R.reach = rr
            R.reach_x = rx if rx != rr else 0
            q = _box_quantum(np.zeros(3), L)
            R.quantum = q
            for d in range(3):
                lh = round(L[d] / q) * q
                R.len_hi[d] = lh
                R.len_lo[d] = L[d] - lh
                R.fx_scale[d] = 2.0 ** 32 / L[d]
                R.fx_unit[d] = float(np.float32(L[d] / 2.0 ** 32))
            cell0 += nc
        self.ncells = cell0
        self.e.ncells = cell0
        t = self.t
        t["replicas"] = torch.frombuffer(bytearray(bytes(reps)), dtype=torch.uint8).to(self.dev)
        self.e.replicas = t["replicas"].data_ptr()
        self.cells = A.PgCells()
        self.cells.ncells = cell0
        self.cells.dims[0], self.cells.dims[1], self.cells.dims[2] = cell0, 1, 1
        t["cell_start"] = torch.zeros(cell0 + 2, dtype=torch.int32, device=self.dev)
        t["cell_count"] = torch.zeros(cell0 + 1, dtype=torch.int32, device=self.dev)
        t["particle_cell"] = torch.zeros(self.n, dtype=torch.int32, device=self.dev)
        self.cells.cell_start = t["cell_start"].data_ptr()
        self.cells.cell_count = t["cell_count"].data_ptr()
        self.cells.particle_cell = t["particle_cell"].data_ptr()
        wsb = A.load().pg_workspace_bytes(self.n, cell0)
        t["ws"] = torch.empty((int(wsb),), dtype=torch.uint8, device=self.dev)
        self.ws = A.PgWorkspace(t["ws"].data_ptr(), int(wsb))
        self._alloc_list(self._max_nb)
        self._graphs = {}
        self._full_next = True                 # new cell arrays: the next build bins every replica
        torch.cuda.synchronize(self.dev)       # the new buffers are used on self.stream

    def _alloc_list(self, max_nb):
        self._max_nb = max_nb
        self.list.max_neighbors = max_nb
        t = self.t
        if self.pair_lists:
            # nbr[k * stride + slot] over the slots of every cell of every replica
            stride = int(A.load().pg_pair_slots(self.n, self.ncells))
            t["pair_table"] = torch.zeros((stride,), dtype=torch.int32, device=self.dev)
            t["nbr"] = torch.zeros((max_nb * stride,), dtype=torch.int32, device=self.dev)
            t["count"] = torch.zeros((stride,), dtype=torch.int32, device=self.dev)
            self.list.stride = stride
            self.list.pair_table = t["pair_table"].data_ptr()
        else:
            rows = -(-max_nb // self.tpa) * self.tpa
            t.pop("pair_table", None)
            t["nbr"] = torch.zeros((rows * self.n,), dtype=torch.int32, device=self.dev)
            t["count"] = torch.zeros((self.n,), dtype=torch.int32, device=self.dev)
            self.list.stride = self.n
            self.list.pair_table = None
        self.list.nbr = t["nbr"].data_ptr()
        self.list.count = t["count"].data_ptr()
        self._graphs = {}

    # ------------------------------------------------------------------ modules

    def read_status(self):
        self.host_syncs += 1
        with torch.cuda.stream(self.stream):
            s = self.t["status"].cpu().numpy()
        self._flags = s[self.nstatus:]
        return A.PgStatus.from_buffer_copy(s[: self.nstatus].tobytes())

    def _wait_status(self):
        """The status copied by the last snapshot (the host waits for that copy only)."""
        self.status_event.synchronize()
        self.host_syncs += 1
        s = self.status_host.numpy()
        self._flags = s[self.nstatus:].copy()
        return A.PgStatus.from_buffer_copy(s[: self.nstatus].tobytes())

    def rebuild(self, partial=False, then=None):
        """Bin and list every replica again, or with partial=True (and the ensemble's
        `partial` option) only those selected by displacement.  then, if given, queues the
        work that uses the new lists (the force pass) before the host waits for the
        build's status; it is queued again if the lists had to grow."""
        # the status resets below are torch ops: they must run on the stream the
        # library's kernels run on, whichever stream the caller has current
        with torch.cuda.stream(self.stream):
            self._rebuild(partial and self.partial and not self._full_next, then)

    def _rebuild(self, partial, then=None):
        by = C.byref
        self.p.guard = None
        if partial:
            A.call("pg_ensemble_select", by(self.e), by(self.p), self.select2, self.flags_ptr, self.sh)
            self.e.rebuild = self.flags_ptr.value
        else:
            self.t["status"][self.nstatus:] = 1
        try:
            A.call("pg_ensemble_bin", by(self.e), by(self.p), by(self.cells), self.ws, self.status_ptr, self.sh)
            while True:
                self.t["status"][0] = 0
                self.t["status"][2] = 0
                A.call("pg_ensemble_build_lists", by(self.e), by(self.p), by(self.cells), by(self.list),
                       self.r_list2, self.status_ptr, self.sh)
                self.status_host.copy_(self.t["status"], non_blocking=True)
                self.status_event.record(self.stream)
                if then is not None:
                    then()
                st = self._wait_status()
                if st.nonfinite:
                    raise A.PairsError("non-finite particle position met while binning")
                if st.overflow & 32:
                    raise A.PairsError("a replica's cell grid is too small for pair-cluster lists")
                if st.overflow & 2:
                    # new (empty) list arrays: every replica is binned and listed again (the
                    # force pass queued on the short lists is redone; half lists add into
                    # the force, so it starts from zero again)
                    self._alloc_list(int(st.max_neighbors * 1.15) + 8)
                    if then is not None and self.half:
                        self.t["force32"].zero_()
                    if self.e.rebuild:
                        self.e.rebuild = None
                        self.t["status"][self.nstatus:] = 1
                        A.call("pg_ensemble_bin", by(self.e), by(self.p), by(self.cells), self.ws, self.status_ptr,
                               self.sh)
                    continue
                break
        finally:
            self.e.rebuild = None
        self.rebuilt_atoms += int(np.dot(self._flags != 0, self.sizes))
        self._full_next = False
        self.t["status"][4] = INT32_MAX
        self.nbuilds += 1
        self._build_ts = self.ts

    def _force(self, step):
        self.p.step = step
        A.call("pg_ensemble_force", C.byref(self.e), C.byref(self.p), C.byref(self.list), C.byref(self.lj), self.ws,
               self.sh)

    def _integrate(self, step, kicks, drift=1):
        self.p.step = step
        A.call("pg_ensemble_integrate", C.byref(self.e), C.byref(self.p), self.dt, kicks, drift, self.half_skin2,
               step, self.status_ptr, self.sh)

    def _chunk_launches(self, k):
        """Steps 0..k-1 of a speculative chunk (relative step numbers): one launch per
        phase and step, or one persistent launch for the chunk."""
        if self.persistent:
            A.call("pg_ensemble_steps", C.byref(self.e), C.byref(self.p), C.byref(self.list), C.byref(self.lj),
                   self.dt, self.half_skin2, 0, k, self.status_ptr, self.ws, 0.0, self.sh)
            return
        self.p.guard = self.t["status"].data_ptr() + 4 * 4
        for s in range(k):
            self._integrate(s, 2)
            self._force(s)
        self.p.guard = None

    def _run_chunk(self, k):
        if not self.graphs:
            self._chunk_launches(k)
            return
        entry = self._graphs.get(k)
        if entry is None:
            if self.persistent:
                # size the cooperative grid now: no device query inside the capture
                A.call("pg_ensemble_steps", C.byref(self.e), C.byref(self.p), C.byref(self.list),
                       C.byref(self.lj), self.dt, self.half_skin2, 0, 0, self.status_ptr, self.ws, 0.0, self.sh)
            # first use of this length: capture it (the launches of the capture are
            # not executed; the replay below runs them)
            g = torch.cuda.CUDAGraph()
            lib = A.load()
            l0 = lib.pg_kernel_launches()
            with torch.cuda.graph(g, stream=self.stream):
                self._chunk_launches(k)
            entry = (g, lib.pg_kernel_launches() - l0)
            self.graph_captured += entry[1]         # counted at capture, run by the replays
            self._graphs[k] = entry
        entry[0].replay()
        self.graph_kernels += entry[1]

    def run(self, nsteps):
        """Advance every replica by nsteps time steps."""
        target = self.ts + nsteps
        with torch.cuda.stream(self.stream):
            while self.ts < target:
                if self.policy == "every" or not self._pending:
                    # one plain step (every step with policy "every"; the first step
                    # after step 0 otherwise, which owes no final half kick)
                    self._integrate(self.ts, 2 if self._pending else 1)
                    if self.policy == "every" or self.read_status().guard_tripped != INT32_MAX:
                        self.rebuild(partial=True, then=lambda: self._force(self.ts))
                    else:
                        self._force(self.ts)
                    self.ts += 1
                    self._pending = True
                    continue
                # run up to one step past the predicted trip (the last cycle's length)
                k = self.chunk or max(2, self._cycle - (self.ts - self._build_ts) + 1)
                k = min(k, target - self.ts)
                start = self.ts
                self._run_chunk(k)
                st = self.read_status()
                g = st.guard_tripped
                if g != INT32_MAX:
                    # the device froze after the integration of relative step g: the
                    # positions are those of step start + g; rebuild, then its force
                    self.ts = start + g
                    self._cycle = max(1, self.ts - self._build_ts)
                    self.rebuild(partial=True, then=lambda: self._force(self.ts))
                    self.ts += 1
                else:
                    self.ts = start + k
                    self._cycle = max(self._cycle, self.ts - self._build_ts)
        return self

    def synchronize(self):
        self.stream.synchronize()

    # ------------------------------------------------------------------ readout

    def thermo(self):
        """Per-replica temperature at the last completed step (the owed final half
        kick is applied to a copy of the velocities)."""
        with torch.cuda.stream(self.stream):
            vel = self.t["vel"].clone()
            if self._pending:
                self._integrate(self.ts - 1, 1, drift=0)
            A.call("pg_ensemble_thermo", C.byref(self.e), C.byref(self.p), C.c_void_p(self.t["thermo"].data_ptr()),
                   self.sh)
            out = self.t["thermo"].cpu().numpy().reshape(self.nrep, 2)
            self.t["vel"].copy_(vel)
        return out[:, 0].copy()

    def replica_state(self, r):
        """(pos, vel after the pending final kick is NOT applied, force) of replica r
        in uid order."""
        self.stream.synchronize()
        a, b = int(self.first[r]), int(self.first[r] + self.sizes[r])
        uid = self.t["uid"][a:b].cpu().numpy()
        order = np.argsort(uid, kind="stable")
        pos = self.t["pos"][a:b, :3].cpu().numpy()[order]
        vel = self.t["vel"][a:b, :3].cpu().numpy()[order]
        frc = self.t["force32"][a:b, :3].cpu().numpy().astype(np.float64)[order]
        return pos, vel, frc

    def replica_pairs(self, r):
        """Verlet entries (uid_i, uid_j, sx, sy, sz) of replica r, uids counted from the
        replica's first particle."""
        self.stream.synchronize()
        a, b = int(self.first[r]), int(self.first[r] + self.sizes[r])
        if self.pair_lists:
            return self._cluster_pairs(r, a, b)
        cnt = self.t["count"].cpu().numpy()[a:b]
        nbr = self.t["nbr"].cpu().numpy().astype(np.int64) & 0xFFFFFFFF
        uid = self.t["uid"].cpu().numpy()
        tpa, stride = self.tpa, self.n
        kmax = int(cnt.max()) if len(cnt) else 0
        k = np.arange(kmax)[:, None]
        i = np.arange(a, b)[None, :]
        mask = k < cnt[None, :]
        idx = ((k // tpa) * stride + i) * tpa + k % tpa
        e = nbr[idx[mask]]
        ii = np.broadcast_to(i, mask.shape)[mask]
        j = e & ((1 << A.NBR_INDEX_BITS) - 1)
        code = e >> A.NBR_INDEX_BITS
        dec = lambda c: np.where(c == 1, 1, np.where(c == 2, -1, 0))
        return np.stack([uid[ii] - a, uid[j] - a, dec(code & 3), dec((code >> 2) & 3), dec((code >> 4) & 3)],
                        axis=1).astype(np.int32)

    def _cluster_pairs(self, r, a, b):
        """Pair-cluster entries of replica r: the member that stores the pair first; the
        image is the partner's nearest to that member at the last rebuild."""
        stride = self.list.stride
        table = self.t["pair_table"].cpu().numpy().astype(np.int64)
        cnt = self.t["count"].cpu().numpy()
        first = table & ((1 << 30) - 1)
        slots = np.nonzero((table >= 0) & (first >= a) & (first < b))[0]
        nbr = self.t["nbr"].cpu().numpy().view(np.uint32).reshape(-1, stride)
        uid = self.t["uid"].cpu().numpy()
        ref = self.t["pos_ref"][:, :3].cpu().numpy()
        kmax = int(cnt[slots].max()) if len(slots) else 0
        k = np.arange(kmax)[:, None]
        mask = k < cnt[slots][None, :]
        e = nbr[:kmax, slots][mask]
        slot_first = np.broadcast_to(first[slots][None, :], mask.shape)[mask]
        j = (e & ((1 << 30) - 1)).astype(np.int64)
        half = 0.5 * self.boxes[r]
        rows = []
        for member, bit in ((0, 1 << 30), (1, 1 << 31)):
            m = (e & np.uint32(bit)) != 0
            i = slot_first[m] + member
            d = ref[i] - ref[j[m]]
            img = np.where(d > half, 1, np.where(d < -half, -1, 0))
            rows.append(np.concatenate([(uid[i] - a)[:, None], (uid[j[m]] - a)[:, None], img], axis=1))
        return np.concatenate(rows).astype(np.int32)

    def list_size(self):
        """(pairs, entries) of the current Verlet list over all replicas: a per-particle
        entry holds one pair, a pair-cluster entry one or two (its member bits)."""
        cnt = self.t["count"][: self.list.stride]
        entries = int(cnt.sum().item())
        if not self.pair_lists:
            return entries, entries
        nbr = self.t["nbr"].view(-1, self.list.stride)
        k = torch.arange(nbr.shape[0], device=self.dev)[:, None]
        e = nbr.to(torch.int64) & 0xFFFFFFFF
        bits = ((e >> 30) & 1) + ((e >> 31) & 1)
        return int(bits[k < cnt[None, :]].sum().item()), entries


def autotune(replicas, candidates=None, steps=6, cycle=5.0, finalists=3, trial_steps=40, **kw):
    """Time layout candidates (tpa, block, reach, half) on this ensemble: threads per
    atom, block size, cell size (cells of >= r_list / reach; reach 0 per replica) and
    list layout (half lists with reactions, full lists, or half = "pairs": pair-cluster
    half lists, for the replica grids that have 2 reach + 1 cells per axis).

    Stage 1, every candidate: one list build and `steps` force passes (CUDA events);
    score = force time + build time / `cycle`, the steps between two builds of an atom.
    Stage 2, the `finalists` best scores: `trial_steps` real steps each (the guard
    schedule, partial rebuilds and CUDA-graph chunks as the ensemble runs them, after a
    few warm-up steps), timed with CUDA events; the fastest wins.  The stage-1 score
    misses what the schedule adds (how a layout's partial rebuilds and host stops
    cost), and scores within a few per cent of each other do not order the real steps.
    Returns (best, table); finalists carry step_ms in the table."""
    if candidates is None:
        candidates = [(t, b, r, h) for h in (True, False) for r in (1, 2, 3) for t in (1, 2, 4, 8) for b in (128, 256)]
        candidates += [(1, 192, r, "pairs") for r in (0, 1, 2, 3)]
    ens = Ensemble(replicas, graphs=False, **kw)
    table = []
    for tpa, block, reach, half in candidates:
        pairs = half == "pairs"
        if pairs and not ens.fixed_point:
            continue
        try:
            ens.configure(tpa, block, reach, half=True if pairs else half, pair_lists=pairs)
        except ValueError:                     # a replica grid too small for this layout
            continue
        with torch.cuda.stream(ens.stream):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(ens.stream)
            ens.rebuild()
            e1.record(ens.stream)
            f = []
            for _ in range(steps + 1):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(ens.stream)
                ens._force(0)
                b.record(ens.stream)
                f.append((a, b))
        ens.synchronize()
        build = e0.elapsed_time(e1)
        force = float(np.median([a.elapsed_time(b) for a, b in f[1:]]))
        score = force + build / cycle
        table.append(dict(tpa=tpa, block=block, reach=reach, half=half, force_ms=force, build_ms=build, score=score))
    del ens
    torch.cuda.empty_cache()
    for row in sorted(table, key=lambda r: r["score"])[:max(1, finalists)]:
        pairs = row["half"] == "pairs"
        trial = Ensemble(replicas, tpa=row["tpa"], block=row["block"], reach=row["reach"],
                         half=True if pairs else row["half"], pair_lists=pairs, **kw)
        trial.run(max(3, trial_steps // 4))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(trial.stream)
        trial.run(trial_steps)
        b.record(trial.stream)
        trial.synchronize()
        row["step_ms"] = a.elapsed_time(b) / trial_steps
        del trial
        torch.cuda.empty_cache()
    best = min((r for r in table if "step_ms" in r), key=lambda r: r["step_ms"])
    return (best["tpa"], best["block"], best["reach"], best["half"]), table
