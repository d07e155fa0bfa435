"""DEM particle path on one GPU: spheres and half-space walls with the linear
spring-dashpot contact model of the reference's DEM example (examples/dem.py).

`DEMEngine` owns the device state as torch tensors and runs, per time step, the
reference's DEM program order (sim/simulation.py:387-417 with a cell-list program):

    rebuild (when needed):  wrap + bin + sort (pg_dem_bin), sphere list (pg_dem_build_list)
    always:                 gravity + contacts + history clean-up (pg_dem_force)
                            Euler with rotation + displacement guard (pg_dem_euler)

The reference rebins every step and scans the 27 cells around each sphere.  Here a
candidate list with skin is rebuilt only when the FP64 guard saw a sphere move more
than skin/2 since the last build; steps run speculatively in chunks (each kernel
does nothing once the guard tripped at an earlier step, the host then rebuilds and
resumes at the step after the trip), so the contacts found are the reference's.
policy="every" rebuilds every step instead.

The module also holds the recognition templates of the DEM kernels and the plan
that Simulation.generate() builds for a DEM program.
"""
import ctypes as C
import math

import numpy as np
import torch

from . import _capi as A
from . import kernels as K

INT32_MAX = 2 ** 31 - 1

# ---------------------------------------------------------------------------- templates
# The kernels of examples/dem.py in the placeholder form of pairs_gb300.kernels
# (I/J particles, P_ properties, S_ symbols, L_ locals).  A user function matches
# only if it has exactly this statement and expression structure.

DEM_SETUP = """
def f(I):
    P_rotation_matrix[I] = diagonal_matrix(1.0)
    P_rotation_quat[I] = default_quaternion()

    if is_sphere(I):
        P_inv_inertia[I] = inversed(diagonal_matrix(0.4 * P_mass[I] * P_radius[I] * P_radius[I]))

    else:
        P_mass[I] = S_infinity
        P_inv_inertia[I] = 0.0
"""

DEM_GRAVITY = """
def f(I):
    L_volume = (4.0 / 3.0) * S_pi * P_radius[I] * P_radius[I] * P_radius[I]
    P_force[I][2] = P_force[I][2] - (S_rho_p - S_rho_f) * L_volume * S_gravity
"""

DEM_CONTACT = """
def f(I, J):
    L_delta = -penetration_depth(I, J)
    skip_when(L_delta < 0.0)

    L_meff = 1.0 / ((1.0 / P_mass[I]) + (1.0 / P_mass[J]))
    L_kn = L_meff * (S_pi * S_pi + S_ln_e * S_ln_e) / (S_tc * S_tc)
    L_kt = S_kappa * L_kn
    L_dn = -2.0 * L_meff * S_ln_e / S_tc
    L_dt_ = sqrt(S_kappa) * L_dn

    L_vwi = P_linear_velocity[I] + cross(P_angular_velocity[I], contact_point(I, J) - P_position[I])
    L_vwj = P_linear_velocity[J] + cross(P_angular_velocity[J], contact_point(I, J) - P_position[J])

    L_rel = -(L_vwi - L_vwj)
    L_reln = dot(L_rel, contact_normal(I, J)) * contact_normal(I, J)
    L_relt = L_rel - L_reln
    L_fN = L_kn * L_delta * contact_normal(I, J) + L_dn * L_reln

    L_tsd = P_tsd[I, J]
    L_ivm0 = P_ivm[I, J]
    L_ivm = select(L_ivm0 > 0.0, L_ivm0, length(L_rel))
    L_stick = P_sticking[I, J]

    L_rot = L_tsd - contact_normal(I, J) * dot(L_tsd, contact_normal(I, J))
    L_rl2 = squared_length(L_rot)
    L_nts = S_dt * L_relt + select(L_rl2 <= 0.0, zero_vector(), L_rot * sqrt(squared_length(L_tsd) / L_rl2))

    L_fTLS = L_kt * L_nts + L_dt_ * L_relt
    L_fTLS_len = length(L_fTLS)
    L_t = normalized(L_fTLS)

    L_fstat = P_friction_static[I, J] * length(L_fN)
    L_fdyn = P_friction_dynamic[I, J] * length(L_fN)
    L_thr = 1e-8

    L_c1 = L_stick == 1 and length(L_relt) < L_thr and L_fTLS_len < L_fstat
    L_c2 = L_stick == 1 and L_fTLS_len < L_fdyn
    L_ffa = select(L_c1, L_fstat, L_fdyn)
    L_nstick = select(L_c1 or L_c2 or L_fTLS_len < L_fdyn, 1, 0)
    P_tsd[I, J] = select(not L_c1 and not L_c2 and L_kt > 0.0, (L_ffa * L_t - L_dt_ * L_relt) / L_kt, L_nts)

    P_ivm[I, J] = L_ivm
    P_sticking[I, J] = L_nstick

    L_fTabs = min(L_fTLS_len, L_ffa)
    L_fT = L_fTabs * L_t
    L_pf = L_fN + L_fT

    apply(P_force, L_pf)
    apply(P_torque, cross(contact_point(I, J) - P_position, L_pf))
"""

DEM_EULER = """
def f(I):
    L_im = 1.0 / P_mass[I]
    P_position[I] += 0.5 * L_im * P_force[I] * S_dt * S_dt + P_linear_velocity[I] * S_dt
    P_linear_velocity[I] += L_im * P_force[I] * S_dt
    L_wdot = P_rotation_matrix[I] * (P_inv_inertia[I] * P_torque[I]) * transposed(P_rotation_matrix[I])
    L_phi = P_angular_velocity[I] * S_dt + 0.5 * L_wdot * S_dt * S_dt
    P_rotation_quat[I] = quaternion(L_phi, length(L_phi)) * P_rotation_quat[I]
    P_rotation_matrix[I] = quaternion_to_rotation_matrix(P_rotation_quat[I])
    P_angular_velocity[I] += L_wdot * S_dt
"""

for _name, _src in (("dem_setup", DEM_SETUP), ("dem_gravity", DEM_GRAVITY), ("dem_contact", DEM_CONTACT),
                    ("dem_euler", DEM_EULER)):
    K.register(_name, _src)

DEM_FAMILIES = ("dem_gravity", "dem_contact", "dem_euler")


def _ptr(t):
    return None if t is None else t.data_ptr()


def _sym(entry, match, name):
    sym = match.symbol(name)
    if sym not in entry["symbols"]:
        raise ValueError(f"{entry['func'].__name__}: symbol {sym!r} missing from symbols")
    return entry["symbols"][sym]


def plan_dem(sim):
    """Recognise the DEM program (setup, gravity, contact, Euler, in that order) and
    collect its constants."""
    if len(sim.setup_functions) != 1:
        raise NotImplementedError("the DEM program needs exactly one setup kernel (update_mass_and_inertia)")
    se = sim.setup_functions[0]
    sm = K.recognize(se["func"], families=("dem_setup",))
    if not math.isinf(float(_sym(se, sm, "infinity"))):
        raise ValueError("the half-space mass of the setup kernel must be infinity")
    if sim.pre_step_functions:
        raise NotImplementedError("the DEM program has no pre-step kernels")
    found = [(e, K.recognize(e["func"], families=DEM_FAMILIES)) for e in sim.functions]
    if [m.family for _, m in found] != list(DEM_FAMILIES):
        raise NotImplementedError("the DEM program is gravity, linear spring-dashpot contact, Euler, in that order "
                                  f"(got {[m.family for _, m in found]})")
    (ge, gm), (ce, cm), (ee, em) = found
    pos = sim.position_prop.name
    if cm.prop("position") != pos or em.prop("position") != pos:
        raise ValueError("contact and Euler kernels must use the position property")
    force, torque = cm.prop("force"), cm.prop("torque")
    if gm.prop("force") != force or em.prop("force") != force or em.prop("torque") != torque:
        raise ValueError("gravity, contact and Euler must act on the same force / torque properties")
    for name in ("tsd", "ivm", "sticking"):
        if sim.contact_property(cm.prop(name)) is None:
            raise ValueError(f"{cm.prop(name)} must be a contact property")
    fs, fd = sim.feature_property(cm.prop("friction_static")), sim.feature_property(cm.prop("friction_dynamic"))
    if fs is None or fd is None or fs.feature != fd.feature:
        raise ValueError("friction_static / friction_dynamic must be feature properties of one feature")
    dt = float(_sym(ce, cm, "dt"))
    if float(_sym(ee, em, "dt")) != dt:
        raise ValueError("contact and Euler kernels must use the same dt")
    pi = float(_sym(ce, cm, "pi"))
    if float(_sym(ge, gm, "pi")) != pi:
        raise ValueError("gravity and contact kernels must use the same pi")
    if ce["cutoff"] is None:
        raise ValueError("the contact kernel needs a cutoff radius (the linked-cell width)")
    if sim.cell_spacing is None:
        raise NotImplementedError("the DEM program needs build_cell_lists(spacing)")
    # (rho_p - rho_f) in the symbols' own type, as the generated expression
    drho = float(_sym(ge, gm, "rho_p") - _sym(ge, gm, "rho_f"))
    ntypes = sim.features[fs.feature]
    return dict(program="dem", dt=dt, pi=pi, kappa=float(_sym(ce, cm, "kappa")),
                ln_e=float(_sym(ce, cm, "ln_e")), tc=float(_sym(ce, cm, "tc")), drho=drho,
                gravity=float(_sym(ge, gm, "gravity")), ntypes=ntypes, friction_static=list(fs.data),
                friction_dynamic=list(fd.data), cell_spacing=float(sim.cell_spacing),
                contact_capacity=int(sim.neighbor_capacity))


def dem_params(dt, kappa, ln_e, tc, drho, gravity, friction_static, friction_dynamic, pi=math.pi, ntypes=1,
               skin=0.0, kn=0.0):
    """Contact-model constants.  kn = 0: normal stiffness from the collision time tc
    (examples/dem.py:22-26); kn > 0: that fixed stiffness, damping from the
    restitution coefficient (ln_e)."""
    p = A.PgDemParams()
    p.dt, p.pi, p.kappa, p.ln_e, p.tc, p.drho, p.gravity, p.skin = dt, pi, kappa, ln_e, tc, drho, gravity, skin
    p.kn = kn
    p.ntypes = ntypes
    fs = list(friction_static)
    fd = list(friction_dynamic)
    if len(fs) != ntypes * ntypes or len(fd) != ntypes * ntypes or ntypes > 4:
        raise ValueError("friction tables must have ntypes*ntypes entries, ntypes <= 4")
    for k in range(ntypes * ntypes):
        p.friction_static[k], p.friction_dynamic[k] = fs[k], fd[k]
    return p


class DEMEngine:
    """Spheres and half spaces in an orthorhombic box (periodic or walled per axis)."""

    GATHERED = ("vel", "angvel", "quat", "normal", "mass", "radius", "inv_inertia", "type", "shape")
    CONTACT = ("ccount", "partner", "sticking", "history")
    MAX_CONTACTS = 64            # the contact kernels mark a sphere's used records in a 64-bit mask

    def __init__(self, state, *, lo, hi, periodic=(True, True, False), params, skin=None, contact_capacity=20,
                 neighbor_capacity=32, policy="guard", chunk=None, capacity=None, device="cuda", precision="fp64"):
        A.load()
        if not torch.cuda.is_available():
            raise A.PairsError("a CUDA device is required: the particle path runs only on the GPU")
        if policy not in ("guard", "every"):
            raise ValueError(f"unknown DEM rebuild policy {policy!r}")
        self.dev = torch.device(device)
        self.policy = policy
        self.precision = {"fp64": A.PG_FP64, "mixed": A.PG_MIXED}[precision]
        pos = np.asarray(state["pos"], dtype=np.float64).reshape(-1, 3)
        n = len(pos)
        self.n = n
        self.cap = int(capacity or n)
        lo = np.asarray(lo, dtype=np.float64)
        hi = np.asarray(hi, dtype=np.float64)
        shape = np.asarray(state.get("shape", np.zeros(n)), dtype=np.int32)
        radius = np.asarray(state["radius"], dtype=np.float64)
        rmax = float(radius[shape == 0].max()) if (shape == 0).any() else 1.0
        self.skin = 0.5 * rmax if skin is None else float(skin)
        self.half_skin2 = (0.5 * self.skin) ** 2
        self.prm = params
        self.prm.skin = self.skin
        self.dt = params.dt
        self.ts = 0
        self.nbuilds = 0
        self.host_syncs = 0
        self.need_build = True
        self.contact_regrows = 0
        self.chunk = chunk
        self._cycle = 4
        self._build_ts = 0

        self.box = A.PgBox()
        for d in range(3):
            self.box.lo[d], self.box.hi[d] = lo[d], hi[d]
            self.box.len[d] = hi[d] - lo[d]
            self.box.periodic[d] = int(bool(periodic[d]))
        self.box.quantum = 1.0

        f64, i32 = torch.float64, torch.int32
        cap = self.cap
        z = lambda shp, dt: torch.zeros(shp, dtype=dt, device=self.dev)
        t = self.t = {}
        for name in ("pos", "force", "torque", "pos_ref"):
            t[name] = z((cap, 4), f64)
        t["pos32"] = z((cap, 4), torch.float32)
        for name in ("uid", "flags"):
            t[name] = z((cap,), i32)
        self.sets = []
        ccap = int(contact_capacity)
        if not 1 <= ccap <= self.MAX_CONTACTS:
            raise ValueError(f"contact_capacity must be in 1..{self.MAX_CONTACTS}")
        for _ in range(2):
            s = {}
            for name in ("vel", "angvel", "quat", "normal"):
                s[name] = z((cap, 4), f64)
            for name in ("mass", "radius", "inv_inertia"):
                s[name] = z((cap,), f64)
            for name in ("type", "shape"):
                s[name] = z((cap,), i32)
            s["ccount"] = z((cap,), i32)
            s["partner"] = z((ccap, cap), i32)
            s["sticking"] = z((ccap, cap), i32)
            s["history"] = z((ccap, cap, 4), f64)
            self.sets.append(s)
        self.ccap = ccap
        self.n_infinite = int((shape != 0).sum())

        def put(tensor, arr, width=None):
            a = torch.from_numpy(np.ascontiguousarray(arr))
            if width:
                h = torch.zeros((n, 4), dtype=tensor.dtype)
                h[:, :width] = a.reshape(n, width).to(tensor.dtype)
                tensor[:n].copy_(h)
            else:
                tensor[:n].copy_(a.to(tensor.dtype))

        cur = self.sets[0]
        put(t["pos"], pos, 3)
        put(cur["vel"], np.asarray(state["vel"], dtype=np.float64), 3)
        put(cur["angvel"], np.asarray(state.get("angvel", np.zeros((n, 3))), dtype=np.float64), 3)
        put(cur["normal"], np.asarray(state.get("normal", np.zeros((n, 3))), dtype=np.float64), 3)
        put(cur["mass"], np.asarray(state["mass"], dtype=np.float64))
        put(cur["radius"], radius)
        put(cur["type"], np.asarray(state.get("type", np.zeros(n)), dtype=np.int32))
        put(cur["shape"], shape)
        put(t["uid"], np.asarray(state["uid"], dtype=np.int32))
        put(t["flags"], np.asarray(state.get("flags", np.zeros(n)), dtype=np.int32))

        self.d = A.PgDemParticles()
        self.spare = A.PgDemParticles()
        self.c = A.PgContacts()
        self.spare_c = A.PgContacts()
        self._bind()

        # cell grid: cells at least as wide as the largest list radius 2 r_max + skin
        self.cells = A.PgCells()
        reach = 2.0 * rmax + self.skin
        ncells = 1
        for d in range(3):
            L = self.box.len[d]
            dims = max(1, int(math.floor(L / reach)))
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
        self._alloc_list(int(neighbor_capacity))

        init = A.PgStatus()
        init.guard_tripped = INT32_MAX
        t["status_init"] = torch.tensor(np.frombuffer(bytes(init), dtype=np.int32).copy(), device=self.dev)
        t["status"] = t["status_init"].clone()
        self.status_ptr = C.c_void_p(t["status"].data_ptr())
        wsb = A.load().pg_workspace_bytes(cap, ncells)
        t["ws"] = torch.empty((int(wsb),), dtype=torch.uint8, device=self.dev)
        self.ws = A.PgWorkspace(t["ws"].data_ptr(), int(wsb))
        self.stream = torch.cuda.current_stream(self.dev)
        self.sh = C.c_void_p(self.stream.cuda_stream)
        if policy == "guard":
            self.d.guard = t["status"].data_ptr() + 4 * 4          # &status->guard_tripped
        A.call("pg_dem_setup", C.byref(self.d), C.byref(self.prm), self.sh)
        # a state taken mid-run carries its rotations and contact history
        if state.get("quat") is not None:
            put(cur["quat"], np.asarray(state["quat"], dtype=np.float64).reshape(n, 4))
        if state.get("contacts") is not None:
            self._load_contacts(*state["contacts"])

    def _load_contacts(self, ids, vals):
        """Contact records (uid_i, partner uid, sticking) + (tsd xyz, ivm), kept in the
        given order per particle."""
        ids = np.asarray(ids, dtype=np.int64).reshape(-1, 3)
        vals = np.asarray(vals, dtype=np.float64).reshape(-1, 4)
        uid = self.t["uid"][:self.n].cpu().numpy()
        index = {int(u): k for k, u in enumerate(uid)}
        if len(ids):
            most = int(np.bincount([index[int(u)] for u in ids[:, 0]], minlength=self.n).max())
            if most > self.ccap:
                self._grow_contacts(most)
        cnt = np.zeros(self.n, np.int32)
        part = np.zeros((self.ccap, self.n), np.int32)
        stick = np.zeros((self.ccap, self.n), np.int32)
        hist = np.zeros((self.ccap, self.n, 4))
        for (ui, uj, sk), v in zip(ids, vals):
            i = index[int(ui)]
            k = cnt[i]
            if k >= self.ccap:
                raise A.CapacityOverflow("contact records exceed contact_capacity")
            part[k, i], stick[k, i], hist[k, i] = uj, sk, v
            cnt[i] = k + 1
        s = self.sets[0]
        s["ccount"][:self.n].copy_(torch.from_numpy(cnt))
        s["partner"][:, :self.n].copy_(torch.from_numpy(part))
        s["sticking"][:, :self.n].copy_(torch.from_numpy(stick))
        s["history"][:, :self.n].copy_(torch.from_numpy(hist))

    # ------------------------------------------------------------------ buffers

    def _bind(self):
        t, cur, spare = self.t, self.sets[0], self.sets[1]
        for st, s, c in ((self.d, cur, self.c), (self.spare, spare, self.spare_c)):
            st.n, st.capacity = self.n, self.cap
            for name in ("pos", "force", "torque", "pos_ref", "uid", "flags", "pos32"):
                setattr(st, name, t[name].data_ptr())
            for name in ("vel", "angvel", "quat", "normal", "mass", "radius", "inv_inertia", "type", "shape"):
                setattr(st, name, s[name].data_ptr())
            c.capacity, c.stride = self.ccap, self.cap
            c.count, c.partner = s["ccount"].data_ptr(), s["partner"].data_ptr()
            c.sticking, c.history = s["sticking"].data_ptr(), s["history"].data_ptr()

    def _grow_contacts(self, need):
        """Give both contact sets room for `need` records per sphere, keeping the
        current records (the reference's resize of its contact arrays,
        transformations/modules.py:159-205)."""
        if need > self.MAX_CONTACTS:
            raise A.CapacityOverflow(f"a sphere may need {need} contact records, more than the "
                                     f"{self.MAX_CONTACTS} the contact kernels track")
        old = self.ccap
        for s in self.sets:
            for name in ("partner", "sticking", "history"):
                t = s[name]
                grown = torch.zeros((need,) + tuple(t.shape[1:]), dtype=t.dtype, device=self.dev)
                grown[:old].copy_(t)
                s[name] = grown
        self.ccap = need
        guard = self.d.guard
        self._bind()
        self.d.guard = guard
        self.contact_regrows += 1

    def _alloc_list(self, max_nb):
        self.list.max_neighbors = max_nb
        self.t["nbr"] = torch.zeros((max_nb, self.cap), dtype=torch.int32, device=self.dev)
        self.t["count"] = torch.zeros((self.cap,), dtype=torch.int32, device=self.dev)
        self.list.nbr = self.t["nbr"].data_ptr()
        self.list.count = self.t["count"].data_ptr()

    def read_status(self):
        self.host_syncs += 1
        s = self.t["status"].cpu().numpy()
        return A.PgStatus.from_buffer_copy(s.tobytes())

    # ------------------------------------------------------------------ modules

    def rebuild(self):
        by = C.byref
        A.call("pg_dem_bin", by(self.box), by(self.d), by(self.spare), by(self.c), by(self.spare_c),
               by(self.cells), self.ws, self.status_ptr, self.sh)
        self.sets.reverse()
        guard = self.d.guard
        self._bind()
        self.d.guard = guard
        while True:
            self.t["status"][0] = 0
            self.t["status"][2] = 0
            A.call("pg_dem_build_list", by(self.box), by(self.d), by(self.cells), by(self.list), by(self.prm),
                   self.status_ptr, self.sh)
            st = self.read_status()
            if st.nonfinite:
                raise A.PairsError("non-finite particle position met while binning")
            if st.overflow & 2:
                self._alloc_list(int(st.max_neighbors * 1.2) + 8)
                continue
            break
        # A sphere's contact records name partners it touches this step: list partners
        # and half spaces.  Room for that many records per sphere means the contact
        # kernel can never run out of records before the next build.
        need = int(st.max_neighbors) + self.n_infinite
        if need > self.ccap:
            self._grow_contacts(min(need, self.MAX_CONTACTS))
        self.t["status"][4] = INT32_MAX
        self.nbuilds += 1
        self.need_build = False
        self._build_ts = self.ts

    def _force(self, step):
        self.d.step = step
        A.call("pg_dem_force", C.byref(self.box), C.byref(self.d), C.byref(self.cells), C.byref(self.list),
               C.byref(self.c), C.byref(self.prm), self.precision, self.status_ptr, self.sh)

    def _euler(self, step):
        self.d.step = step
        A.call("pg_dem_euler", C.byref(self.d), C.byref(self.prm), self.precision, self.half_skin2, step,
               self.status_ptr, self.sh)

    def _check(self, st):
        if st.overflow & 8:
            raise A.CapacityOverflow(f"a particle needed more than {self.ccap} contact-history records; "
                                     "raise contact_capacity (the steps since the last check are invalid)")

    def run(self, nsteps):
        """Advance nsteps time steps."""
        target = self.ts + nsteps
        while self.ts < target:
            if self.policy == "every" or self.need_build:
                self.rebuild()
            if self.policy == "every":
                self._force(self.ts)
                self._euler(self.ts)
                self.ts += 1
                if self.ts == target:
                    self._check(self.read_status())
                continue
            if self.chunk:
                k = self.chunk
            else:
                # run up to one step past the predicted trip (the last cycle's length)
                k = max(2, self._cycle - (self.ts - self._build_ts) + 1)
            k = min(k, target - self.ts)
            start = self.ts
            for s in range(start, start + k):
                self._force(s)
                self._euler(s)
            st = self.read_status()
            self._check(st)
            if st.guard_tripped != INT32_MAX:
                self.ts = st.guard_tripped + 1
                self.need_build = True
                self._cycle = max(1, self.ts - self._build_ts)
            else:
                self.ts = start + k
                self._cycle = max(self._cycle, self.ts - self._build_ts)
        return self

    def step(self):
        return self.run(1)

    # ------------------------------------------------------------------ readout

    def vtk_fields(self):
        """Device tensors (pos n x 4, mass, flags, uid) for the device VTK writer."""
        cur = lambda k: (self.t[k] if k in self.t else self.sets[0][k])[:self.n]
        return cur("pos"), cur("mass"), cur("flags"), cur("uid")

    def _host(self, name, width=None):
        src = self.t[name] if name in self.t else self.sets[0][name]
        a = src[:self.n].cpu().numpy()
        return a[:, :width] if width else a

    def state(self):
        """Per-particle arrays ordered by uid."""
        uid = self._host("uid")
        order = np.argsort(uid, kind="stable")
        out = dict(uid=uid[order])
        for name, w in (("pos", 3), ("vel", 3), ("angvel", 3), ("force", 3), ("torque", 3), ("quat", 4)):
            out[name] = self._host(name, w)[order]
        for name in ("mass", "radius", "inv_inertia", "type", "shape"):
            out[name] = self._host(name)[order]
        out["flags"] = self._host("flags")[order]
        out["ncontacts"] = self._host("ccount")[order]
        return out

    def contacts(self):
        """Contact records: ids (m, 3) = (uid_i, partner uid, sticking) and vals (m, 4) =
        (tangential spring displacement xyz, impact velocity magnitude), sorted by
        (uid_i, partner uid)."""
        s = self.sets[0]
        uid = self._host("uid")
        cnt = s["ccount"][:self.n].cpu().numpy()
        part = s["partner"][:, :self.n].cpu().numpy()
        stick = s["sticking"][:, :self.n].cpu().numpy()
        hist = s["history"][:, :self.n].cpu().numpy()
        ids, vals = [], []
        for k in range(self.ccap):
            sel = np.nonzero(cnt > k)[0]
            if len(sel) == 0:
                continue
            ids.append(np.stack([uid[sel], part[k, sel], stick[k, sel]], axis=1))
            vals.append(hist[k, sel])
        if not ids:
            return np.zeros((0, 3), np.int32), np.zeros((0, 4))
        ids = np.concatenate(ids).astype(np.int32)
        vals = np.concatenate(vals)
        order = np.lexsort((ids[:, 1], ids[:, 0]))
        return ids[order], vals[order]


def build_dem_engine(sim, **over):
    """DEMEngine for a recognised DEM Simulation (spheres from dem_sc_grid and/or
    read_particle_data, half spaces from read_particle_data)."""
    from . import lattice
    from .io import read_particle_data
    p = sim.plan
    parts = []
    lo, hi = sim.grid
    for kind, args in sim.setups:
        if kind == "dem_sc_grid":
            xmax, ymax, zmax, spacing, diam, dmin, dmax, v0, dens, ntypes = args
            # generated on the device (bit-identical to the host restatement lattice.dem_sc_grid)
            g = lattice.dem_sc_grid_device(xmax, ymax, zmax, spacing, diam, dmin, dmax, v0, dens, ntypes,
                                           lo=lo, hi=hi)
            g = {k: v.cpu().numpy() for k, v in g.items()}
            g["pos"], g["vel"] = g["pos"][:, :3], g["vel"][:, :3]
            parts.append(g)
        elif kind == "read":
            st = read_particle_data(sim, *args)
            m = len(st["pos"])
            st.setdefault("radius", np.zeros(m))
            st["radius"] = np.asarray(st["radius"], dtype=np.float64).reshape(m)
            if "normal" in st:
                st["normal"] = np.asarray(st["normal"], dtype=np.float64).reshape(m, 3)
            parts.append(st)
        else:
            raise NotImplementedError(f"setup {kind!r} is not part of the DEM program")
    keys = ("pos", "vel", "mass", "radius", "type", "uid", "flags", "shape", "normal")
    state = {}
    for k in keys:
        arrs = []
        for st in parts:
            m = len(st["pos"])
            if k in st:
                arrs.append(np.asarray(st[k]).reshape((m, 3) if k in ("pos", "vel", "normal") else (m,)))
            else:
                arrs.append(np.zeros((m, 3)) if k in ("pos", "vel", "normal") else np.zeros(m))
        state[k] = np.concatenate(arrs) if arrs else np.zeros(0)
    prm = dem_params(p["dt"], p["kappa"], p["ln_e"], p["tc"], p["drho"], p["gravity"], p["friction_static"],
                     p["friction_dynamic"], pi=p["pi"], ntypes=p["ntypes"])
    kw = dict(lo=lo, hi=hi, periodic=sim._pbc, params=prm, contact_capacity=p["contact_capacity"],
              device=sim.device)
    kw.update(over)
    return DEMEngine(state, **kw)
