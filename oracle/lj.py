"""ctypes front end of the LJ oracle (oracle/lj_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the CPU
baseline leg of bench.py, never by the product package.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(_build.build())
        L = _lib
        L.lj_fcc_lattice.restype = C.c_int
        L.lj_fcc_lattice.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int,
                                     _dp, _dp, _dp, _ip]
        L.lj_temperature.restype = C.c_double
        L.lj_temperature.argtypes = [C.c_int, _dp, _dp, C.c_double, C.c_double, C.c_double,
                                     C.POINTER(C.c_double)]
        L.lj_adjust_thermo.restype = None
        L.lj_adjust_thermo.argtypes = [C.c_int, _dp, _dp, C.c_double, C.c_double, C.c_double,
                                       C.c_double]
        L.lj_create.restype = C.c_void_p
        L.lj_create.argtypes = [C.c_int, C.c_int, _dp, _dp, C.c_double, C.c_double, C.c_double,
                                _dp, _dp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.lj_destroy.argtypes = [C.c_void_p]
        L.lj_set_state.argtypes = [C.c_void_p, C.c_int, _ip, _ip, _dp, _dp, _dp]
        L.lj_step.restype = C.c_int
        L.lj_step.argtypes = [C.c_void_p, C.c_void_p]
        L.lj_run.restype = C.c_int
        L.lj_run.argtypes = [C.c_void_p, C.c_int]
        for f in ("lj_nlocal", "lj_nghost", "lj_timestep"):
            getattr(L, f).restype = C.c_int
            getattr(L, f).argtypes = [C.c_void_p]
        L.lj_get_state.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.lj_thermo.restype = C.c_double
        L.lj_thermo.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.lj_list_size.restype = C.c_long
        L.lj_list_size.argtypes = [C.c_void_p]
        L.lj_list_pairs.restype = C.c_long
        L.lj_list_pairs.argtypes = [C.c_void_p, _ip, C.c_long]
        L.lj_cell_counts.restype = C.c_int
        L.lj_cell_counts.argtypes = [C.c_void_p, _ip, _ip, C.c_int]
        L.lj_grid.argtypes = [C.c_void_p, _ip]
    return _lib


def fcc_box(nx, ny, nz, rho=0.8442):
    a = pow(4.0 / rho, 1.0 / 3.0)
    return np.array([nx * a, ny * a, nz * a])


def fcc_lattice(nx, ny, nz, rho=0.8442, temp=1.44, ntypes=1):
    """Initial state of copper_fcc_lattice + adjust_thermo, in creation order.

    Returns dict(pos, vel, mass, type, uid, box)."""
    cap = 4 * nx * ny * nz + 16
    pos = np.zeros((cap, 3)); vel = np.zeros((cap, 3)); mass = np.zeros(cap)
    typ = np.zeros(cap, dtype=np.int32)
    n = lib().lj_fcc_lattice(nx, ny, nz, rho, ntypes, cap, pos, vel, mass, typ)
    pos, vel, mass, typ = pos[:n].copy(), vel[:n].copy(), mass[:n].copy(), typ[:n].copy()
    box = fcc_box(nx, ny, nz, rho)
    lib().lj_adjust_thermo(n, mass, vel, box[0], box[1], box[2], temp)
    return dict(pos=pos, vel=vel, mass=mass, type=typ, uid=np.arange(n, dtype=np.int32), box=box)


def temperature(mass, vel, box):
    p = C.c_double()
    t = lib().lj_temperature(len(mass), np.ascontiguousarray(mass, dtype=np.float64),
                             np.ascontiguousarray(vel, dtype=np.float64), box[0], box[1], box[2],
                             C.byref(p))
    return t, p.value


class Sim:
    """The reference's LJ time loop on one rank (see lj_oracle.c header)."""

    def __init__(self, state, ntypes=1, epsilon=None, sigma6=None, cutoff=2.5, skin=0.3,
                 dt=0.005, every=20, half=False, exact_sync=False, neigh_cap=128, nthreads=1,
                 lo=None, hi=None):
        n = len(state["mass"])
        box = np.asarray(state["box"], dtype=np.float64)
        lo = np.zeros(3) if lo is None else np.asarray(lo, dtype=np.float64)
        hi = lo + box if hi is None else np.asarray(hi, dtype=np.float64)
        eps = np.ones(ntypes * ntypes) if epsilon is None else np.asarray(epsilon, dtype=np.float64)
        sig6 = np.ones(ntypes * ntypes) if sigma6 is None else np.asarray(sigma6, dtype=np.float64)
        # ghosts: up to ~ 6 * (2.8/L) * N per face set, bounded generously
        cap = int(n * 8 + 4096)
        self.n = n
        self.box = hi - lo
        self._h = lib().lj_create(cap, ntypes, eps, sig6, cutoff, skin, dt, lo, hi, every,
                                  int(half), int(exact_sync), neigh_cap, nthreads)
        lib().lj_set_state(self._h, n, np.ascontiguousarray(state["uid"], dtype=np.int32),
                           np.ascontiguousarray(state["type"], dtype=np.int32),
                           np.ascontiguousarray(state["mass"], dtype=np.float64),
                           np.ascontiguousarray(state["pos"], dtype=np.float64),
                           np.ascontiguousarray(state["vel"], dtype=np.float64))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().lj_destroy(self._h)
            self._h = None

    def step(self, energy=False):
        e = np.zeros(2)
        rc = lib().lj_step(self._h, e.ctypes.data if energy else None)
        if rc:
            raise RuntimeError(f"oracle capacity overflow code {rc}")
        return e if energy else None

    def run(self, nsteps):
        rc = lib().lj_run(self._h, nsteps)
        if rc:
            raise RuntimeError(f"oracle capacity overflow code {rc}")

    @property
    def ts(self):
        return lib().lj_timestep(self._h)

    @property
    def nghost(self):
        return lib().lj_nghost(self._h)

    def state(self):
        """Positions, velocities, forces in uid order."""
        pos = np.zeros((self.n, 3)); vel = np.zeros((self.n, 3)); frc = np.zeros((self.n, 3))
        lib().lj_get_state(self._h, pos.ctypes.data, vel.ctypes.data, frc.ctypes.data)
        return pos, vel, frc

    def thermo(self):
        p = C.c_double()
        t = lib().lj_thermo(self._h, C.byref(p))
        return t, p.value

    def pairs(self):
        """Verlet entries (uid_i, uid_j, sx, sy, sz) of the last rebuild."""
        m = lib().lj_list_size(self._h)
        out = np.zeros(5 * max(m, 1), dtype=np.int32)
        k = lib().lj_list_pairs(self._h, out, m)
        return out[:5 * k].reshape(k, 5)

    def cell_counts(self):
        dims = np.zeros(3, dtype=np.int32)
        lib().lj_grid(self._h, dims)
        nc = int(np.prod(dims)) + 1
        sizes = np.zeros(nc, dtype=np.int32); loc = np.zeros(nc, dtype=np.int32)
        lib().lj_cell_counts(self._h, sizes, loc, nc)
        return dims, sizes, loc
