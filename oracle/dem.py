"""ctypes front end of the DEM oracle (oracle/dem_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/ and the CPU-baseline leg of bench.py,
never by the product package.
"""
import ctypes as C
import math
import os

import numpy as np

from . import build as _build

_lib = None
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(_build.build())
        L.dem_create.restype = C.c_void_p
        L.dem_create.argtypes = [C.c_int, _dp, _dp, _ip, C.c_double, C.c_double, C.c_double, C.c_double,
                                 C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, _dp, _dp,
                                 C.c_int, C.c_int]
        L.dem_destroy.argtypes = [C.c_void_p]
        L.dem_sc_grid.restype = C.c_int
        L.dem_sc_grid.argtypes = [C.c_void_p] + [C.c_double] * 9 + [C.c_int]
        L.dem_add_particle.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double, _dp, C.c_void_p,
                                       C.c_void_p, C.c_int, C.c_int]
        L.dem_setup.argtypes = [C.c_void_p]
        L.dem_step.restype = C.c_int
        L.dem_step.argtypes = [C.c_void_p]
        L.dem_nlocal.restype = C.c_int
        L.dem_nlocal.argtypes = [C.c_void_p]
        L.dem_get.argtypes = [C.c_void_p, C.c_int, _ip] + [C.c_void_p] * 7
        L.dem_get_initial.argtypes = [C.c_void_p] + [C.c_void_p] * 9
        L.dem_set_normal_stiffness.argtypes = [C.c_void_p, C.c_double]
        L.dem_contacts.restype = C.c_long
        L.dem_contacts.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_long]
        _lib = L
    return _lib


# the reference's DEM example parameters (examples/dem.py:100-127)
EXAMPLE = dict(diameter=0.0029, gravity=9.81, rho_f=1000.0, rho_p=2550.0, spacing=0.005, v0=1.0, dt=5e-5,
               mu=0.5, e=0.1, tc=5e-4, poisson=0.22)


def example_params(**over):
    p = dict(EXAMPLE, **over)
    p["kappa"] = 2.0 * (1.0 - p["poisson"]) / (2.0 - p["poisson"])
    p["ln_e"] = math.log(p["e"])
    p["cell"] = 1.01 * (p["diameter"] * 1.1)
    return p


class Sim:
    """The reference's DEM time loop on one rank (see dem_oracle.c header)."""

    def __init__(self, domain_size, planes, params=None, cap=None, history_fixed=False, ccap=20, spheres=None,
                 kn=0.0):
        """spheres: None for the example's dem_sc_grid, else a dict of arrays (uid,
        type, mass, radius, pos, vel) added in that order.  kn > 0: fixed normal
        stiffness (damping from the restitution coefficient)."""
        p = params or example_params()
        self.p = p
        lo = np.zeros(3)
        hi = np.asarray(domain_size, dtype=np.float64)
        cap = cap or max(200000, 2 * (len(spheres["pos"]) if spheres is not None else 0) + 1000)
        fs = np.zeros(1); fd = np.array([p["mu"]])
        self._h = lib().dem_create(cap, lo, hi, np.array([1, 1, 0], dtype=np.int32), p["cell"], p["dt"], math.pi,
                                   p["kappa"], p["ln_e"], p["tc"], p["rho_p"], p["rho_f"], p["gravity"], 1, fs, fd,
                                   ccap, int(history_fixed))
        if kn:
            lib().dem_set_normal_stiffness(self._h, float(kn))
        if spheres is None:
            d = p["diameter"]
            lib().dem_sc_grid(self._h, hi[0], hi[1], hi[2], p["spacing"], d, d * 0.9, d * 1.1, p["v0"], p["rho_p"],
                              1)
        else:
            for k in range(len(spheres["pos"])):
                pos = np.ascontiguousarray(spheres["pos"][k], dtype=np.float64)
                vel = np.ascontiguousarray(spheres["vel"][k], dtype=np.float64)
                lib().dem_add_particle(self._h, int(spheres["uid"][k]), int(spheres["type"][k]),
                                       float(spheres["mass"][k]), float(spheres["radius"][k]), pos, vel.ctypes.data,
                                       None, 0, 0)
        for pl in planes:
            uid, typ, mass = int(pl[0]), int(pl[1]), float(pl[2])
            pos = np.array(pl[3:6], dtype=np.float64)
            nrm = np.array(pl[6:9], dtype=np.float64)
            lib().dem_add_particle(self._h, uid, typ, mass, 0.0, pos, None, nrm.ctypes.data, int(pl[9]), 1)
        lib().dem_setup(self._h)
        self.ts = 0

    def __del__(self):
        if getattr(self, "_h", None):
            lib().dem_destroy(self._h)
            self._h = None

    def initial(self):
        n = lib().dem_nlocal(self._h)
        out = dict(uid=np.zeros(n, np.int32), type=np.zeros(n, np.int32), flags=np.zeros(n, np.int32),
                   shape=np.zeros(n, np.int32), mass=np.zeros(n), radius=np.zeros(n), pos=np.zeros((n, 3)),
                   vel=np.zeros((n, 3)), normal=np.zeros((n, 3)))
        lib().dem_get_initial(self._h, *[out[k].ctypes.data for k in
                                         ("uid", "type", "flags", "shape", "mass", "radius", "pos", "vel", "normal")])
        return out

    def step(self):
        rc = lib().dem_step(self._h)
        if rc:
            raise RuntimeError(f"DEM oracle overflow {rc}")
        self.ts += 1

    def run(self, n):
        for _ in range(n):
            self.step()

    def state(self, uids):
        uids = np.ascontiguousarray(uids, dtype=np.int32)
        n = len(uids)
        out = {k: np.zeros((n, 3)) for k in ("pos", "vel", "angvel", "force", "torque")}
        out["quat"] = np.zeros((n, 4))
        out["ncontacts"] = np.zeros(n, np.int32)
        lib().dem_get(self._h, n, uids, *[out[k].ctypes.data for k in
                                          ("pos", "vel", "angvel", "force", "torque", "quat", "ncontacts")])
        return out

    def contacts(self):
        m = 200000
        ids = np.zeros((m, 3), np.int32); vals = np.zeros((m, 4))
        k = lib().dem_contacts(self._h, ids.ctypes.data, vals.ctypes.data, m)
        return ids[:k], vals[:k]
