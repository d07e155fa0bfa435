"""Reader for the dumps written by oracle/ref_hooks.hpp (test infrastructure)."""
import glob
import os

import numpy as np


class _Reader:
    def __init__(self, path):
        with open(path, "rb") as f:
            self.buf = f.read()
        self.off = 0

    def i32(self, n=None):
        cnt = 1 if n is None else n
        a = np.frombuffer(self.buf, dtype="<i4", count=cnt, offset=self.off)
        self.off += 4 * cnt
        return int(a[0]) if n is None else a.copy()

    def f64(self, n):
        a = np.frombuffer(self.buf, dtype="<f8", count=n, offset=self.off)
        self.off += 8 * n
        return a.copy()


def read_init(dump_dir):
    r = _Reader(os.path.join(dump_dir, "init.bin"))
    n = r.i32()
    return dict(n=n, uid=r.i32(n), type=r.i32(n), flags=r.i32(n), mass=r.f64(n),
                position=r.f64(3 * n).reshape(n, 3), velocity=r.f64(3 * n).reshape(n, 3))


def read_step(path):
    r = _Reader(path)
    ts, rebuilt, nlocal, nghost = r.i32(), r.i32(), r.i32(), r.i32()
    uid = r.i32(nlocal)
    out = dict(ts=ts, rebuilt=bool(rebuilt), nlocal=nlocal, nghost=nghost, uid=uid,
               position=r.f64(3 * nlocal).reshape(nlocal, 3),
               velocity=r.f64(3 * nlocal).reshape(nlocal, 3),
               force=r.f64(3 * nlocal).reshape(nlocal, 3))
    npairs = r.i32()
    if npairs >= 0:
        out["pairs"] = r.i32(5 * npairs).reshape(npairs, 5)
        ncells = r.i32()
        out["cell_sizes"] = r.i32(ncells)
        out["cell_local_counts"] = r.i32(ncells)
    return out


def by_uid(step):
    """Return a copy of the per-particle arrays permuted into uid order."""
    order = np.argsort(step["uid"], kind="stable")
    res = dict(step)
    for k in ("uid", "position", "velocity", "force"):
        res[k] = step[k][order]
    return res


def read_all(dump_dir):
    steps = {}
    for p in sorted(glob.glob(os.path.join(dump_dir, "step_*.bin"))):
        s = read_step(p)
        steps[s["ts"]] = s
    return read_init(dump_dir), steps


def read_dem_init(dump_dir):
    r = _Reader(os.path.join(dump_dir, "init.bin"))
    n = r.i32()
    return dict(n=n, uid=r.i32(n), type=r.i32(n), flags=r.i32(n), shape=r.i32(n), mass=r.f64(n), radius=r.f64(n),
                pos=r.f64(3 * n).reshape(n, 3), vel=r.f64(3 * n).reshape(n, 3), normal=r.f64(3 * n).reshape(n, 3))


def read_dem_step(path):
    r = _Reader(path)
    ts, n = r.i32(), r.i32()
    uid = r.i32(n)
    out = dict(ts=ts, n=n, uid=uid, pos=r.f64(3 * n).reshape(n, 3), vel=r.f64(3 * n).reshape(n, 3),
               angvel=r.f64(3 * n).reshape(n, 3), force=r.f64(3 * n).reshape(n, 3),
               torque=r.f64(3 * n).reshape(n, 3), quat=r.f64(4 * n).reshape(n, 4))
    m = r.i32()
    out["contact_ids"] = r.i32(3 * m).reshape(m, 3)
    out["contact_vals"] = r.f64(4 * m).reshape(m, 4)
    return out


def dem_by_uid(step):
    order = np.argsort(step["uid"], kind="stable")
    res = dict(step)
    for k in ("uid", "pos", "vel", "angvel", "force", "torque", "quat"):
        res[k] = step[k][order]
    return res


def read_dem_all(dump_dir):
    steps = {}
    for p in sorted(glob.glob(os.path.join(dump_dir, "step_*.bin"))):
        s = read_dem_step(p)
        steps[s["ts"]] = s
    return read_dem_init(dump_dir), steps
