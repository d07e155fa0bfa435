"""Generate the golden fixtures under tests/golden/ from the reference itself.

Needs the reference source tree (PAIRS_REFERENCE, default: a checkout named
"reference" beside this repository) and g++:
for each configuration it runs oracle/ref_build.py (generate the reference's CPU
program, insert the dump hooks, compile), runs the program, and stores a compact
record of its output:

  thermo        the "T<TAB>P" lines the program prints (runtime/thermo.hpp:45-46)
  init_*        initial state in creation order (uid = creation index)
  step<ts>_*    positions, velocities, forces in uid order at selected steps
  pairs<ts>     full Verlet entries (uid_i, uid_j, sx, sy, sz) where stored
  pairs_sha     SHA-256 of every rebuild's canonically sorted entries
  cells<ts>     reference grid occupancy (locals+ghosts, locals only)

The fixtures let the CPU tests pin the oracle without the reference present.
Usage: python tests/golden/make_golden.py [names...]
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref_build, ref_dump  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

# which steps keep full per-particle arrays / full pair lists
KEEP = {
    "lj4": dict(steps=[0, 1, 2, 5, 18, 19, 20, 21, 50, 99, 100], pairs=[0, 19]),
    "lj4_half": dict(steps=[0, 1, 19, 20, 100], pairs=[0]),
    "lj4_t4": dict(steps=[0, 1, 100], pairs=[]),
    "lj8": dict(steps=[1, 100], pairs=[]),
    "lj6x5x4": dict(steps=[0, 1, 10, 11, 60], pairs=[]),
    "custom6": dict(steps=[0, 1, 9, 10, 11, 30, 60], pairs=[]),
    "custom6_half": dict(steps=[0, 1, 10, 60], pairs=[]),
    "custom_wca": dict(steps=[0, 1, 7, 8, 9, 20, 40], pairs=[]),
}


def canonical_pairs(p):
    """Sort Verlet entries (uid_i, uid_j, sx, sy, sz) lexicographically."""
    p = np.asarray(p, dtype=np.int32).reshape(-1, 5)
    order = np.lexsort(p.T[::-1])
    return np.ascontiguousarray(p[order])


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def make(name):
    exe, cfg = ref_build.build(name)
    dump = os.path.join(ref_build.OUT, name, "dump")
    stdout = ref_build.run(exe, dump)
    thermo = [l for l in stdout.splitlines() if "\t" in l and ":" not in l]
    init, steps = ref_dump.read_all(dump)
    keep = KEEP[name]
    rec = {
        "cfg": np.array(json.dumps({k: v for k, v in cfg.items() if not k.startswith("_")})),
        "thermo": np.array(thermo),
        "init_pos": init["position"], "init_vel": init["velocity"],
        "init_type": init["type"].astype(np.int8), "init_mass": init["mass"],
    }
    shas, rebuild_steps = [], []
    for ts in sorted(steps):
        s = ref_dump.by_uid(steps[ts])
        if ts in keep["steps"]:
            rec[f"step{ts}_pos"] = s["position"]
            rec[f"step{ts}_vel"] = s["velocity"]
            rec[f"step{ts}_force"] = s["force"]
        if s["rebuilt"]:
            cp = canonical_pairs(s["pairs"])
            rebuild_steps.append(ts)
            shas.append(sha(cp))
            rec[f"nghost{ts}"] = np.array(s["nghost"])
            rec[f"cells{ts}"] = np.stack([s["cell_sizes"], s["cell_local_counts"]]).astype(np.int16)
            if ts in keep["pairs"]:
                rec[f"pairs{ts}"] = np.concatenate(
                    [cp[:, :2].astype(np.int16).view(np.int8).reshape(-1, 4), cp[:, 2:].astype(np.int8)],
                    axis=1)
    rec["rebuild_steps"] = np.array(rebuild_steps)
    rec["pairs_sha"] = np.array(shas)
    path = os.path.join(OUT, name + ".npz")
    np.savez_compressed(path, **rec)
    print(name, os.path.getsize(path), "bytes")


DEM_KEEP = {
    "dem_small": [0, 1, 100, 150, 300],
    "dem_dense": [0, 1, 50, 150, 300],
}


def make_dem(name):
    exe, cfg = ref_build.build(name)
    dump = os.path.join(ref_build.OUT, name, "dump")
    ref_build.run(exe, dump)
    init, steps = ref_dump.read_dem_all(dump)
    rec = {"cfg": np.array(json.dumps({k: v for k, v in cfg.items() if not k.startswith("_")}))}
    for k in ("uid", "type", "flags", "shape", "mass", "radius", "pos", "vel", "normal"):
        rec["init_" + k] = init[k]
    for ts in DEM_KEEP[name]:
        s = ref_dump.dem_by_uid(steps[ts])
        for k in ("uid", "pos", "vel", "angvel", "force", "torque", "quat"):
            rec[f"step{ts}_{k}"] = s[k]
        ids, vals = s["contact_ids"], s["contact_vals"]
        order = np.lexsort((ids[:, 1], ids[:, 0]))
        rec[f"step{ts}_contact_ids"] = ids[order]
        rec[f"step{ts}_contact_vals"] = vals[order]
    rec["ncontacts"] = np.array([len(steps[t]["contact_ids"]) for t in sorted(steps)])
    path = os.path.join(OUT, name + ".npz")
    np.savez_compressed(path, **rec)
    print(name, os.path.getsize(path), "bytes")


def unpack_pairs(packed):
    """Inverse of the compact pair encoding used above."""
    ij = packed[:, :4].copy().view(np.int16).astype(np.int32)
    return np.concatenate([ij, packed[:, 4:].astype(np.int32)], axis=1)


if __name__ == "__main__":
    for n in (sys.argv[1:] or list(KEEP) + list(DEM_KEEP)):
        (make_dem if n in DEM_KEEP else make)(n)
