"""Particle input and output formats of the reference.

read_particle_data  runtime/read_from_file.hpp:121-203: CSV, one particle per line,
                    fields in the declared property order; a vector property takes
                    3 fields, a matrix 9, a quaternion 4; a particle is kept when its
                    position is inside the domain (x >= min, x < max - 1e-5 per
                    dimension, regular_6d_stencil.cpp:96-100) or its flags mark it
                    infinite, fixed or global; its shape is set to `shape_id`.
write_vtk           runtime/vtk.hpp:11-86: legacy VTK ASCII unstructured grid of the
                    positions (vertices) with the mass as point data, 8 decimals,
                    infinite particles left out, file <name>_<timestep>.vtk.
"""
import numpy as np

from .types import Flags, Types

_SMALL = 0.00001
_WIDTH = {Types.Vector: 3, Types.Matrix: 9, Types.Quaternion: 4}


def parse_particle_csv(lines, prop_types):
    """Parse CSV lines into per-property lists (numbers as float, ints as int)."""
    cols = {k: [] for k in range(len(prop_types))}
    for line in lines:
        line = line.strip()
        if not line:
            continue
        fields = line.split(",")
        off = 0
        for k, t in enumerate(prop_types):
            w = _WIDTH.get(t, 1)
            vals = fields[off:off + w]
            if len(vals) != w:
                raise ValueError(f"particle line has too few fields: {line!r}")
            if t in (Types.Int32, Types.Int64, Types.UInt64):
                cols[k].append(int(vals[0]))
            else:
                cols[k].append([float(v) for v in vals] if w > 1 else float(vals[0]))
            off += w
    return cols


def read_particle_data(sim, filename, prop_names, shape_id):
    """State dict (pos, vel, mass, type, uid, flags, shape, and any other declared
    per-particle property by name) from a reference-format CSV file."""
    with open(filename) as f:
        lines = f.readlines()
    props = [sim.property(p) for p in prop_names]
    cols = parse_particle_csv(lines, [p.type for p in props])
    n = len(lines) if not cols else len(cols[0])
    data = {p.name: np.array(cols[k]) for k, p in enumerate(props)}
    pos_name = sim.position_prop.name
    lo, hi = sim.grid if sim.grid is not None else ([-np.inf] * 3, [np.inf] * 3)
    pos = data[pos_name].reshape(n, 3)
    inside = np.ones(n, dtype=bool)
    for d in range(3):
        inside &= (pos[:, d] >= lo[d]) & (pos[:, d] < hi[d] - _SMALL)
    flags = data.get("flags", np.zeros(n, dtype=np.int64)).astype(np.int64)
    keep = inside | ((flags & (Flags.Infinite | Flags.Fixed | Flags.Global)) != 0)
    out = {}
    for name, arr in data.items():
        out[name] = arr[keep]
    m = int(keep.sum())

    def get(name, default):
        if name in out:
            return out[name]
        prop = sim.property(name)
        val = prop.value if prop is not None else default
        if isinstance(val, (list, tuple)):
            return np.tile(np.asarray(val, dtype=np.float64), (m, 1))
        width = _WIDTH.get(prop.type, 1) if prop is not None else 1
        # a scalar default of a vector/matrix property fills every component
        return np.full((m,) if width == 1 else (m, width), val, dtype=np.float64)

    vel_name = "linear_velocity"
    state = dict(pos=out[pos_name].reshape(m, 3).astype(np.float64),
                 vel=np.asarray(get(vel_name, 0.0), dtype=np.float64).reshape(m, 3) if vel_name in sim.properties
                 else np.zeros((m, 3)),
                 mass=np.asarray(get("mass", 1.0), dtype=np.float64).reshape(m),
                 type=np.asarray(out.get("type", np.zeros(m)), dtype=np.int32),
                 uid=np.asarray(out["uid"], dtype=np.int32) if "uid" in out else np.arange(m, dtype=np.int32),
                 flags=np.asarray(out.get("flags", np.zeros(m)), dtype=np.int32),
                 shape=np.full(m, shape_id, dtype=np.int32))
    for name, arr in out.items():
        if name not in (pos_name, vel_name, "mass", "type", "uid", "flags"):
            state[name] = arr
    return state


def format_vtk(pos, mass, flags=None):
    """Legacy VTK text of the particles (vtk.hpp:11-86 layout)."""
    keep = np.ones(len(pos), dtype=bool) if flags is None else (np.asarray(flags) & Flags.Infinite) == 0
    p = np.asarray(pos)[keep]
    m = np.asarray(mass)[keep]
    n = len(p)
    out = ["# vtk DataFile Version 2.0\n", "Particle data\n", "ASCII\n", "DATASET UNSTRUCTURED_GRID\n",
           f"POINTS {n} double\n"]
    out += ["%.8f %.8f %.8f\n" % tuple(r) for r in p]
    out.append("\n\n")
    out.append(f"CELLS {n} {n * 2}\n")
    out += [f"1 {k}\n" for k in range(n)]
    out.append("\n\n")
    out.append(f"CELL_TYPES {n}\n")
    out += ["1\n"] * n
    out.append("\n\n")
    out += [f"POINT_DATA {n}\n", "SCALARS mass double\n", "LOOKUP_TABLE default\n"]
    out += ["%.8f\n" % v for v in m]
    out.append("\n\n")
    return "".join(out)


def write_vtk(sim, engine, timestep):
    st = engine.state()
    if isinstance(st, dict):                      # DEM engine: arrays by name
        pos, mass, flags = st["pos"], st["mass"], st["flags"]
    else:
        pos, mass, flags = st[0], engine.masses(), engine.flags()
    with open(f"{sim.vtk_file}_{timestep}.vtk", "w") as f:
        f.write(format_vtk(pos, mass, flags))
