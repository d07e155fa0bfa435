"""Particle input and output formats of the reference.

read_particle_data  runtime/read_from_file.hpp:121-203: CSV, one particle per line,
                    fields in the declared property order; a vector property takes
                    3 fields, a matrix 9, a quaternion 4; a particle is kept when its
                    position is inside the domain (x >= min, x < max - 1e-5 per
                    dimension, regular_6d_stencil.cpp:96-100) or its flags mark it
                    infinite, fixed or global; its shape is set to `shape_id`.
write_vtk           runtime/vtk.hpp:11-86: legacy VTK ASCII unstructured grid of the
                    positions (vertices) with the mass as point data, 8 decimals,
                    infinite particles left out, file <name>_<timestep>.vtk.  The rows
                    are formatted on the device (pg_vtk_format_rows / pg_vtk_pack_rows)
                    and only the text comes back; format_vtk is the host restatement
                    the device text is tested against.
"""
import ctypes as C

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
    """Legacy VTK text of the particles (vtk.hpp:11-86 layout): infinite particles left
    out, CELLS rows "1 i" with i the particle's index among all particles
    (vtk.hpp:57-60 writes i - start, so an infinite particle leaves a gap)."""
    keep = np.ones(len(pos), dtype=bool) if flags is None else (np.asarray(flags) & Flags.Infinite) == 0
    p = np.asarray(pos)[keep]
    m = np.asarray(mass)[keep]
    idx = np.nonzero(keep)[0]
    n = len(p)
    out = ["# vtk DataFile Version 2.0\n", "Particle data\n", "ASCII\n", "DATASET UNSTRUCTURED_GRID\n",
           f"POINTS {n} double\n"]
    out += ["%.8f %.8f %.8f\n" % tuple(r) for r in p]
    out.append("\n\n")
    out.append(f"CELLS {n} {n * 2}\n")
    out += [f"1 {k}\n" for k in idx]
    out.append("\n\n")
    out.append(f"CELL_TYPES {n}\n")
    out += ["1\n"] * n
    out.append("\n\n")
    out += [f"POINT_DATA {n}\n", "SCALARS mass double\n", "LOOKUP_TABLE default\n"]
    out += ["%.8f\n" % v for v in m]
    out.append("\n\n")
    return "".join(out)


def device_vtk_text(pos, mass, flags=None, uid=None):
    """The text of format_vtk, formatted on the device from device tensors: pos
    (n x 4 FP64), mass (n, FP64), flags (n, int32; infinite particles left out) and
    uid (n, int32; rows in uid order, as the host arrays of engine.state()).  One
    thread formats one row into a fixed-width slot, a scan of the row lengths gives
    the offsets and a second kernel packs the rows; the host adds the header lines.
    Returns bytes; raises PairsError for a value that %.8f cannot hold (|x| >= 9.2e10,
    NaN, infinity)."""
    import torch
    from . import _capi as A
    lib = A.load()
    dev = pos.device
    n = pos.shape[0]
    order = torch.argsort(uid.long(), stable=True) if uid is not None else torch.arange(n, device=dev)
    index = torch.arange(n, dtype=torch.int32, device=dev)     # row k's index among all particles
    if flags is not None:
        keep = (flags[order] & int(Flags.Infinite)) == 0
        order, index = order[keep], index[keep]
    order = order.to(torch.int32).contiguous()
    index = index.contiguous()
    rows = int(order.numel())
    pos, mass = pos.contiguous(), mass.to(torch.float64).contiguous()
    wsb = int(lib.pg_vtk_workspace_bytes(rows))
    ws = torch.empty(max(wsb, 16), dtype=torch.uint8, device=dev)
    w = A.PgWorkspace(ws.data_ptr(), ws.numel())
    lens = ws[wsb - 4 * rows: wsb].view(torch.int32)    # the row lengths end the workspace
    sh = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    ptr = lambda x: C.c_void_p(x.data_ptr())

    def section(what):
        if rows == 0:
            return b""
        A.call("pg_vtk_format_rows", what, rows, ptr(order), ptr(pos), ptr(mass), ptr(index), w, sh)
        ln = lens.to(torch.int64)
        if bool((ln < 0).any()):
            raise A.PairsError("VTK output: a position or mass outside the range of %.8f")
        off = torch.cumsum(ln, 0) - ln
        total = int(ln.sum())
        out = torch.empty(total, dtype=torch.uint8, device=dev)
        A.call("pg_vtk_pack_rows", rows, w, ptr(off), ptr(out), sh)
        return out.cpu().numpy().tobytes()

    head = (b"# vtk DataFile Version 2.0\nParticle data\nASCII\nDATASET UNSTRUCTURED_GRID\n"
            + f"POINTS {rows} double\n".encode())
    parts = [head, section(0), b"\n\n", f"CELLS {rows} {rows * 2}\n".encode(), section(1), b"\n\n",
             f"CELL_TYPES {rows}\n".encode(), b"1\n" * rows, b"\n\n",
             f"POINT_DATA {rows}\nSCALARS mass double\nLOOKUP_TABLE default\n".encode(), section(2), b"\n\n"]
    return b"".join(parts)


def write_vtk(sim, engine, timestep):
    """<file>_local_<timestep>.vtk, the reference's file of the local particles
    (sim/vtk.py:20).  Its second file, <file>_ghost_<timestep>.vtk, lists the copies its
    border exchange made; this engine makes none (periodic images are formed inside the
    pair kernels), so that file is not written."""
    pos, mass, flags, uid = engine.vtk_fields()
    with open(f"{sim.vtk_file}_local_{timestep}.vtk", "wb") as f:
        f.write(device_vtk_text(pos, mass, flags, uid))
