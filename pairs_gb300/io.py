"""Particle input and output formats of the reference.

read_particle_data  runtime/read_from_file.hpp:33-116: CSV, one particle per line,
                    fields in the declared property order; a vector property takes
                    3 fields, a matrix 9, a quaternion 4; a particle is kept when its
                    position is inside the domain (x >= min, x < max - 1e-5 per
                    dimension, regular_6d_stencil.cpp:96-100) or its flags mark it
                    infinite, fixed or global; its shape is set to `shape_id`.  With a
                    GPU the file's bytes go to the device and are indexed, parsed,
                    filtered and compacted there (pg_csv_parse, csrc/csv.cu);
                    parse_particle_csv is the host restatement it is tested against.
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


def _field_plan(props):
    """Per property its first field and width; the field kinds (PG_CSV_INT for the
    integer types, PG_CSV_REAL otherwise)."""
    from . import _capi as A
    plan, kinds, off = [], [], 0
    for p in props:
        w = _WIDTH.get(p.type, 1)
        plan.append((p, off, w))
        kinds += [A.PG_CSV_INT if p.type in (Types.Int32, Types.Int64, Types.UInt64) else A.PG_CSV_REAL] * w
        off += w
    return plan, kinds


def csv_table_device(data, kinds, pos_field=-1, flags_field=-1, lo=None, hi=None, device=None):
    """Parse CSV bytes on the GPU (pg_count_lines + pg_csv_parse): the kept rows as a
    float64 tensor [nfields, rows] on the device (integer fields as exact doubles).
    Raises PairsError for a malformed line (naming it) or a number outside the exact
    conversion range."""
    import torch
    from . import _capi as A
    lib = A.load()
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    raw = np.frombuffer(bytes(data), dtype=np.uint8)
    nbytes, nf = int(raw.size), len(kinds)
    text = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=dev)
    if nbytes:
        text[:nbytes].copy_(torch.from_numpy(raw.copy()).pin_memory())
    sh = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    cb = int(lib.pg_csv_count_bytes(nbytes))
    ws = torch.empty(max(cb, 16), dtype=torch.uint8, device=dev)
    lines = C.c_int64(0)
    A.call("pg_csv_count_lines", C.c_void_p(text.data_ptr()), nbytes, C.byref(lines),
           A.PgWorkspace(ws.data_ptr(), ws.numel()), sh)
    nl = int(lines.value)
    wb = int(lib.pg_csv_workspace_bytes(nbytes, nl, nf))
    if wb < 0:
        raise A.PairsError(f"CSV input: {nf} fields per line is more than the reader takes")
    ws = torch.empty(max(wb, 16), dtype=torch.uint8, device=dev)
    table = torch.empty((nf, max(nl, 1)), dtype=torch.float64, device=dev)
    kind_arr = (C.c_int32 * nf)(*kinds)
    dlo = (C.c_double * 3)(*lo) if lo is not None else None
    dhi = (C.c_double * 3)(*hi) if hi is not None else None
    res = A.PgCsvResult()
    rc = lib.pg_csv_parse(C.c_void_p(text.data_ptr()), nbytes, nl, nf, kind_arr, int(pos_field), int(flags_field),
                          dlo, dhi, C.c_void_p(table.data_ptr()), max(nl, 1), C.byref(res),
                          A.PgWorkspace(ws.data_ptr(), ws.numel()), sh)
    if res.bad_line >= 0:
        raise A.PairsError(f"CSV input: line {res.bad_line + 1} has a missing or malformed field")
    if res.inexact > 0:
        raise A.PairsError(f"CSV input: {res.inexact} numbers have more than 19 significant digits or a decimal "
                           "exponent beyond +-27 (outside the reader's exact conversion)")
    if rc != A.PG_OK:
        raise A.PairsError(f"pg_csv_parse failed: {rc}")
    return table[:, : res.rows]


def _kept_host(sim, props, lines):
    """The host restatement: per property the kept rows as numpy arrays."""
    cols = parse_particle_csv(lines, [p.type for p in props])
    n = 0 if not cols else len(cols[0])
    data = {p.name: np.array(cols[k]) for k, p in enumerate(props)}
    pos_name = sim.position_prop.name
    lo, hi = sim.grid if sim.grid is not None else ([-np.inf] * 3, [np.inf] * 3)
    pos = data[pos_name].reshape(n, 3)
    inside = np.ones(n, dtype=bool)
    for d in range(3):
        inside &= (pos[:, d] >= lo[d]) & (pos[:, d] < hi[d] - _SMALL)
    flags = data.get("flags", np.zeros(n, dtype=np.int64)).astype(np.int64)
    keep = inside | ((flags & (Flags.Infinite | Flags.Fixed | Flags.Global)) != 0)
    return {name: arr[keep] for name, arr in data.items()}


def _kept_device(sim, props, raw):
    """The device reader: per property the kept rows, parsed on the GPU."""
    plan, kinds = _field_plan(props)
    pos_name = sim.position_prop.name
    pos_field = next((off for p, off, w in plan if p.name == pos_name), -1)
    flags_field = next((off for p, off, w in plan if p.name == "flags"), -1)
    lo, hi = (sim.grid if sim.grid is not None else (None, None))
    table = csv_table_device(raw, kinds, pos_field, flags_field, lo, hi).cpu().numpy()
    out = {}
    for p, off, w in plan:
        col = table[off:off + w].T if w > 1 else table[off]
        out[p.name] = col.astype(np.int64) if kinds[off] == 1 else col
    return out


def read_particle_data(sim, filename, prop_names, shape_id, device=None):
    """State dict (pos, vel, mass, type, uid, flags, shape, and any other declared
    per-particle property by name) from a reference-format CSV file.  device: parse on
    the GPU (the default when one is present) or with the host restatement (False)."""
    props = [sim.property(p) for p in prop_names]
    if device is None:
        try:
            import torch
            device = torch.cuda.is_available()
        except ImportError:
            device = False
    if device:
        with open(filename, "rb") as f:
            out = _kept_device(sim, props, f.read())
    else:
        with open(filename) as f:
            out = _kept_host(sim, props, f.readlines())
    pos_name = sim.position_prop.name
    m = len(out[pos_name])

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
    state = dict(pos=np.asarray(out[pos_name], dtype=np.float64).reshape(m, 3),
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
