"""pg_bin_particles_noalloc against pg_bin_particles, through the C ABI.

The no-allocation entry point serves callers that cannot allocate device memory
while they bin (a host program with a fixed device-memory budget that forbids
allocations after start-up, or one that must not stall or fail on an allocation
inside its time loop).  It bins with a fixed scratch array inside the library
instead of a caller-made workspace, so its results must be those of the
workspace entry point.  Binning is integer work: the comparison is bit-exact.
The test runs two calls in a row on each entry point (new positions in between),
so a second call that read the first call's leftovers in the shared scratch would
show up.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from pairs_gb300 import _capi as A  # noqa: E402


def make_set(n, box, ncells_axis, seed, dev):
    """Particles (device tensors) and the structs describing them."""
    g = np.random.default_rng(seed)
    pos = np.zeros((n, 4))
    pos[:, :3] = g.uniform(0.0, box, size=(n, 3))
    pos[: n // 50, 0] += box * 1.01                # some left the periodic box
    vel = np.zeros((n, 4))
    vel[:, :3] = g.normal(size=(n, 3))
    t = dict(pos=torch.tensor(pos, device=dev), vel=torch.tensor(vel, device=dev),
             mass=torch.tensor(g.uniform(0.5, 2.0, n), device=dev),
             type=torch.tensor(g.integers(0, 3, n, dtype=np.int32), device=dev),
             uid=torch.tensor(g.permutation(n).astype(np.int32), device=dev),
             flags=torch.zeros(n, dtype=torch.int32, device=dev))
    ncells = ncells_axis ** 3
    t["cell_start"] = torch.zeros(ncells + 2, dtype=torch.int32, device=dev)
    t["cell_count"] = torch.zeros(ncells + 1, dtype=torch.int32, device=dev)
    t["particle_cell"] = torch.zeros(n, dtype=torch.int32, device=dev)
    t["status"] = torch.zeros(8, dtype=torch.int32, device=dev)
    p = A.PgParticles()
    p.n, p.capacity = n, n
    for name in ("pos", "vel", "mass", "type", "uid", "flags"):
        setattr(p, name, t[name].data_ptr())
    cells = A.PgCells()
    for d in range(3):
        cells.dims[d] = ncells_axis
        cells.cell_len[d] = box / ncells_axis
    cells.ncells = ncells
    cells.cell_start = t["cell_start"].data_ptr()
    cells.cell_count = t["cell_count"].data_ptr()
    cells.particle_cell = t["particle_cell"].data_ptr()
    bx = A.PgBox()
    for d in range(3):
        bx.lo[d], bx.hi[d], bx.len[d], bx.periodic[d] = 0.0, box, box, 1
    bx.quantum = 1.0
    return t, p, cells, bx


def host_recount(out, box, nc):
    """Cell of every binned particle recomputed on the host from its (wrapped)
    position: floor((x - lo) * (1 / cell_len)) per axis in FP64, clamped to the grid,
    exactly the kernel's arithmetic.  Returns (counts per cell, cell of each particle)."""
    inv = 1.0 / (box / nc)
    c = np.clip(np.floor((out["pos"][:, :3] - 0.0) * inv).astype(np.int64), 0, nc - 1)
    flat = (c[:, 0] * nc + c[:, 1]) * nc + c[:, 2]
    return np.bincount(flat, minlength=nc ** 3), flat


def outputs(t):
    return {k: t[k].cpu().numpy().copy() for k in
            ("pos", "vel", "mass", "type", "uid", "flags", "cell_start", "cell_count", "particle_cell")}


def test_no_alloc_binning_matches_workspace_binning():
    lib = A.load()
    dev = torch.device("cuda")
    n, box, nc = 100000, 30.0, 12
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    ref_t, ref_p, ref_c, bx = make_set(n, box, nc, 1, dev)
    new_t, new_p, new_c, _ = make_set(n, box, nc, 1, dev)
    wsb = lib.pg_workspace_bytes(n, nc ** 3)
    ws_t = torch.empty(int(wsb), dtype=torch.uint8, device=dev)
    ws = A.PgWorkspace(ws_t.data_ptr(), int(wsb))
    for call in range(2):
        if call == 1:
            # new positions (same on both sides) for the second call in a row
            g = np.random.default_rng(7)
            shift = torch.tensor(g.uniform(-2.0, 2.0, size=(n, 3)), device=dev)
            for t in (ref_t, new_t):
                t["pos"][:, :3] += shift
        rc = lib.pg_bin_particles(C.byref(bx), C.byref(ref_p), C.byref(ref_c), ws,
                                  C.c_void_p(ref_t["status"].data_ptr()), stream)
        assert rc == A.PG_OK
        rc = lib.pg_bin_particles_noalloc(C.byref(bx), C.byref(new_p), C.byref(new_c),
                                          C.c_void_p(new_t["status"].data_ptr()), stream)
        assert rc == A.PG_OK
        torch.cuda.synchronize()
        a, b = outputs(ref_t), outputs(new_t)
        for k in a:
            assert np.array_equal(a[k], b[k]), (call, k)
        # both entry points share their kernels, so the cells are also checked against
        # an independent count on the host
        counts, flat = host_recount(b, box, nc)
        assert np.array_equal(b["cell_count"][: nc ** 3], counts), call
        assert b["cell_count"][nc ** 3] == 0, call              # no particle parked in the extra bucket
        assert np.array_equal(b["cell_start"][: nc ** 3 + 1], np.concatenate([[0], np.cumsum(counts)])), call
        assert np.array_equal(b["particle_cell"], flat), call
        assert np.all(np.diff(flat) >= 0), call                 # particles stored in cell order
        assert np.array_equal(ref_t["status"].cpu().numpy(), new_t["status"].cpu().numpy())


def test_no_alloc_rejects_inputs_beyond_its_scratch():
    lib = A.load()
    p = A.PgParticles()
    p.n = p.capacity = A.NOALLOC_MAX_PARTICLES + 1
    cells = A.PgCells()
    cells.dims[0] = cells.dims[1] = cells.dims[2] = 4
    cells.cell_len[0] = cells.cell_len[1] = cells.cell_len[2] = 1.0
    cells.ncells = 64
    bx = A.PgBox()
    st = torch.zeros(8, dtype=torch.int32, device="cuda")
    # rejected before any device work: no pointers are dereferenced
    assert lib.pg_bin_particles_noalloc(C.byref(bx), C.byref(p), C.byref(cells), C.c_void_p(st.data_ptr()),
                                        None) == A.PG_ERR_LIMIT
    p.n = p.capacity = 10
    cells.dims[0] = cells.dims[1] = cells.dims[2] = 41
    cells.ncells = 41 ** 3
    assert cells.ncells > A.NOALLOC_MAX_CELLS
    assert lib.pg_bin_particles_noalloc(C.byref(bx), C.byref(p), C.byref(cells), C.c_void_p(st.data_ptr()),
                                        None) == A.PG_ERR_LIMIT
