"""Cell binning, list-count publication and the near-cutoff queue on the GPU.

* Binning counts are integer work and are compared bit-exactly:
  - on the reference's own cell geometry (origin one spacing below the domain,
    cells of r_list, ceil((L + 2 r_list) / r_list) + 1 per axis,
    src/pairs/sim/cell_lists.py:46-134), the GPU's per-cell counts of the local
    particles equal the reference's (golden fixtures) and the oracle's (32^3);
  - on the engine's own grid, cell_count, cell_start and particle_cell equal a host
    recount of the wrapped positions with the kernel's FP64 arithmetic.
* The list builds publish the largest per-particle count; with a particle count that
  is not a multiple of 32 (warps with exited lanes) it still equals the host maximum
  of the stored counts (LJ, DEM, ensemble).
* The mixed path's queue of near-cutoff pairs may overflow a small workspace; the
  fixup pass then walks every list again and the forces equal those of a large queue
  to FP32 summation order.
"""
import ctypes as C
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import lj as olj  # noqa: E402
from pairs_gb300 import _capi as A  # noqa: E402
from pairs_gb300 import lattice  # noqa: E402

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
R_LIST = 2.5 + 0.3


def bin_on_gpu(pos, lo, cell_len, dims, periodic=(False, False, False), hi=None):
    """pg_bin_particles through the C ABI on host positions (n x 3).  Returns the
    per-cell counts (ncells + trailing bucket), cell starts, the cell of each sorted
    particle and the sorted (wrapped) positions."""
    lib = A.load()
    dev = torch.device("cuda")
    n = len(pos)
    p4 = np.zeros((n, 4))
    p4[:, :3] = pos
    ncells = int(np.prod(dims))
    t = dict(pos=torch.tensor(p4, device=dev), uid=torch.arange(n, dtype=torch.int32, device=dev),
             cell_start=torch.zeros(ncells + 2, dtype=torch.int32, device=dev),
             cell_count=torch.zeros(ncells + 1, dtype=torch.int32, device=dev),
             particle_cell=torch.zeros(n, dtype=torch.int32, device=dev),
             status=torch.zeros(8, dtype=torch.int32, device=dev))
    p = A.PgParticles()
    p.n = p.capacity = n
    p.pos, p.uid = t["pos"].data_ptr(), t["uid"].data_ptr()
    cells = A.PgCells()
    for d in range(3):
        cells.dims[d] = int(dims[d])
        cells.cell_len[d] = float(cell_len[d])
    cells.ncells = ncells
    cells.cell_start, cells.cell_count = t["cell_start"].data_ptr(), t["cell_count"].data_ptr()
    cells.particle_cell = t["particle_cell"].data_ptr()
    bx = A.PgBox()
    hi = hi if hi is not None else [lo[d] + cell_len[d] * dims[d] for d in range(3)]
    for d in range(3):
        bx.lo[d], bx.hi[d], bx.len[d], bx.periodic[d] = lo[d], hi[d], hi[d] - lo[d], int(periodic[d])
    bx.quantum = 1.0
    wsb = int(lib.pg_workspace_bytes(n, ncells))
    ws_t = torch.empty(wsb, dtype=torch.uint8, device=dev)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.pg_bin_particles(C.byref(bx), C.byref(p), C.byref(cells), A.PgWorkspace(ws_t.data_ptr(), wsb),
                              C.c_void_p(t["status"].data_ptr()), stream)
    assert rc == A.PG_OK
    torch.cuda.synchronize()
    return (t["cell_count"].cpu().numpy(), t["cell_start"].cpu().numpy(), t["particle_cell"].cpu().numpy(),
            t["pos"].cpu().numpy()[:, :3])


def reference_grid(box):
    """The reference's cell grid for a domain [0, L) (sim/cell_lists.py:67-76): origin
    0 - spacing, cells of the spacing, ceil((L + 2 s) / s) + 1 per axis."""
    s = R_LIST
    lo = [0.0 - s] * 3
    dims = [int(np.ceil(((box[d] + s) - (0.0 - s)) / s)) + 1 for d in range(3)]
    return lo, [s] * 3, dims


def check_reference_counts(pos, box, local_counts):
    """GPU counts on the reference geometry against the reference's local counts
    (its flat index is the cell's index + 1: cell 0 is its extra cell)."""
    lo, cl, dims = reference_grid(box)
    counts, start, pcell, _ = bin_on_gpu(pos, lo, cl, dims)
    nc = int(np.prod(dims))
    assert len(local_counts) == nc + 1
    assert local_counts[0] == 0
    assert np.array_equal(counts[:nc], local_counts[1:].astype(np.int32))
    assert counts[nc] == 0
    assert np.array_equal(start[: nc + 1], np.concatenate([[0], np.cumsum(counts[:nc])]))


@pytest.mark.parametrize("name,ts", [("lj4", 0), ("lj4", 19), ("lj8", 0), ("lj6x5x4", 0), ("lj4_half", 19)])
def test_cell_counts_bit_exact_against_reference_fixtures(name, ts):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    cfg = json.loads(str(g["cfg"]))
    pos = g["init_pos"] if ts == 0 else g[f"step{ts}_pos"]
    box = olj.fcc_box(*cfg["n"])
    check_reference_counts(pos, box, g[f"cells{ts}"][1])


def test_cell_counts_bit_exact_against_oracle_at_32cube():
    """fcc 32^3 (131,072 atoms) after the rebuild of step 19 of the reference's loop:
    the oracle's cell counts (pinned to the reference's generated program) against the
    GPU's on the same positions and geometry."""
    st = olj.fcc_lattice(32, 32, 32)
    sim = olj.Sim(st, every=20, nthreads=os.cpu_count() or 1)
    sim.run(20)
    dims, _, loc = sim.cell_counts()
    lo, cl, rdims = reference_grid(st["box"])
    assert list(dims) == rdims
    pos, _, _ = sim.state()
    check_reference_counts(pos, st["box"], loc)


@pytest.mark.parametrize("cube,half", [(4, False), (8, False), (8, True), (32, False), (32, True)])
def test_engine_grid_matches_host_recount(cube, half):
    """The engine's own grid (cells of at least r_list, half-width in x for half
    lists) after a liquid run and a rebuild: counts, starts and per-particle cells
    equal a host recount of the binned, wrapped positions."""
    from pairs_gb300.engine import LJEngine
    st = lattice.copper_fcc_lattice(cube, cube, cube)
    eng = LJEngine(st, precision="mixed" if cube > 4 else "fp64", half=half, sync="exact", policy="guard")
    eng.run(30)
    eng.settle()
    eng.rebuild()
    torch.cuda.synchronize()
    n = eng.n
    dims = [eng.cells.dims[d] for d in range(3)]
    inv = [1.0 / eng.cells.cell_len[d] for d in range(3)]
    lo = [eng.box.lo[d] for d in range(3)]
    pos = eng.t["pos"][:n, :3].cpu().numpy()
    assert np.all(pos >= np.array(lo)) and np.all(pos <= np.array([eng.box.hi[d] for d in range(3)]))
    c = np.stack([np.clip(np.floor((pos[:, d] - lo[d]) * inv[d]).astype(np.int64), 0, dims[d] - 1)
                  for d in range(3)], axis=1)
    flat = (c[:, 0] * dims[1] + c[:, 1]) * dims[2] + c[:, 2]
    nc = eng.cells.ncells
    counts = np.bincount(flat, minlength=nc)
    assert np.array_equal(eng.t["cell_count"][:nc].cpu().numpy(), counts)
    assert eng.t["cell_count"][nc].item() == 0
    assert np.array_equal(eng.t["cell_start"][: nc + 1].cpu().numpy(), np.concatenate([[0], np.cumsum(counts)]))
    assert np.array_equal(eng.t["particle_cell"][:n].cpu().numpy(), flat)
    # within a cell by z, then uid: every z column of cells is sorted by z
    uid = eng.t["uid"][:n].cpu().numpy()
    same = flat[1:] == flat[:-1]
    z = pos[:, 2]
    assert np.all((z[1:][same] > z[:-1][same]) | ((z[1:][same] == z[:-1][same]) & (uid[1:][same] > uid[:-1][same])))
    column = flat // dims[2]
    run = column[1:] == column[:-1]
    assert np.all(z[1:][run] >= z[:-1][run])


@pytest.mark.parametrize("half,precision", [(False, "fp64"), (True, "mixed"), (False, "mixed")])
def test_lj_list_publishes_max_count_with_partial_warps(half, precision):
    """fcc 7^3 = 1372 atoms (1372 = 42 * 32 + 28: the last warp has 4 exited lanes)."""
    from pairs_gb300.engine import LJEngine
    st = lattice.copper_fcc_lattice(7, 7, 7)
    assert len(st["mass"]) % 32 != 0
    eng = LJEngine(st, precision=precision, half=half, sync="exact", policy="guard")
    eng.run(20)
    eng.settle()
    eng.rebuild()
    s = eng.read_status()
    cnt = eng.list_counts()
    assert s.max_neighbors == cnt.max()
    assert s.overflow == 0


def test_ensemble_list_publishes_max_count_with_partial_warps():
    from pairs_gb300.ensemble import Ensemble
    reps = [lattice.trimmed_fcc(natoms=n, rho=0.8, temperature=1.0) for n in (501, 733, 1291)]
    total = sum(len(r["mass"]) for r in reps)
    assert total % 32 != 0
    ens = Ensemble(reps, tpa=2, reach=1, policy="every", half=True)
    ens.rebuild()
    s = ens.read_status()
    ens.synchronize()
    cnt = ens.t["count"][:total].cpu().numpy()
    assert s.max_neighbors == cnt.max()


def test_dem_list_publishes_max_count_with_partial_warps():
    from tests.test_gpu_dem import engine_from_oracle, golden_cfg, oracle_sim
    cfg = golden_cfg("dem_dense")
    sim, p = oracle_sim(cfg)
    sim.run(100)
    eng = engine_from_oracle(sim, p, cfg, policy="every")
    assert eng.n % 32 != 0
    eng.rebuild()
    s = eng.read_status()
    cnt = eng.t["count"][: eng.n].cpu().numpy()
    assert s.max_neighbors == cnt.max()


@pytest.mark.parametrize("half", [False, True])
def test_near_cutoff_queue_overflow_loses_no_force(half):
    """A one-record queue (the smallest workspace pg_lj_force accepts) overflows on a
    liquid of 16384 atoms (about 28 pairs in the band with a full list, 14 with a
    half list): the fixup pass walks every list
    again and the forces and energy equal those computed with the engine's large
    queue, to FP32 summation order."""
    from pairs_gb300.engine import LJEngine
    lib = A.load()
    st = lattice.copper_fcc_lattice(16, 16, 16)
    eng = LJEngine(st, precision="mixed", half=half, sync="exact", policy="guard")
    eng.run(40)
    eng.settle()
    eng.rebuild()
    eng.p.step = eng.device_step(eng.ts)
    eng.force(energy=True)
    torch.cuda.synchronize()
    queued = int(eng.t["ws"][:4].view(torch.int32).item())
    ref_f = eng.t["force32"][: eng.n, :3].cpu().numpy().astype(np.float64)
    ref_e = eng.t["energy"].cpu().numpy().copy()
    assert queued >= 2                                    # the small queue will overflow
    small = torch.zeros(256 + 8, dtype=torch.uint8, device=eng.dev)
    ws = A.PgWorkspace(small.data_ptr(), small.numel())
    rc = lib.pg_lj_force(C.byref(eng.box), C.byref(eng.p), C.byref(eng.cells), C.byref(eng.list), C.byref(eng.lj),
                         A.PG_MIXED, A.PG_SYNC_EXACT, C.c_void_p(eng.t["energy"].data_ptr()), ws, eng.sh)
    assert rc == A.PG_OK
    torch.cuda.synchronize()
    assert int(small[:4].view(torch.int32).item()) == queued
    got_f = eng.t["force32"][: eng.n, :3].cpu().numpy().astype(np.float64)
    got_e = eng.t["energy"].cpu().numpy()
    rms = np.sqrt((ref_f ** 2).mean())
    # FP32 sums in another order differ by ~1e-7 of the RMS force; one lost band pair
    # would change a force by |F(rc)| = 0.039, about 1e-3 of it
    assert np.abs(got_f - ref_f).max() / rms < 1e-5
    assert np.allclose(got_e, ref_e, rtol=1e-9, atol=0.0)
