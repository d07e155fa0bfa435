"""The persistent time-step kernel (pg_lj_steps) against the separate kernels.

* The plain steps between rebuild points, run as one cooperative launch per chunk,
  give the trajectory of the same steps launched kernel by kernel: the same rebuilds,
  rewinds and skipped steps (the guard keeps its meaning inside the launch), and
  positions and velocities equal to FP32 summation order (full lists: the same
  arithmetic; half lists: reactions summed by atomics in another order).
* A graph chunk then holds one launch instead of four per step.
* No grid barrier waits without limit: with an arrival count that can never be
  reached, every block gives up after the time limit, status->overflow bit 4 is set,
  and the device stays usable.  The failure is made on the host (the expected count);
  nothing faults, traps or waits forever.
"""
import ctypes as C
import time

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from pairs_gb300 import _capi as A  # noqa: E402
from pairs_gb300 import lattice  # noqa: E402

pytestmark = pytest.mark.gpu


def liquid(cube=16, steps=60):
    from pairs_gb300.engine import LJEngine
    st = lattice.copper_fcc_lattice(cube, cube, cube)
    warm = LJEngine(st, precision="fp64", sync="exact", policy="guard")
    warm.run(steps)
    pos, vel, _ = warm.state()
    return dict(st, pos=pos, vel=vel)


@pytest.mark.parametrize("half,policy", [(False, "interval:6"), (True, "interval:6"), (False, "interval:12"),
                                         (True, "interval:12")])
def test_persistent_chunks_follow_the_separate_kernels(half, policy):
    from pairs_gb300.engine import LJEngine
    st = liquid()
    runs = {}
    for persistent in (True, False):
        e = LJEngine(st, precision="mixed", half=half, sync="exact", policy=policy, persistent=persistent,
                     pair_lists=False)
        assert e.persistent == persistent
        e.run(80)
        pos, vel, frc = e.state()
        runs[persistent] = dict(pos=pos, vel=vel, frc=frc, builds=e.nbuilds, rewinds=e.rewinds,
                                skipped=e.skipped_steps, replays=e.graph_replays, kernels=e.graph_kernels)
        del e
    a, b = runs[True], runs[False]
    assert a["replays"] > 0 and a["replays"] == b["replays"]
    assert (a["builds"], a["rewinds"], a["skipped"]) == (b["builds"], b["rewinds"], b["skipped"])
    if policy == "interval:12":
        assert a["rewinds"] > 0                         # chunks that ended in a guard trip
    # full lists: the same arithmetic up to the order of the few band pairs' additions;
    # half lists: reactions summed by atomics in any order (two runs of the separate
    # kernels differ as much), ~1e-7 of a force, grown by the liquid's chaos over 80
    # steps (measured up to 1.6e-5); test_persistent_chunk_from_a_common_state bounds
    # one chunk tightly
    tol = 1e-10 if not half else 1e-4
    assert np.abs(a["pos"] - b["pos"]).max() < tol
    assert np.abs(a["vel"] - b["vel"]).max() < tol * 100
    rms = np.sqrt((b["frc"] ** 2).mean())
    assert np.abs(a["frc"] - b["frc"]).max() / rms < (1e-6 if not half else 1e-3)
    # one cooperative launch per replayed chunk, against four kernels per step
    assert a["kernels"] == a["replays"]
    assert b["kernels"] > 4 * b["replays"]


@pytest.mark.parametrize("half", [False, True])
def test_persistent_chunk_from_a_common_state(half):
    """From one state (uploaded into both engines: a fresh first step and rebuild), a
    chunk of plain steps in the persistent launch equals the separate kernels' chunk to
    FP32 summation order, before chaos can grow it."""
    from pairs_gb300.engine import LJEngine
    st = liquid()
    engines = [LJEngine(st, precision="mixed", half=half, sync="exact", policy="interval:6", persistent=pers,
                        pair_lists=False) for pers in (True, False)]
    for e in engines:
        e.run(20)
    pos, vel, _ = engines[1].state()
    order = np.argsort(np.asarray(st["uid"]), kind="stable")
    uid = np.asarray(st["uid"], dtype=np.int32)[order]
    mass = np.asarray(st["mass"], dtype=np.float64)[order]
    out = []
    for e in engines:
        e.upload(torch.from_numpy(pos).pin_memory(), torch.from_numpy(vel).pin_memory(),
                 mass=torch.from_numpy(mass).pin_memory(), uid=torch.from_numpy(uid).pin_memory())
        r0 = e.graph_replays
        e.run(7)
        assert e.graph_replays > r0
        out.append(e.state())
    (pa, va, fa), (pb, vb, fb) = out
    tol = 1e-11 if not half else 1e-8
    assert np.abs(pa - pb).max() < tol
    assert np.abs(va - vb).max() < 100 * tol
    assert np.abs(fa - fb).max() / np.sqrt((fb ** 2).mean()) < (1e-6 if not half else 1e-5)


def test_persistent_steps_match_fp64_oracle_forces():
    """After persistent chunks, the mixed forces agree with the FP64 oracle on the same
    positions to the mixed path's tolerance (a stale position read inside the launch
    would show up here as a gross error)."""
    from oracle import lj as olj
    from pairs_gb300.engine import LJEngine
    st = liquid()
    e = LJEngine(st, precision="mixed", half=True, sync="exact", policy="interval:7", persistent=True)
    e.run(50)
    assert e.graph_replays > 0
    pos, vel, frc = e.state()
    ref = olj.Sim(dict(st, pos=pos, vel=vel), every=20, exact_sync=True)
    ref.step()
    _, _, rf = ref.state()
    assert np.abs(frc - rf).max() / max(np.sqrt((rf ** 2).mean()), 1.0) < 1e-5


def test_grid_barrier_gives_up_after_its_time_limit():
    lib = A.load()
    dev = torch.device("cuda")
    ws = torch.zeros(4096, dtype=torch.uint8, device=dev)
    w = A.PgWorkspace(ws.data_ptr(), ws.numel())
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for extra, expect in ((0, 0), (1, 16), (0, 0)):
        status = torch.zeros(8, dtype=torch.int32, device=dev)
        t0 = time.perf_counter()
        assert lib.pg_grid_barrier_check(extra, 0.05, C.c_void_p(status.data_ptr()), w, stream) == A.PG_OK
        torch.cuda.synchronize()
        assert time.perf_counter() - t0 < 10.0
        assert int(status[0].item()) & 16 == expect, extra
    # the device is still usable for ordinary work
    from pairs_gb300.engine import LJEngine
    e = LJEngine(lattice.copper_fcc_lattice(8, 8, 8), precision="mixed", policy="interval:7")
    e.run(20)
    assert np.isfinite(e.state()[0]).all()
