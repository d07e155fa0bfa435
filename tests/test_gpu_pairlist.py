"""Pair-cluster half lists (pairlist.cu) against the per-particle half lists and the oracle.

* The cluster table covers every particle exactly once, two consecutive particles of
  one cell per slot (the last of an odd cell alone).
* The pair set equals the per-particle half list's and the oracle's (unordered pairs
  with the partner's image), on cubic and non-cubic boxes, with one and several types.
* Forces agree with the per-particle kernel to FP32 summation order and with the FP64
  oracle within the mixed path's tolerance; potential energy and virial agree.
* A cutoff-band queue too small for the step walks the cluster lists again and loses
  no force (the reference's resize protocol has no counterpart here: the fallback is
  exact, only slower).
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import lj as olj  # noqa: E402
from pairs_gb300 import _capi as A  # noqa: E402
from pairs_gb300 import lattice  # noqa: E402

pytestmark = pytest.mark.gpu


def unordered(p):
    p = np.asarray(p)
    sw = p[:, 0] > p[:, 1]
    a = np.where(sw, p[:, 1], p[:, 0]); b = np.where(sw, p[:, 0], p[:, 1])
    s = np.where(sw[:, None], -p[:, 2:], p[:, 2:])
    return np.unique(np.concatenate([a[:, None], b[:, None], s], axis=1), axis=0)


def rms_rel(a, b):
    return np.abs(a - b).max() / np.sqrt((b ** 2).mean())


def liquid(nx, ny, nz, steps=30, ntypes=1):
    from pairs_gb300.engine import LJEngine
    st = lattice.copper_fcc_lattice(nx, ny, nz, ntypes=ntypes)
    warm = LJEngine(st, precision="fp64", sync="exact", policy="guard")
    warm.run(steps)
    pos, vel, _ = warm.state()
    return dict(st, pos=pos, vel=vel)


def engines(st, **kw):
    from pairs_gb300.engine import LJEngine
    a = LJEngine(st, precision="mixed", half=True, sync="exact", pair_lists=True, **kw)
    b = LJEngine(st, precision="mixed", half=True, sync="exact", pair_lists=False, **kw)
    assert a.pair_lists and not b.pair_lists and a.fixed_point and b.fixed_point
    return a, b


def test_cluster_table_covers_every_particle_once():
    a, _ = engines(liquid(10, 10, 10))
    a.rebuild()
    tab = a.t["pair_table"].cpu().numpy().astype(np.int64)
    used = tab[tab >= 0]
    first = used & ((1 << 30) - 1)
    has_b = (used >> 30) & 1
    members = np.concatenate([first, first[has_b == 1] + 1])
    assert np.array_equal(np.sort(members), np.arange(a.n))
    cell = a.t["particle_cell"][: a.n].cpu().numpy()
    pair_first = first[has_b == 1]
    assert np.array_equal(cell[pair_first], cell[pair_first + 1])      # both members in one cell
    assert len(tab) == int(A.load().pg_pair_slots(a.n, a.cells.ncells))


@pytest.mark.parametrize("shape,ntypes", [((12, 12, 12), 1), ((11, 9, 14), 1), ((10, 10, 10), 3)])
def test_pair_set_forces_and_energy_match_per_particle_lists(shape, ntypes):
    st = liquid(*shape, ntypes=ntypes)
    kw = {}
    if ntypes > 1:
        eps = np.linspace(0.8, 1.2, ntypes * ntypes).reshape(ntypes, ntypes)
        eps = 0.5 * (eps + eps.T)
        kw = dict(ntypes=ntypes, epsilon=eps.ravel(), sigma6=np.ones(ntypes * ntypes))
    a, b = engines(st, **kw)
    a.step(); b.step()
    pa, pb = a.pairs(), b.pairs()
    assert np.array_equal(unordered(pa), unordered(pb))
    assert len(unordered(pa)) == len(pa)                   # every pair stored once
    fa, fb = a.state()[2], b.state()[2]
    assert rms_rel(fa, fb) < 1e-5                           # FP32 sums in another order
    ea, eb = a.potential_energy(), b.potential_energy()
    assert abs(ea[0] - eb[0]) <= 1e-6 * abs(eb[0])
    assert abs(ea[1] - eb[1]) <= 1e-6 * abs(eb[1])
    if ntypes == 1:
        ref = olj.Sim(st, every=20, half=True, exact_sync=True)
        ref.step()
        assert np.array_equal(unordered(pa), unordered(ref.pairs()))
        assert rms_rel(fa, ref.state()[2]) < 1e-5


def test_trajectory_follows_per_particle_lists():
    """100 steps with guard-driven rebuilds: same rebuild steps, positions equal to the
    chaos of FP32 summation order (the reactions' atomics add in any order; two runs
    of one kind differ by ~1e-5 after 100 steps of this liquid)."""
    st = liquid(14, 14, 14)
    from pairs_gb300.engine import LJEngine
    runs = []
    for pc in (True, False):
        e = LJEngine(st, precision="mixed", half=True, sync="exact", policy="guard", pair_lists=pc)
        e.run(100)
        runs.append((e.state(), e.nbuilds))
    (sa, na), (sb, nb) = runs
    assert na == nb
    assert np.abs(sa[0] - sb[0]).max() < 1e-4
    assert rms_rel(sa[2], sb[2]) < 1e-3


def test_small_cutoff_queue_walks_the_lists_again():
    st = liquid(20, 20, 20)                      # about 27 band pairs expected per pass
    a, _ = engines(st)
    a.rebuild()
    a.force()
    full = a.t["force32"][: a.n].clone()
    small = torch.zeros(256 + 8, dtype=torch.uint8, device=a.dev)   # one queue record
    ws = A.PgWorkspace(small.data_ptr(), small.numel())
    A.call("pg_lj_force", C.byref(a.box), C.byref(a.p), C.byref(a.cells), C.byref(a.list), C.byref(a.lj),
           a.precision, a.sync, None, ws, a.sh)
    torch.cuda.synchronize()
    queued = int(small[:4].view(torch.int32).item())
    assert queued > 1                                       # more band pairs than the queue held
    got = a.t["force32"][: a.n]
    err = (got - full).abs().max().item() / full.pow(2).mean().sqrt().item()
    assert err < 1e-6


def test_pair_lists_are_the_default_on_the_fixed_point_half_path():
    from pairs_gb300.engine import LJEngine
    st = lattice.copper_fcc_lattice(8, 8, 8)
    assert LJEngine(st, precision="mixed", half=True).pair_lists
    assert not LJEngine(st, precision="mixed", half=False).pair_lists
    assert not LJEngine(st, precision="fp64", half=True).pair_lists
    with pytest.raises(ValueError):
        LJEngine(st, precision="mixed", half=False, pair_lists=True)
