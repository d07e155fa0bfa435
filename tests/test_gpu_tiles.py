"""Tile-local (shared-memory neighbourhood) Verlet lists of the mixed path.

The tile list build must accept exactly the reference's pair set (the same FP64
acceptance as the global-index build), including boxes with fewer than three cells
per dimension (every periodic image is a separate segment) and non-cubic boxes;
the tile force kernel must agree with the global-index kernel.
"""
import numpy as np
import pytest

from oracle import lj as olj
from pairs_gb300 import lattice
from tests.golden.make_golden import canonical_pairs

pytestmark = pytest.mark.gpu


def _engine(st, **kw):
    from pairs_gb300.engine import LJEngine
    return LJEngine(st, sync="exact", **kw)


@pytest.mark.parametrize("n,half", [((4, 4, 4), False), ((4, 4, 4), True), ((6, 5, 4), False),
                                    ((6, 5, 4), True), ((12, 12, 12), False), ((20, 20, 20), True)])
def test_tile_pairs_equal_global_pairs(n, half):
    st = lattice.copper_fcc_lattice(*n)
    warm = _engine(st, precision="fp64")
    warm.run(15)                                  # a liquid-like, unsorted state
    pos, vel, _ = warm.state()
    st2 = dict(st, pos=pos, vel=vel)
    g = _engine(st2, precision="fp64", half=half)
    t = _engine(st2, precision="mixed", half=half)
    assert t.tiles and not g.tiles
    g.rebuild(); t.rebuild()
    assert np.array_equal(canonical_pairs(g.pairs()), canonical_pairs(t.pairs()))


@pytest.mark.parametrize("half", [False, True])
def test_tile_force_matches_global_mixed_force(half):
    st = lattice.copper_fcc_lattice(10, 10, 10)
    a = _engine(st, precision="mixed", half=half, tiles=True)
    b = _engine(st, precision="mixed", half=half, tiles=False)
    a.run(12); b.run(12)
    fa, fb = a.state()[2], b.state()[2]
    assert np.abs(fa - fb).max() < 1e-5 * max(np.sqrt((fb ** 2).mean()), 1.0)


def test_tile_overflow_regrows():
    from pairs_gb300.engine import LJEngine
    st = lattice.copper_fcc_lattice(10, 10, 10)
    e = LJEngine(st, precision="mixed", sync="exact")
    e._set_tile_capacity(64)                       # far too small: the build must recover
    e.run(3)
    ref = olj.Sim(olj.fcc_lattice(10, 10, 10), every=20, exact_sync=True)
    ref.run(3)
    f, rf = e.state()[2], ref.state()[2]
    assert np.abs(f - rf).max() < 1e-5 * max(np.sqrt((rf ** 2).mean()), 1.0)
