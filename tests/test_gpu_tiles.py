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


@pytest.mark.parametrize("n", [(4, 4, 4), (6, 5, 4), (12, 12, 12), (20, 20, 20)])
def test_tile_pairs_equal_global_pairs(n):
    st = lattice.copper_fcc_lattice(*n)
    warm = _engine(st, precision="fp64")
    warm.run(15)                                  # a liquid-like, unsorted state
    pos, vel, _ = warm.state()
    st2 = dict(st, pos=pos, vel=vel)
    g = _engine(st2, precision="fp64")
    t = _engine(st2, precision="mixed", tiles=True)
    assert t.tiles and not g.tiles
    g.rebuild(); t.rebuild()
    assert np.array_equal(canonical_pairs(g.pairs()), canonical_pairs(t.pairs()))


def test_half_lists_use_global_lists():
    st = lattice.copper_fcc_lattice(6, 6, 6)
    e = _engine(st, precision="mixed", half=True)
    assert not e.tiles
    with pytest.raises(ValueError):
        _engine(st, precision="mixed", half=True, tiles=True)


@pytest.mark.parametrize("tpa", [1, 2, 4])
def test_tile_force_matches_global_mixed_force(tpa):
    st = lattice.copper_fcc_lattice(10, 10, 10)
    a = _engine(st, precision="mixed", tiles=True, tile_tpa=tpa)
    b = _engine(st, precision="mixed", tiles=False, fixed_point=False)     # same position records
    a.run(12); b.run(12)
    fa, fb = a.state()[2], b.state()[2]
    assert np.abs(fa - fb).max() < 1e-5 * max(np.sqrt((fb ** 2).mean()), 1.0)
    pa, _ = a.potential_energy()
    pb, _ = b.potential_energy()
    assert abs(pa - pb) <= 1e-6 * abs(pb)


@pytest.mark.parametrize("limit,keeps_tiles", [(1200, True), (64, False)])
def test_tile_overflow_recovers(limit, keeps_tiles):
    """A neighbourhood above the shared-memory limit makes the build shorten the
    tiles, and give them up when a single cell's neighbourhood is still too large."""
    from pairs_gb300.engine import LJEngine
    st = lattice.copper_fcc_lattice(10, 10, 10)
    e = LJEngine(st, precision="mixed", sync="exact", tiles=True)
    tz0 = e.list.tile_z
    e.TILE_LIMIT = limit
    e.run(3)
    assert e.tiles == keeps_tiles
    if keeps_tiles:
        assert e.list.tile_z < tz0 and e.list.tile_capacity <= limit
    ref = olj.Sim(olj.fcc_lattice(10, 10, 10), every=20, exact_sync=True)
    ref.run(3)
    f, rf = e.state()[2], ref.state()[2]
    assert np.abs(f - rf).max() < 1e-5 * max(np.sqrt((rf ** 2).mean()), 1.0)
