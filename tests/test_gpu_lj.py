"""GPU parity of the LJ path against the reference's output and the CPU oracle.

Bars (from the path's specification):
  * Verlet pair sets bit-exact after canonical sorting (given the same positions);
  * FP64 forces within 1e-12 of the reference, relative to the RMS force;
  * thermo (T, P) within 1e-10 relative over 100 steps;
  * mixed precision: forces within 1e-5 RMS-relative of FP64.
All calls go through the C ABI (pairs_gb300._capi / libpairs_gb300.so).
"""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import lj as olj
from pairs_gb300 import lattice
from tests.golden.make_golden import canonical_pairs, unpack_pairs

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
FORCE_TOL = 1e-12      # relative to RMS force, FP64
THERMO_TOL = 1e-10     # relative, FP64, 100 steps
MIXED_FORCE_TOL = 1e-5


def load(name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    return g, json.loads(str(g["cfg"]))


def engine(cfg, **kw):
    from pairs_gb300.engine import LJEngine
    st = lattice.copper_fcc_lattice(*cfg["n"], ntypes=cfg["ntypes"])
    args = dict(every=cfg["reneighbor_every"], half=cfg.get("half", False), ntypes=cfg["ntypes"],
                sync="reference", precision="fp64")
    args.update(kw)
    return LJEngine(st, **args)


def rms_rel(a, b):
    """Max abs error over the RMS of the reference force (at least 1 force unit: a
    perfect lattice has forces ~1e-14 by symmetry)."""
    return np.abs(a - b).max() / max(np.sqrt((b ** 2).mean()), 1.0)


def unordered(p):
    """Canonical unordered pair set: (min uid, max uid, image of the larger seen from the smaller)."""
    p = np.asarray(p)
    sw = p[:, 0] > p[:, 1]
    a = np.where(sw, p[:, 1], p[:, 0]); b = np.where(sw, p[:, 0], p[:, 1])
    s = np.where(sw[:, None], -p[:, 2:], p[:, 2:])
    u = np.unique(np.concatenate([a[:, None], b[:, None], s], axis=1), axis=0)
    return u


@pytest.mark.parametrize("name", ["lj4", "lj4_t4", "lj8", "lj6x5x4"])
def test_reference_sync_matches_reference(name):
    g, cfg = load(name)
    eng = engine(cfg)
    rebuilds = list(g["rebuild_steps"])
    thermo = []
    for ts in range(cfg["timesteps"] + 1):
        eng.step()
        if f"step{ts}_pos" in g:
            pos, vel, frc = eng.state()
            assert rms_rel(frc, g[f"step{ts}_force"]) < FORCE_TOL, ts
            assert np.abs(pos - g[f"step{ts}_pos"]).max() < 1e-11, ts
            assert np.abs(vel - g[f"step{ts}_vel"]).max() < 1e-11, ts
        if ts == 0:
            cp = canonical_pairs(eng.pairs())
            assert hashlib.sha256(cp.tobytes()).hexdigest() == g["pairs_sha"][0]
        if ts == 0 or (ts + 1) % cfg["thermo_every"] == 0:
            thermo.append("%g\t%g" % eng.compute_thermo())
    assert thermo == list(g["thermo"])


def test_thermo_within_1e10_of_oracle_over_100_steps():
    g, cfg = load("lj4")
    eng = engine(cfg)
    ref = olj.Sim(olj.fcc_lattice(4, 4, 4), every=20)
    for ts in range(101):
        eng.step(); ref.step()
        if ts in (0, 50, 99, 100):
            t, p = eng.compute_thermo()
            rt, rp = ref.thermo()
            assert abs(t - rt) <= THERMO_TOL * abs(rt), ts
            assert abs(p - rp) <= THERMO_TOL * abs(rp), ts


@pytest.mark.parametrize("name,ts", [("lj4", 19), ("lj4", 0)])
def test_pair_set_bit_exact_on_reference_positions(name, ts):
    """Given the reference's own positions at a rebuild step, the GPU Verlet list is
    exactly the reference's (same SHA-256 of the canonically sorted entries)."""
    from pairs_gb300.engine import LJEngine
    g, cfg = load(name)
    st = lattice.copper_fcc_lattice(*cfg["n"])
    st = dict(st, pos=g[f"step{ts}_pos"], vel=g[f"step{ts}_vel"])
    eng = LJEngine(st, every=cfg["reneighbor_every"])
    eng.rebuild()
    cp = canonical_pairs(eng.pairs())
    rebuilds = list(g["rebuild_steps"])
    assert hashlib.sha256(cp.tobytes()).hexdigest() == g["pairs_sha"][rebuilds.index(ts)]
    if f"pairs{ts}" in g:
        assert np.array_equal(cp, unpack_pairs(g[f"pairs{ts}"]))


def test_half_list_matches_reference_half():
    g, cfg = load("lj4_half")
    eng = engine(cfg)
    eng.step()
    ref_pairs = unpack_pairs(g["pairs0"])
    assert np.array_equal(unordered(eng.pairs()), unordered(ref_pairs))
    # interior pairs once, pairs through a periodic image from both sides
    p = eng.pairs()
    image = np.any(p[:, 2:] != 0, axis=1)
    assert len(unordered(p)) == (~image).sum() + image.sum() // 2
    for ts in range(1, cfg["timesteps"] + 1):
        eng.step()
        if f"step{ts}_force" in g:
            assert rms_rel(eng.state()[2], g[f"step{ts}_force"]) < FORCE_TOL, ts


@pytest.mark.parametrize("half", [False, True])
def test_exact_sync_matches_oracle_exact(half):
    st = olj.fcc_lattice(6, 5, 4)
    ref = olj.Sim(st, every=10, half=half, exact_sync=True)
    eng = engine(dict(n=[6, 5, 4], ntypes=1, reneighbor_every=10, half=half), sync="exact")
    for ts in range(31):
        ref.step(); eng.step()
        _, _, rf = ref.state()
        _, _, ef = eng.state()
        assert rms_rel(ef, rf) < FORCE_TOL, ts


@pytest.mark.parametrize("fixed_point", [True, False])
def test_mixed_precision_forces_close_to_fp64(fixed_point):
    st = olj.fcc_lattice(8, 8, 8)
    ref = olj.Sim(st, every=20, exact_sync=True)
    eng = engine(dict(n=[8, 8, 8], ntypes=1, reneighbor_every=20), sync="exact", precision="mixed",
                 fixed_point=fixed_point)
    assert eng.fixed_point == fixed_point
    for ts in range(41):
        ref.step(); eng.step()
        if ts in (1, 20, 40):
            rp, rv, rf = ref.state()
            ep, ev, ef = eng.state()
            assert rms_rel(ef, rf) < MIXED_FORCE_TOL, ts
            assert np.abs(ep - rp).max() < 1e-6, ts


def _oracle_energy(st, pos, vel):
    """Oracle PE and virial of the given positions (one force pass, no integration)."""
    return olj.Sim(dict(st, pos=pos, vel=vel), every=20, exact_sync=True).step(energy=True)


def _gpu_engine_at(st, pos, vel, **kw):
    from pairs_gb300.engine import LJEngine
    e = LJEngine(dict(st, pos=pos, vel=vel), every=20, **kw)
    e.rebuild()
    return e


def test_energy_and_virial_match_oracle():
    st = olj.fcc_lattice(6, 6, 6)
    ref = olj.Sim(st, every=20, exact_sync=True)
    ref.run(25)
    pos, vel, _ = ref.state()
    e = _oracle_energy(st, pos, vel)
    pe, vir = _gpu_engine_at(st, pos, vel).potential_energy()
    assert abs(pe - e[0]) <= 1e-10 * abs(e[0])
    assert abs(vir - e[1]) <= 1e-10 * abs(e[1])
    pe, vir = _gpu_engine_at(st, pos, vel, half=True).potential_energy()
    assert abs(pe - e[0]) <= 1e-10 * abs(e[0])
    pe, vir = _gpu_engine_at(st, pos, vel, half=True, precision="mixed").potential_energy()
    assert abs(pe - e[0]) <= 1e-5 * abs(e[0])
    assert abs(vir - e[1]) <= 1e-5 * abs(e[1])


def test_momentum_conserved_and_deterministic_at_32cube():
    from pairs_gb300.engine import LJEngine
    st = lattice.copper_fcc_lattice(32, 32, 32)
    runs = []
    for _ in range(2):
        eng = LJEngine(st, every=20, sync="exact")
        eng.run(30)
        pos, vel, frc = eng.state()
        assert np.abs(frc.sum(axis=0)).max() < 1e-8 * np.abs(frc).mean() * len(frc) ** 0.5
        runs.append((pos, vel, frc))
    assert np.array_equal(runs[0][0], runs[1][0])
    assert np.array_equal(runs[0][2], runs[1][2])


def test_pair_set_matches_oracle_and_is_symmetric_at_32cube():
    from pairs_gb300.engine import LJEngine
    st = lattice.copper_fcc_lattice(32, 32, 32)
    eng = LJEngine(st, every=20, sync="exact")
    eng.run(25)
    pos, vel, _ = eng.state()
    p = _gpu_engine_at(st, pos, vel).pairs()
    fwd = set(map(tuple, p.tolist()))
    assert fwd == set((b, a, -x, -y, -z) for a, b, x, y, z in fwd)
    ref = olj.Sim(dict(st, pos=pos, vel=vel), every=20, exact_sync=True)
    ref.step()
    assert np.array_equal(canonical_pairs(ref.pairs()), canonical_pairs(p))


def test_half_and_full_forces_agree_at_64cube():
    from pairs_gb300.engine import LJEngine
    st = lattice.copper_fcc_lattice(64, 64, 64)
    a = LJEngine(st, every=20, sync="exact")
    b = LJEngine(st, every=20, sync="exact", half=True)
    a.run(3); b.run(3)
    fa, fb = a.state()[2], b.state()[2]
    assert rms_rel(fb, fa) < 1e-11      # different FP64 summation order (atomics)


@pytest.mark.parametrize("half", [True, False])
def test_fixed_point_and_compensated_layouts_match_fp64_forces(half):
    """On the same (liquid) positions, fixed-point positions (one int4 per particle,
    2^32 units per box length) and compensated hi/lo positions give the oracle's pair
    set and forces within the mixed path's tolerance, and the same energy."""
    from pairs_gb300.engine import LJEngine
    st = olj.fcc_lattice(12, 12, 12)
    warm = olj.Sim(st, every=20, exact_sync=True)
    warm.run(20)
    pos, vel, _ = warm.state()
    here = dict(st, pos=pos, vel=vel)
    ref = olj.Sim(here, every=20, half=half, exact_sync=True)
    ref.step()
    _, _, rf = ref.state()
    pe_ref = _oracle_energy(st, pos, vel)[0]
    for fx in (True, False):
        e = LJEngine(here, every=20, precision="mixed", half=half, sync="exact", fixed_point=fx)
        assert bool(e.p.pos_fx) == fx and bool(e.p.pos_hi) != fx
        e.step()
        same = unordered if half else canonical_pairs         # a half list may store either side
        assert np.array_equal(same(e.pairs()), same(ref.pairs())), fx
        assert rms_rel(e.state()[2], rf) < MIXED_FORCE_TOL, fx
        pe, _ = e.potential_energy()
        assert abs(pe - pe_ref) <= 1e-6 * abs(pe_ref), fx


def test_fixed_point_layout_needs_a_large_periodic_box():
    from pairs_gb300 import lattice
    from pairs_gb300.engine import LJEngine
    st = lattice.copper_fcc_lattice(4, 4, 4)              # 2 cells per axis
    assert not LJEngine(st, precision="mixed").fixed_point
    with pytest.raises(ValueError):
        LJEngine(st, precision="mixed", fixed_point=True)
    big = lattice.copper_fcc_lattice(8, 8, 8)             # 4 cells per axis
    assert LJEngine(big, precision="mixed").fixed_point
    assert not LJEngine(big, precision="mixed", periodic=(True, True, False)).fixed_point


def test_half_list_counts_are_balanced_within_warps():
    """A half list keeps the partners above each particle in x, so counts vary only
    with the local density: on a liquid (fcc 16^3 after 40 steps) a warp's 32
    consecutive particles have lists of nearly one length (mean over max above 0.75;
    splitting the pairs by cell order gave about 0.6), and the half list holds half
    the full list's interior pairs plus its image pairs."""
    from pairs_gb300.engine import LJEngine
    st = lattice.copper_fcc_lattice(16, 16, 16)
    e = LJEngine(st, precision="mixed", half=True, policy="guard", pair_lists=False)
    e.run(40)
    e.settle()
    e.rebuild()
    cnt = e.t["count"][: e.n].cpu().numpy().astype(np.int64)
    w = cnt[: len(cnt) // 32 * 32].reshape(-1, 32)
    assert w.sum() / (32 * w.max(axis=1)).sum() > 0.75
    full = LJEngine(dict(st, pos=e.state()[0], vel=e.state()[1]), precision="mixed", half=False)
    full.rebuild()
    assert np.array_equal(unordered(e.pairs()), unordered(full.pairs()))
