"""Batched ensemble of LJ replicas on the GPU.

* each replica's Verlet list equals the oracle's (the reference's arithmetic) for
  that replica alone, bit-exact after canonical sorting, for every stencil / threads
  per atom layout;
* forces agree with the FP64 oracle to the mixed path's 1e-5 (RMS-normalised), and
  the layouts agree with each other;
* a replica advanced inside the ensemble follows the single-system mixed engine
  (same kernels' arithmetic) to round-off, step for step, and the fixed-point layout
  follows the compensated one;
* speculative chunks replayed as CUDA graphs give the same trajectory as the same
  chunks launched one by one;
* per-replica thermo equals the oracle's temperature of the same velocities;
* pair-cluster half lists over the ensemble (two particles of a cell per row) hold
  every pair of the oracle's list once, non-cubic replicas included, their forces
  agree with the oracle, and their trajectory follows the per-particle half lists;
* a partial rebuild bins and lists only the selected replicas: the others keep their
  particle order and list rows entry for entry, the selected ones get the oracle's
  list of their current positions, and a guarded run with partial rebuilds keeps every
  pair (forces against the oracle's) while listing fewer atoms than full rebuilds.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import lj as olj  # noqa: E402
from pairs_gb300 import lattice  # noqa: E402
from tests.golden.make_golden import canonical_pairs  # noqa: E402

pytestmark = pytest.mark.gpu

CONFIGS = [dict(natoms=500, rho=0.9, temperature=1.0), dict(natoms=864, rho=0.7, temperature=1.4),
           dict(natoms=1331, rho=0.85, temperature=0.8), dict(natoms=2000, rho=0.6, temperature=1.2)]


def replicas():
    return [lattice.trimmed_fcc(**c) for c in CONFIGS]


def rms_rel(a, b):
    return np.abs(a - b).max() / max(np.sqrt(np.mean(b * b)), 1.0)


def unordered(p):
    """Canonical unordered pair set: (min uid, max uid, image of the larger seen from the smaller)."""
    p = np.asarray(p)
    sw = p[:, 0] > p[:, 1]
    a = np.where(sw, p[:, 1], p[:, 0])
    b = np.where(sw, p[:, 0], p[:, 1])
    s = np.where(sw[:, None], -p[:, 2:], p[:, 2:])
    return np.unique(np.concatenate([a[:, None], b[:, None], s], axis=1), axis=0)


@pytest.mark.parametrize("tpa,reach,half", [(1, 1, False), (4, 1, False), (2, 2, False), (8, 2, False),
                                            (1, 1, True), (2, 2, True), (4, 2, True), (2, 3, True), (1, 3, False)])
def test_lists_and_forces_match_oracle(tpa, reach, half):
    from pairs_gb300.ensemble import Ensemble
    reps = replicas()
    ens = Ensemble(reps, tpa=tpa, reach=reach, policy="every", half=half)
    ens.synchronize()
    for r, st in enumerate(reps):
        sim = olj.Sim(st, every=1, exact_sync=True)
        sim.step()
        got, ref = ens.replica_pairs(r), sim.pairs()
        if half:
            # each interior pair once, pairs through an image from both sides
            assert np.array_equal(unordered(got), unordered(ref)), r
            image = np.any(np.asarray(got)[:, 2:] != 0, axis=1)
            assert len(unordered(got)) == (~image).sum() + image.sum() // 2, r
        else:
            assert np.array_equal(canonical_pairs(got), canonical_pairs(ref)), r
        _, _, f_ref = sim.state()
        _, _, f = ens.replica_state(r)
        assert rms_rel(f, f_ref) < 1e-5, (r, rms_rel(f, f_ref))


def test_replica_follows_single_system_engine():
    from pairs_gb300.engine import LJEngine
    from pairs_gb300.ensemble import Ensemble
    reps = replicas()
    # the engine's 27-cell stencil and its compensated hi/lo positions
    ens = Ensemble(reps, tpa=1, reach=1, policy="every", fixed_point=False, half=False)
    ens.run(25)
    ens.synchronize()
    worst = 0.0
    for r, st in enumerate(reps):
        eng = LJEngine(st, precision="mixed", half=False, tiles=False, fixed_point=False, policy="fixed", every=1,
                       sync="exact")
        eng.run(26)
        pos, _, _ = eng.state()
        p2, _, _ = ens.replica_state(r)
        worst = max(worst, np.abs(pos - p2).max())
    print("max position difference after 25 steps", worst)
    # same arithmetic per pair; the single-system kernel applies a pair within 1e-5 of
    # the cutoff in a second pass, so such a particle's force sums in another order
    assert worst < 1e-8


def test_fixed_point_replicas_follow_compensated_replicas():
    """Fixed-point positions (each replica box 2^32 units) in the force pass and the
    guard give the trajectory of the compensated hi/lo layout to FP32 round-off."""
    from pairs_gb300.ensemble import Ensemble
    reps = replicas()
    a = Ensemble(reps, tpa=2, policy="every")
    b = Ensemble(reps, tpa=2, policy="every", fixed_point=False)
    assert a.fixed_point and not b.fixed_point
    a.run(25)
    b.run(25)
    a.synchronize()
    b.synchronize()
    worst = max(np.abs(a.replica_state(r)[0] - b.replica_state(r)[0]).max() for r in range(len(reps)))
    print("max position difference after 25 steps", worst)
    assert worst < 1e-6


def test_graph_chunks_equal_plain_chunks():
    """CUDA-graph chunks replay the plain launches bit for bit (full lists: the half
    lists' reaction atomics sum in a run-dependent order)."""
    from pairs_gb300.ensemble import Ensemble
    reps = replicas()
    a = Ensemble(reps, tpa=2, graphs=True, half=False)
    b = Ensemble(reps, tpa=2, graphs=False, half=False)
    a.run(120)
    b.run(120)
    a.synchronize()
    b.synchronize()
    assert a.nbuilds == b.nbuilds and a.nbuilds > 1
    for r in range(len(reps)):
        pa, va, _ = a.replica_state(r)
        pb, vb, _ = b.replica_state(r)
        assert np.array_equal(pa, pb) and np.array_equal(va, vb)


@pytest.mark.parametrize("half", [False, True])
def test_persistent_chunks_equal_graph_chunks(half):
    """A chunk's plain steps in one cooperative launch (pg_ensemble_steps) follow the
    same chunks as separate kernels under a graph: the same rebuild steps, and the same
    state bit for bit with full lists (half lists: the reactions' atomics sum in any
    order, ~1e-7 of a force per step, grown by the liquid's chaos)."""
    from pairs_gb300.ensemble import Ensemble
    reps = replicas()
    a = Ensemble(reps, tpa=2, graphs=True, half=half, persistent=True)
    b = Ensemble(reps, tpa=2, graphs=True, half=half, persistent=False)
    assert a.persistent and not b.persistent
    steps = 30 if half else 120
    a.run(steps)
    b.run(steps)
    a.synchronize()
    b.synchronize()
    assert a.nbuilds == b.nbuilds and a.nbuilds > 1
    for r in range(len(reps)):
        pa, va, fa = a.replica_state(r)
        pb, vb, fb = b.replica_state(r)
        if half:
            # reaction sums in a run-dependent order; 30 steps keep the liquid's chaos
            # from growing them (after 120 steps: up to 1.3e-5 in position)
            assert np.abs(pa - pb).max() < 1e-7 and np.abs(va - vb).max() < 1e-5
            assert rms_rel(fa, fb) < 1e-4
        else:
            assert np.array_equal(pa, pb) and np.array_equal(va, vb)
    # every chunk was one launch
    assert a.graph_kernels < b.graph_kernels


@pytest.mark.parametrize("half", [False, True])
def test_guard_schedule_keeps_the_pair_set(half):
    """Speculative chunks: after a run, the list rebuilt from the final positions
    holds every pair within the cutoff that the guarded list held (half lists: the
    integration pass zeroes the force that the next force pass accumulates into)."""
    from pairs_gb300.ensemble import Ensemble
    reps = replicas()
    ens = Ensemble(reps, tpa=4, half=half)
    ens.run(80)
    ens.synchronize()
    assert ens.nbuilds >= 2
    for r, st in enumerate(reps):
        pos, vel, f = ens.replica_state(r)
        sim = olj.Sim(dict(st, pos=pos, vel=vel), every=1, exact_sync=True)
        sim.step()
        _, _, f_ref = sim.state()
        # a pair missing from the list would change a force by |F(rc)| = 0.039, ~2e-3
        # of the RMS force; FP32 sums (reactions by atomics, in any order) stay within
        # ~1.6e-5 of it at the largest (measured up to 1.6e-5 at 1M atoms)
        assert rms_rel(f, f_ref) < 2e-5


def test_thermo_matches_oracle_temperature():
    from pairs_gb300.ensemble import Ensemble
    reps = replicas()
    ens = Ensemble(reps)
    t = ens.thermo()
    for r, st in enumerate(reps):
        t_ref, _ = olj.temperature(st["mass"], st["vel"], st["box"])
        assert abs(t[r] - t_ref) <= 1e-12 * t_ref


def stretched(st, f):
    """A replica with its box and positions scaled per axis (a non-cubic box)."""
    f = np.asarray(f, dtype=np.float64)
    return dict(st, pos=st["pos"] * f, box=st["box"] * f)


@pytest.mark.parametrize("reach", [2, 0])
def test_pair_cluster_lists_and_forces_match_oracle(reach):
    """reach 0: per replica the largest cells that fit (here cells of >= r_list for
    most replicas, of >= r_list / 2 for the smallest)."""
    from pairs_gb300.ensemble import Ensemble
    reps = replicas() + [stretched(lattice.trimmed_fcc(natoms=1500, rho=0.8, temperature=1.0), (1.2, 1.0, 0.9))]
    ens = Ensemble(reps, reach=reach, policy="every", pair_lists=True)
    if reach == 0:
        assert ens.ncells < sum(int(np.prod(np.floor(2 * st["box"] / 2.8))) for st in reps)
    ens.synchronize()
    total = 0
    for r, st in enumerate(reps):
        sim = olj.Sim(st, every=1, exact_sync=True)
        sim.step()
        got, ref = ens.replica_pairs(r), sim.pairs()
        # every pair once, images included
        assert len(got) == len(unordered(got)), r
        assert np.array_equal(unordered(got), unordered(ref)), r
        total += len(got)
        _, _, f_ref = sim.state()
        _, _, f = ens.replica_state(r)
        assert rms_rel(f, f_ref) < 1e-5, (r, rms_rel(f, f_ref))
    pairs, entries = ens.list_size()
    assert pairs == total and total / 2 < entries < total


def test_pair_cluster_grid_too_small_is_refused():
    from pairs_gb300.ensemble import Ensemble
    # a 500-atom replica at rho 0.9 has 2 cells of >= r_list per axis: below 2 reach + 1
    with pytest.raises(ValueError, match="pair-cluster"):
        Ensemble(replicas(), reach=1, pair_lists=True)
    with pytest.raises(ValueError, match="fixed-point"):
        Ensemble(replicas(), reach=2, pair_lists=True, fixed_point=False)


def test_pair_cluster_trajectory_follows_per_particle_half_lists():
    """The same steps with pair-cluster and per-particle half lists: the forces of both
    sum in FP32 in different orders, so the trajectories agree to round-off grown by
    the liquid's chaos over 25 steps; after a guarded run of 80 steps the forces match
    the oracle's from the final positions (no pair lost between rebuilds, and the
    integration pass zeroes the force the next pass accumulates into)."""
    from pairs_gb300.ensemble import Ensemble
    reps = replicas()
    a = Ensemble(reps, reach=2, policy="every", pair_lists=True)
    b = Ensemble(reps, tpa=2, reach=2, policy="every", half=True)
    a.run(25)
    b.run(25)
    a.synchronize()
    b.synchronize()
    worst = max(np.abs(a.replica_state(r)[0] - b.replica_state(r)[0]).max() for r in range(len(reps)))
    print("max position difference after 25 steps", worst)
    assert worst < 1e-6
    g = Ensemble(reps, reach=2, pair_lists=True)
    g.run(80)
    g.synchronize()
    assert g.nbuilds >= 2
    for r, st in enumerate(reps):
        pos, vel, f = g.replica_state(r)
        sim = olj.Sim(dict(st, pos=pos, vel=vel), every=1, exact_sync=True)
        sim.step()
        _, _, f_ref = sim.state()
        assert rms_rel(f, f_ref) < 2e-5


@pytest.mark.parametrize("layout", ["full", "pairs"])
def test_partial_rebuild_touches_only_selected_replicas(layout):
    import ctypes as C
    from pairs_gb300 import _capi as A
    from pairs_gb300.ensemble import Ensemble
    reps = replicas()
    kw = dict(tpa=2, reach=2, half=False) if layout == "full" else dict(reach=2, pair_lists=True)
    ens = Ensemble(reps, partial=True, **kw)
    ens.run(12)
    ens.synchronize()
    t = ens.t
    uid0 = t["uid"].cpu().numpy().copy()
    cnt0 = t["count"].cpu().numpy().copy()
    nbr0 = t["nbr"].cpu().numpy().copy()
    table0 = t["pair_table"].cpu().numpy().copy() if layout == "pairs" else None
    flags = np.array([1, 0, 1, 0], dtype=np.int32)
    with torch.cuda.stream(ens.stream):
        t["status"][ens.nstatus:] = torch.from_numpy(flags).to(ens.dev)
        ens.e.rebuild = ens.flags_ptr.value
        by = C.byref
        A.call("pg_ensemble_bin", by(ens.e), by(ens.p), by(ens.cells), ens.ws, ens.status_ptr, ens.sh)
        A.call("pg_ensemble_build_lists", by(ens.e), by(ens.p), by(ens.cells), by(ens.list), ens.r_list2,
               ens.status_ptr, ens.sh)
        ens.e.rebuild = None
        assert ens.read_status().overflow == 0
        t["force32"].zero_()                   # half lists accumulate into zeros
        ens._force(ens.ts)
    ens.synchronize()
    uid1 = t["uid"].cpu().numpy()
    cnt1 = t["count"].cpu().numpy()
    nbr1 = t["nbr"].cpu().numpy()
    cell = t["particle_cell"].cpu().numpy()
    for r, st in enumerate(reps):
        a, b = int(ens.first[r]), int(ens.first[r] + ens.sizes[r])
        assert np.all(np.diff(cell[a:b]) >= 0), r                 # cell order
        if not flags[r]:
            assert np.array_equal(uid1[a:b], uid0[a:b]), r
            if layout == "full":
                assert np.array_equal(cnt1[a:b], cnt0[a:b]), r
                # entry k of particle i at ((k / tpa) * n + i) * tpa + k % tpa
                rows0, rows1 = nbr0.reshape(-1, ens.n, ens.tpa), nbr1.reshape(-1, ens.n, ens.tpa)
                assert np.array_equal(rows1[:, a:b], rows0[:, a:b]), r
        else:
            pos, vel, _ = ens.replica_state(r)
            sim = olj.Sim(dict(st, pos=pos, vel=vel), every=1, exact_sync=True)
            sim.step()
            got, ref = ens.replica_pairs(r), sim.pairs()
            if layout == "full":
                assert np.array_equal(canonical_pairs(got), canonical_pairs(ref)), r
            else:
                assert np.array_equal(unordered(got), unordered(ref)), r
    if layout == "pairs":
        # the rows of the replicas left alone: same slots, same entries
        table1 = t["pair_table"].cpu().numpy()
        first = table1 & ((1 << 30) - 1)
        keep = (table1 >= 0) & np.isin(t["replica_of"].cpu().numpy()[np.clip(first, 0, ens.n - 1)], [1, 3])
        assert np.array_equal(table1[keep], table0[keep])
        assert np.array_equal(cnt1[keep], cnt0[keep])
        stride = ens.list.stride
        for k in range(int(cnt1[keep].max())):
            row0, row1 = nbr0[k * stride:(k + 1) * stride], nbr1[k * stride:(k + 1) * stride]
            live = keep & (cnt1 > k)
            assert np.array_equal(row1[live], row0[live])
    # every replica's force (lists of both kinds) against the oracle's
    for r, st in enumerate(reps):
        pos, vel, f = ens.replica_state(r)
        sim = olj.Sim(dict(st, pos=pos, vel=vel), every=1, exact_sync=True)
        sim.step()
        assert rms_rel(f, sim.state()[2]) < 2e-5, r


@pytest.mark.parametrize("pairs", [False, True])
def test_partial_rebuilds_keep_every_pair(pairs):
    from pairs_gb300.ensemble import Ensemble
    reps = replicas()
    kw = dict(reach=2, pair_lists=True) if pairs else dict(tpa=4, half=True)
    # select 0.9: only replicas close to their own trip join a rebuild (four replicas
    # at the default 0.6 are often all selected)
    ens = Ensemble(reps, partial=True, select=0.9, **kw)
    ens.run(80)
    ens.synchronize()
    assert ens.nbuilds >= 2
    # some builds left replicas alone
    assert ens.rebuilt_atoms < ens.nbuilds * ens.n
    for r, st in enumerate(reps):
        pos, vel, f = ens.replica_state(r)
        sim = olj.Sim(dict(st, pos=pos, vel=vel), every=1, exact_sync=True)
        sim.step()
        assert rms_rel(f, sim.state()[2]) < 2e-5, r


def test_autotune_picks_the_fastest_finalist():
    """Stage 1 scores every layout; stage 2 runs the best scores as real guarded steps
    and returns the fastest of them."""
    from pairs_gb300.ensemble import autotune
    reps = replicas()
    cands = [(2, 128, 2, True), (1, 256, 1, False), (1, 192, 2, "pairs"), (1, 192, 1, "pairs")]
    best, table = autotune(reps, candidates=cands, finalists=2, trial_steps=12)
    # reach-1 pair-cluster lists do not fit the 500-atom replica's grid: skipped
    assert len(table) == 3 and not any(r["half"] == "pairs" and r["reach"] == 1 for r in table)
    timed = [r for r in table if "step_ms" in r]
    assert len(timed) == 2
    assert sorted(table, key=lambda r: r["score"])[:2] == sorted(timed, key=lambda r: r["score"])
    fastest = min(timed, key=lambda r: r["step_ms"])
    assert best == (fastest["tpa"], fastest["block"], fastest["reach"], fastest["half"])


def test_select_flags_the_displaced_replicas():
    """pg_ensemble_select: a replica is flagged when one of its atoms moved more than
    sqrt(thresh2) from its position at the replica's last build (the guard's measure);
    thresh2 < 0 flags every replica."""
    import ctypes as C
    from pairs_gb300 import _capi as A
    from pairs_gb300.ensemble import Ensemble
    reps = replicas()
    ens = Ensemble(reps, tpa=2, policy="every")
    ens.synchronize()
    t = ens.t

    def select(thresh2):
        with torch.cuda.stream(ens.stream):
            A.call("pg_ensemble_select", C.byref(ens.e), C.byref(ens.p), thresh2, ens.flags_ptr, ens.sh)
        ens.synchronize()
        return t["status"][ens.nstatus:].cpu().numpy().copy()

    assert np.array_equal(select(0.0), [0, 0, 0, 0])          # right after the build
    assert np.array_equal(select(-1.0), [1, 1, 1, 1])
    # move one atom of replica 2 by 0.1 along y (0.1 / unit fixed-point steps)
    i = int(ens.first[2]) + 17
    unit = ens.boxes[2][1] / 2.0 ** 32
    with torch.cuda.stream(ens.stream):
        t["pos_fx"][i, 1] += int(round(0.1 / unit))
    assert np.array_equal(select(0.09 ** 2), [0, 0, 1, 0])
    assert np.array_equal(select(0.11 ** 2), [0, 0, 0, 0])


@pytest.mark.parametrize("pairs", [False, True])
def test_tiny_capacity_regrows_in_full_and_partial_builds(pairs):
    """A list capacity of 4 overflows at the first build: the lists grow, the force pass
    queued on the short lists is redone, and the forces equal the oracle's.  An overflow
    inside a partial rebuild bins and lists every replica again (the grown arrays start
    empty), and the forces again equal the oracle's."""
    from pairs_gb300.ensemble import Ensemble
    reps = replicas()
    kw = dict(reach=2, pair_lists=True) if pairs else dict(tpa=2, half=True)
    ens = Ensemble(reps, neighbor_capacity=4, **kw)
    ens.synchronize()
    assert ens._max_nb > 4

    def check():
        for r, st in enumerate(reps):
            pos, vel, f = ens.replica_state(r)
            sim = olj.Sim(dict(st, pos=pos, vel=vel), every=1, exact_sync=True)
            sim.step()
            assert rms_rel(f, sim.state()[2]) < 2e-5, r

    check()
    ens.run(12)
    ens.synchronize()
    grown = ens._max_nb
    # a partial rebuild of every moved replica into lists of capacity 4 (the arrays stay
    # as large as they are: the kernels stop writing at the capacity)
    ens.list.max_neighbors = 4
    ens.select2 = 0.0
    builds = ens.nbuilds
    with torch.cuda.stream(ens.stream):
        ens.t["force32"].zero_()
        ens.rebuild(partial=True, then=lambda: ens._force(ens.ts))
    ens.synchronize()
    assert ens.nbuilds == builds + 1 and ens._max_nb >= 0.9 * grown
    check()
