"""Capacity regrow and non-finite detection (the reference's resize protocol,
src/pairs/transformations/modules.py:159-205 and runtime/devices/device.hpp:63-71:
a kernel reports the size it needed, the host grows the buffer and repeats the work).

All failures here are made on the host (a capacity that is too small, a NaN written
into the uploaded positions); no kernel faults, traps or waits.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from pairs_gb300 import _capi as A  # noqa: E402
from pairs_gb300 import lattice  # noqa: E402
from tests.golden.make_golden import canonical_pairs  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,half", [("fp64", False), ("mixed", True), ("mixed", False)])
def test_tiny_neighbor_capacity_regrows_to_the_same_pair_set(precision, half):
    """A Verlet list of 4 entries per particle (a liquid needs ~80, or ~40 for a half
    list): the build reports the count it needed, the host regrows the list and
    builds again, and the pair set equals the one built with room to spare."""
    from pairs_gb300.engine import LJEngine
    st = lattice.copper_fcc_lattice(10, 10, 10)
    warm = LJEngine(st, precision="fp64", sync="exact", policy="guard")
    warm.run(30)
    pos, vel, _ = warm.state()
    here = dict(st, pos=pos, vel=vel)
    small = LJEngine(here, precision=precision, half=half, sync="exact", neighbor_capacity=4)
    big = LJEngine(here, precision=precision, half=half, sync="exact", neighbor_capacity=200)
    small.rebuild()
    big.rebuild()
    assert small.list.max_neighbors > 4
    cnt = small.list_counts()
    assert cnt.max() <= small.list.max_neighbors
    assert np.array_equal(canonical_pairs(small.pairs()), canonical_pairs(big.pairs()))
    small.force()
    big.force()
    fs, fb = small.state()[2], big.state()[2]
    assert np.abs(fs - fb).max() <= 1e-5 * np.sqrt((fb ** 2).mean())


def _dem_engine(sim, p, cfg, contact_capacity, with_history):
    from pairs_gb300.dem import DEMEngine, dem_params
    ini = sim.initial()
    uid = np.sort(ini["uid"])
    s = sim.state(uid)
    order = np.argsort(ini["uid"], kind="stable")
    state = dict(uid=uid, type=ini["type"][order], flags=ini["flags"][order], shape=ini["shape"][order],
                 mass=ini["mass"][order], radius=ini["radius"][order], normal=ini["normal"][order],
                 pos=s["pos"], vel=s["vel"], angvel=s["angvel"], quat=s["quat"])
    if with_history:
        state["contacts"] = sim.contacts()
    prm = dem_params(p["dt"], p["kappa"], p["ln_e"], p["tc"], 1550.0, p["gravity"], [0.0], [p["mu"]])
    return DEMEngine(state, lo=[0, 0, 0], hi=cfg["domain_size"], periodic=(True, True, False), params=prm,
                     policy="guard", contact_capacity=contact_capacity)


@pytest.mark.parametrize("start,with_history", [(0, False), (120, True)])
def test_dem_contact_capacity_of_one_regrows_with_identical_contacts(start, with_history):
    """dem_dense with one contact record per sphere.  Loaded history that needs more
    records grows the capacity on upload; afterwards every list build grows it to the
    most records a sphere can need before the next build (its list partners plus the
    half spaces), so no step runs out of records.  State and contact records then equal
    those of a run with the default capacity, bit for bit (the capacity changes only
    the allocation)."""
    from tests.test_gpu_dem import golden_cfg, oracle_sim
    cfg = golden_cfg("dem_dense")
    sim, p = oracle_sim(cfg)
    sim.run(start)
    if with_history:
        assert len(sim.contacts()[0]) > 0
    one = _dem_engine(sim, p, cfg, 1, with_history)
    ref = _dem_engine(sim, p, cfg, 20, with_history)
    one.run(150)
    ref.run(150)
    assert one.ccap > 1 and one.contact_regrows >= 1
    a, b = one.state(), ref.state()
    for k in ("pos", "vel", "angvel", "force", "torque", "quat"):
        assert np.array_equal(a[k], b[k]), k
    ia, va = one.contacts()
    ib, vb = ref.contacts()
    assert len(ib) > 0
    assert np.array_equal(ia, ib) and np.array_equal(va, vb)


@pytest.mark.parametrize("precision,half", [("fp64", False), ("mixed", True)])
def test_nan_in_uploaded_positions_raises(precision, half):
    """A NaN written into a host position before upload: binning parks the particle
    in the extra bucket and flags status.nonfinite, and the engine raises PairsError
    at the build instead of integrating garbage."""
    from pairs_gb300.engine import LJEngine
    st = lattice.copper_fcc_lattice(8, 8, 8)
    pos = np.array(st["pos"], dtype=np.float64)
    pos[17, 1] = np.nan
    eng = LJEngine(dict(st, pos=pos), precision=precision, half=half, sync="exact", policy="guard")
    with pytest.raises(A.PairsError, match="non-finite"):
        eng.step()


def test_nan_uploaded_mid_run_raises():
    """The same through upload(): a valid run, then a host state with a NaN."""
    from pairs_gb300.engine import LJEngine
    st = lattice.copper_fcc_lattice(8, 8, 8)
    eng = LJEngine(st, precision="mixed", half=True, sync="exact", policy="learned")
    eng.run(10)
    eng.settle()
    n = eng.n
    pos = torch.zeros((n, 4), dtype=torch.float64)
    pos[:, :3] = torch.from_numpy(np.asarray(st["pos"]))
    pos[5, 2] = float("inf")
    vel = torch.zeros((n, 4), dtype=torch.float64)
    vel[:, :3] = torch.from_numpy(np.asarray(st["vel"]))
    eng.upload(pos.pin_memory(), vel.pin_memory())
    with pytest.raises(A.PairsError, match="non-finite"):
        eng.step()


def test_dem_nan_in_uploaded_positions_raises():
    from tests.test_gpu_dem import golden_cfg, oracle_sim
    cfg = golden_cfg("dem_small")
    sim, p = oracle_sim(cfg)
    sim.run(10)
    ini = sim.initial()
    uid = np.sort(ini["uid"])
    s = sim.state(uid)
    s["pos"] = np.array(s["pos"])
    sphere = int(np.nonzero(ini["shape"][np.argsort(ini["uid"], kind="stable")] == 0)[0][3])
    s["pos"][sphere, 0] = np.nan
    sim2 = type("S", (), {"initial": lambda self: ini, "state": lambda self, u: s,
                          "contacts": lambda self: sim.contacts()})()
    eng = _dem_engine(sim2, p, cfg, 20, False)
    with pytest.raises(A.PairsError, match="non-finite"):
        eng.run(1)
