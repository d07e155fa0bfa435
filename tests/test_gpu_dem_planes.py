"""DEM with half spaces on both sides and dense contacts, against the DEM oracle.

The golden DEM runs have one bottom plane and a few contacts.  Here 2000 spheres sit on an
fcc lattice of 1 mm nearest-neighbour distance with radii U[0.4, 0.6] mm (about 6 of the
12 neighbours overlap), periodic in x and y, between a plane at z = 0 (normal +z) and a
plane at the top (normal -z): half spaces as general shapes in the pair loop
(src/pairs/sim/interaction.py:248-264) and a contact history that the compaction
(src/pairs/sim/contact_history.py:20-127) rewrites every step.  From the oracle's state
after some steps (with its contact history), one GPU step equals one oracle step:
forces, torques, velocities to 1e-12 of their RMS, positions and orientations to
round-off, and the same contact records.

Lattice sites lie on the periodic faces x = 0 and y = 0, so spheres with contacts cross
those faces every few steps.  The reference then packs a leaving sphere's history after
its slot was refilled (sim/comm.py:101-151), and the sphere takes over its filler's
contacts; the GPU path moves each sphere's own records with it.  The oracle runs in
that corrected mode here (history_fixed), as the two modes differ for these spheres.
"""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import dem as odem  # noqa: E402
from pairs_gb300 import lattice  # noqa: E402

pytestmark = pytest.mark.gpu

N = 2000
KN = 1e5


def setup():
    st, box = lattice.dem_compressed_fcc(N, 4e-4, 6e-4, 2500, 1e-3, seed=3)
    planes = [[N + 1, 0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0, 13],
              [N + 2, 0, 1.0, 0.0, 0.0, box[2], 0.0, 0.0, -1.0, 13]]
    e, nu = 0.7, 0.22
    p = dict(dt=1e-6, kappa=2.0 * (1.0 - nu) / (2.0 - nu), ln_e=math.log(e), tc=5e-4, rho_p=2500, rho_f=0,
             gravity=9.81, mu=0.5, cell=1.01 * 1.2e-3)
    spheres = {k: st[k] for k in ("uid", "type", "mass", "radius", "pos", "vel")}
    sim = odem.Sim(box, planes, p, spheres=spheres, kn=KN, ccap=64, history_fixed=True)
    return sim, p, box


def engine(sim, p, box):
    from pairs_gb300.dem import DEMEngine, dem_params
    ini = sim.initial()
    uid = np.sort(ini["uid"])
    s = sim.state(uid)
    order = np.argsort(ini["uid"], kind="stable")
    state = dict(uid=uid, type=ini["type"][order], flags=ini["flags"][order], shape=ini["shape"][order],
                 mass=ini["mass"][order], radius=ini["radius"][order], normal=ini["normal"][order],
                 pos=s["pos"], vel=s["vel"], angvel=s["angvel"], quat=s["quat"], contacts=sim.contacts())
    prm = dem_params(p["dt"], p["kappa"], p["ln_e"], p["tc"], float(p["rho_p"] - p["rho_f"]), p["gravity"], [0.0],
                     [p["mu"]], kn=KN)
    return DEMEngine(state, lo=[0, 0, 0], hi=box, periodic=(True, True, False), params=prm, policy="every",
                     contact_capacity=32)


def rel(a, b):
    return np.abs(a - b).max() / max(np.sqrt(np.mean(b * b)), 1e-300)


def sorted_contacts(ids, vals):
    o = np.lexsort((ids[:, 1], ids[:, 0]))
    return ids[o], vals[o]


@pytest.mark.parametrize("start", [5, 40])
def test_confined_dense_packing_one_step_matches_oracle(start):
    sim, p, box = setup()
    sim.run(start)
    ids, _ = sim.contacts()
    assert len(ids) > 4 * N                       # dense: several contacts per sphere
    top = N + 2
    assert (ids[:, 1] == top).any() and (ids[:, 1] == N + 1).any()   # both planes touched
    eng = engine(sim, p, box)
    sim.step()
    eng.run(1)
    uid = eng.state()["uid"]
    ref = sim.state(uid)
    got = eng.state()
    for k in ("force", "torque", "vel", "angvel"):
        assert rel(got[k], ref[k]) < 1e-12, (k, rel(got[k], ref[k]))
    from tests.test_gpu_dem import wrap
    assert np.abs(wrap(got["pos"], box) - wrap(ref["pos"], box)).max() < 1e-15
    assert np.abs(got["quat"] - ref["quat"]).max() < 1e-14
    gi, gv = eng.contacts()
    ri, rv = sorted_contacts(*sim.contacts())
    assert np.array_equal(gi, ri)
    assert rel(gv[:, :3], rv[:, :3]) < 1e-12
    assert rel(gv[:, 3], rv[:, 3]) < 1e-12
