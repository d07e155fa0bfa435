"""DEM path on the GPU against the DEM oracle (oracle/dem_oracle.c, itself pinned
bit-for-bit to the reference's generated DEM program by test_oracle_golden.py).

* one step from the same state: forces, torques, updated state and contact records
  agree with the oracle to 1e-12 (relative to the RMS force / torque / speed; the
  only difference is the order in which a sphere's few contact forces are summed);
* whole runs (300 steps of the two golden configurations, through the
  reference-style user script): state and contact records stay within the bounds
  below, with the same contacts;
* the candidate list with skin and speculative chunks gives the same trajectory as
  rebinning every step (the reference's cell-list scheme).
"""
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import dem  # noqa: E402

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def golden_cfg(name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    return json.loads(str(g["cfg"]))


def oracle_sim(cfg):
    p = dem.example_params(spacing=cfg["spacing"], v0=cfg.get("initial_velocity", 1.0))
    return dem.Sim(cfg["domain_size"], cfg["planes"], p), p


def engine_from_oracle(sim, p, cfg, policy="every", with_history=True):
    from pairs_gb300.dem import DEMEngine, dem_params
    ini = sim.initial()
    uid = np.sort(ini["uid"])
    st = sim.state(uid)
    order = np.argsort(ini["uid"], kind="stable")
    state = dict(uid=uid, type=ini["type"][order], flags=ini["flags"][order], shape=ini["shape"][order],
                 mass=ini["mass"][order], radius=ini["radius"][order], normal=ini["normal"][order],
                 pos=st["pos"], vel=st["vel"], angvel=st["angvel"], quat=st["quat"])
    if with_history:
        state["contacts"] = sim.contacts()
    prm = dem_params(p["dt"], p["kappa"], p["ln_e"], p["tc"], 1550.0, p["gravity"], [0.0], [p["mu"]])
    return DEMEngine(state, lo=[0, 0, 0], hi=cfg["domain_size"], periodic=(True, True, False), params=prm,
                     policy=policy)


def wrap(pos, L):
    """The reference's exchange wrap (x < 0 -> x + L, x > L -> x - L) on x and y."""
    out = pos.copy()
    for d in range(2):
        out[:, d] = np.where(out[:, d] < 0.0, out[:, d] + L[d], out[:, d])
        out[:, d] = np.where(out[:, d] > L[d], out[:, d] - L[d], out[:, d])
    return out


def rel(a, b, scale=None):
    if b.size == 0:
        return 0.0
    s = scale if scale is not None else max(np.sqrt(np.mean(b * b)), 1e-300)
    return np.abs(a - b).max() / s


def sorted_contacts(ids, vals):
    o = np.lexsort((ids[:, 1], ids[:, 0]))
    return ids[o], vals[o]


@pytest.mark.parametrize("name,start", [("dem_small", 150), ("dem_small", 290), ("dem_dense", 120),
                                        ("dem_dense", 250)])
def test_one_step_matches_oracle(name, start):
    cfg = golden_cfg(name)
    sim, p = oracle_sim(cfg)
    sim.run(start)
    eng = engine_from_oracle(sim, p, cfg)
    sim.step()
    eng.run(1)
    uid = eng.state()["uid"]
    ref = sim.state(uid)
    got = eng.state()
    for k in ("force", "torque"):
        assert rel(got[k], ref[k]) < 1e-12, (k, rel(got[k], ref[k]))
    for k in ("vel", "angvel"):
        assert rel(got[k], ref[k]) < 1e-12, (k, rel(got[k], ref[k]))
    L = cfg["domain_size"]
    assert np.abs(wrap(got["pos"], L) - wrap(ref["pos"], L)).max() < 1e-15
    assert np.abs(got["quat"] - ref["quat"]).max() < 1e-14
    assert np.array_equal(got["ncontacts"], ref["ncontacts"])
    gi, gv = eng.contacts()
    ri, rv = sorted_contacts(*sim.contacts())
    if name == "dem_dense":
        assert len(ri) > 0                        # the dense case has contacts at these steps
    assert np.array_equal(gi, ri)
    assert rel(gv[:, :3], rv[:, :3]) < 1e-12
    assert rel(gv[:, 3], rv[:, 3]) < 1e-12


def write_planes(tmp_path, cfg):
    path = tmp_path / "planes.input"
    with open(path, "w") as f:
        for pl in cfg["planes"]:
            f.write(",".join(repr(x) if isinstance(x, float) else str(x) for x in pl) + "\n")
    return str(path)


@pytest.mark.parametrize("name", ["dem_small", "dem_dense"])
@pytest.mark.parametrize("policy", ["guard", "every"])
def test_run_through_api_matches_oracle(tmp_path, name, policy):
    import pairs_gb300 as pairs
    from tests.scripts import dem_script
    cfg = golden_cfg(name)
    psim = dem_script.build(pairs, domain_size=cfg["domain_size"], spacing=cfg["spacing"],
                            initial_velocity=cfg.get("initial_velocity", 1.0), timesteps=cfg["timesteps"],
                            planes_file=write_planes(tmp_path, cfg))
    from pairs_gb300.dem import build_dem_engine
    eng = build_dem_engine(psim, policy=policy)
    sim, _ = oracle_sim(cfg)
    L = cfg["domain_size"]
    worst = {}
    done = 0
    for stop in (50, 100, 200, 300):
        eng.run(stop - done)
        sim.run(stop - done)
        done = stop
        got = eng.state()
        ref = sim.state(got["uid"])
        vscale = np.sqrt(np.mean(ref["vel"] ** 2))
        errs = dict(pos=np.abs(wrap(got["pos"], L) - wrap(ref["pos"], L)).max(),
                    vel=rel(got["vel"], ref["vel"], vscale), force=rel(got["force"], ref["force"]),
                    angvel=rel(got["angvel"], ref["angvel"]))
        for k, v in errs.items():
            worst[k] = max(worst.get(k, 0.0), v)
        gi, _ = eng.contacts()
        ri, _ = sorted_contacts(*sim.contacts())
        assert np.array_equal(gi[:, :2], ri[:, :2]), stop
    print(name, policy, "worst", worst, "rebuilds", eng.nbuilds, "syncs", eng.host_syncs)
    assert worst["pos"] < 1e-12
    assert worst["vel"] < 1e-9
    assert worst["force"] < 1e-8
    assert worst["angvel"] < 1e-8


def test_skin_list_equals_every_step_rebinning():
    cfg = golden_cfg("dem_dense")
    sim, p = oracle_sim(cfg)
    a = engine_from_oracle(sim, p, cfg, policy="every")
    b = engine_from_oracle(sim, p, cfg, policy="guard")
    a.run(200)
    b.run(200)
    sa, sb = a.state(), b.state()
    L = cfg["domain_size"]
    assert np.abs(wrap(sa["pos"], L) - wrap(sb["pos"], L)).max() < 1e-13
    assert b.nbuilds < a.nbuilds
    ia, _ = a.contacts()
    ib, _ = b.contacts()
    assert np.array_equal(ia, ib)


# ---------------------------------------------------------------------------- granular workload model

def granular_setup(count=900, seed=3, v=2.0):
    """A small version of the 1M-sphere granular workload: radii U[0.4, 0.6] mm,
    2500 kg/m^3, fixed normal stiffness 1e5 N/m, restitution 0.7, friction 0.5,
    dt 1e-6 s, bottom plane; random initial velocities so contacts form quickly."""
    import math
    from pairs_gb300 import lattice
    a = 0.0082
    box = (a, a, 4 * a)
    st = lattice.dem_random_packing(count, box, 4e-4, 6e-4, 2500, seed=seed, spacing=a / 6.5)
    g = np.random.default_rng(seed)
    st["vel"] = g.uniform(-v, v, (count, 3))
    e = 0.7
    p = dict(dt=1e-6, mu=0.5, e=e, tc=5e-4, poisson=0.22, rho_p=2500, rho_f=0, gravity=9.81, diameter=1.2e-3)
    p["kappa"] = 2.0 * (1.0 - p["poisson"]) / (2.0 - p["poisson"])
    p["ln_e"] = math.log(e)
    p["cell"] = 1.01 * 1.2e-3
    planes = [[count + 1, 0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0, 13]]
    return box, st, p, planes


def granular_engine(sim, p, box, precision):
    from pairs_gb300.dem import DEMEngine, dem_params
    ini = sim.initial()
    uid = np.sort(ini["uid"])
    st = sim.state(uid)
    order = np.argsort(ini["uid"], kind="stable")
    state = dict(uid=uid, type=ini["type"][order], flags=ini["flags"][order], shape=ini["shape"][order],
                 mass=ini["mass"][order], radius=ini["radius"][order], normal=ini["normal"][order],
                 pos=st["pos"], vel=st["vel"], angvel=st["angvel"], quat=st["quat"], contacts=sim.contacts())
    prm = dem_params(p["dt"], p["kappa"], p["ln_e"], p["tc"], 2500.0, p["gravity"], [0.0], [p["mu"]], kn=1e5)
    return DEMEngine(state, lo=[0, 0, 0], hi=box, periodic=(True, True, False), params=prm, policy="every",
                     precision=precision)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 2e-5)])
def test_fixed_stiffness_model_one_step(precision, tol):
    """The fixed-stiffness contact model (FP64 and mixed) against the oracle's."""
    box, st, p, planes = granular_setup()
    sim = dem.Sim(box, planes, p, spheres=st, kn=1e5)
    sim.run(200)
    ids, _ = sim.contacts()
    assert len(ids) > 20                          # colliding pairs exist at this step
    eng = granular_engine(sim, p, box, precision)
    sim.step()
    eng.run(1)
    got = eng.state()
    ref = sim.state(got["uid"])
    for k in ("force", "torque"):
        assert rel(got[k], ref[k]) < tol, (k, rel(got[k], ref[k]))
    assert np.array_equal(got["ncontacts"], ref["ncontacts"])
    gi, gv = eng.contacts()
    ri, rv = sorted_contacts(*sim.contacts())
    assert np.array_equal(gi[:, :2], ri[:, :2])
    assert rel(gv[:, 3], rv[:, 3]) < tol


def test_mixed_run_tracks_fp64():
    box, st, p, planes = granular_setup(seed=5)
    sim = dem.Sim(box, planes, p, spheres=st, kn=1e5)
    sim.run(300)
    a = granular_engine(sim, p, box, "fp64")
    b = granular_engine(sim, p, box, "mixed")
    a.run(300)
    b.run(300)
    sa, sb = a.state(), b.state()
    L = box
    assert np.abs(wrap(sa["pos"], L) - wrap(sb["pos"], L)).max() < 1e-9      # metres; radii are 4e-4..6e-4
    assert rel(sb["vel"], sa["vel"]) < 1e-4
