"""Pin the CPU oracle (oracle/lj_oracle.c) against the reference's own output.

The fixtures under tests/golden/ were produced by running the reference's generated
CPU program (tests/golden/make_golden.py).  The oracle must reproduce them
bit-for-bit: initial lattice, positions/velocities/forces at the stored steps,
every rebuild's Verlet entries (SHA-256 of the canonically sorted list, plus the
full list where stored), the reference grid occupancy and the printed thermo.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import lj
from tests.golden.make_golden import canonical_pairs, unpack_pairs

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
NAMES = ["lj4", "lj4_half", "lj4_t4", "lj8", "lj6x5x4"]


def load(name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    return g, json.loads(str(g["cfg"]))


def fmt6(x):
    """std::cout default formatting (6 significant digits, %g style)."""
    return "%g" % x


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference_bit_exact(name):
    g, cfg = load(name)
    st = lj.fcc_lattice(*cfg["n"], ntypes=cfg["ntypes"])
    assert np.array_equal(st["pos"], g["init_pos"])
    assert np.array_equal(st["vel"], g["init_vel"])
    assert np.array_equal(st["type"], g["init_type"].astype(np.int32))

    sim = lj.Sim(st, ntypes=cfg["ntypes"], every=cfg["reneighbor_every"], half=cfg.get("half", False))
    rebuilds = list(g["rebuild_steps"])
    shas = list(g["pairs_sha"])
    thermo = []
    for ts in range(cfg["timesteps"] + 1):
        sim.step()
        if f"step{ts}_pos" in g:
            pos, vel, frc = sim.state()
            assert np.array_equal(pos, g[f"step{ts}_pos"]), ts
            assert np.array_equal(vel, g[f"step{ts}_vel"]), ts
            assert np.array_equal(frc, g[f"step{ts}_force"]), ts
        if ts in rebuilds:
            cp = canonical_pairs(sim.pairs())
            assert hashlib.sha256(cp.tobytes()).hexdigest() == shas[rebuilds.index(ts)], ts
            if f"pairs{ts}" in g:
                assert np.array_equal(cp, unpack_pairs(g[f"pairs{ts}"]))
            assert sim.nghost == int(g[f"nghost{ts}"])
            _, sizes, loc = sim.cell_counts()
            assert np.array_equal(sizes, g[f"cells{ts}"][0].astype(np.int32))
            assert np.array_equal(loc, g[f"cells{ts}"][1].astype(np.int32))
        every = cfg["thermo_every"]
        if ts == 0 or (ts + 1) % every == 0:
            t, p = sim.thermo()
            thermo.append(f"{fmt6(t)}\t{fmt6(p)}")
    assert thermo == list(g["thermo"])


def test_exact_sync_differs_only_off_rebuild():
    """The exact ghost refresh changes nothing at rebuild steps (fresh images) and
    differs from the reference's lagging refresh right after them."""
    st = lj.fcc_lattice(4, 4, 4)
    ref = lj.Sim(st, every=20)
    exact = lj.Sim(st, every=20, exact_sync=True)
    ref.step(); exact.step()
    assert np.array_equal(ref.state()[2], exact.state()[2])
    ref.step(); exact.step()
    assert not np.array_equal(ref.state()[2], exact.state()[2])


DEM_NAMES = ["dem_small", "dem_dense"]


@pytest.mark.parametrize("name", DEM_NAMES)
def test_dem_oracle_matches_reference_bit_exact(name):
    from oracle import dem
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    cfg = json.loads(str(g["cfg"]))
    p = dem.example_params(spacing=cfg["spacing"], v0=cfg.get("initial_velocity", 1.0))
    sim = dem.Sim(cfg["domain_size"], cfg["planes"], p)
    ini = sim.initial()
    for k in ("uid", "type", "flags", "shape", "mass", "radius", "pos", "vel", "normal"):
        assert np.array_equal(ini[k], g["init_" + k]), k
    keep = sorted(int(k[4:].split("_")[0]) for k in g.files if k.startswith("step") and k.endswith("_pos"))
    for ts in range(max(keep) + 1):
        sim.step()
        if ts in keep:
            uid = g[f"step{ts}_uid"]
            st = sim.state(uid)
            for k in ("pos", "vel", "angvel", "force", "torque", "quat"):
                assert np.array_equal(st[k], g[f"step{ts}_{k}"]), (ts, k)
            ids, vals = sim.contacts()
            order = np.lexsort((ids[:, 1], ids[:, 0]))
            assert np.array_equal(ids[order], g[f"step{ts}_contact_ids"]), ts
            assert np.array_equal(vals[order], g[f"step{ts}_contact_vals"]), ts
