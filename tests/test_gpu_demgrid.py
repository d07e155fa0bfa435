"""The DEM simple-cubic initialiser on the device (csrc/demgrid.cu).

The reference's dem_sc_grid (runtime/dem_sc_grid.hpp:62-172) draws every sphere's
diameter and velocity from a default-seeded std::mt19937 and its type from rand().
The device version generates both sequences on the GPU and each sphere in its own
thread; it must give the reference's spheres bit for bit:
* against the reference's own output (tests/golden/dem_small.npz, dem_dense.npz);
* against the host restatement (lattice.dem_sc_grid) on a larger grid with several
  types and a domain that cuts the grid (spheres outside still consume their draw).
"""
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from pairs_gb300 import lattice  # noqa: E402

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def host_view(g):
    out = {k: v.cpu().numpy() for k, v in g.items()}
    out["pos"], out["vel"] = out["pos"][:, :3], out["vel"][:, :3]
    return out


@pytest.mark.parametrize("name", ["dem_small", "dem_dense"])
def test_device_grid_matches_the_reference_output(name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    cfg = json.loads(str(g["cfg"]))
    d = 0.0029
    ds = cfg["domain_size"]
    st = host_view(lattice.dem_sc_grid_device(ds[0], ds[1], ds[2], cfg["spacing"], d, d * 0.9, d * 1.1,
                                              cfg.get("initial_velocity", 1.0), 2550, 1))
    n = len(st["uid"])
    assert n == len(g["init_uid"]) - len(cfg["planes"])
    for k in ("uid", "mass", "radius", "pos", "vel", "type"):
        assert np.array_equal(st[k], g["init_" + k][:n]), k


def test_device_grid_matches_the_host_restatement():
    args = (0.1, 0.08, 0.3, 0.0021, 0.002, 0.0018, 0.0022, 0.5, 2500.0, 3)
    lo, hi = (0.0, 0.01, 0.0), (0.09, 0.08, 0.25)
    dev = host_view(lattice.dem_sc_grid_device(*args, lo=lo, hi=hi))
    host = lattice.dem_sc_grid(*args, lo=lo, hi=hi)
    assert len(host["uid"]) > 50000
    for k in ("uid", "mass", "radius", "pos", "vel", "type", "flags", "shape"):
        assert np.array_equal(dev[k], host[k]), k
    assert set(np.unique(dev["type"])) == {0, 1, 2}
