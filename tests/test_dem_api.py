"""DEM side of the reference-facing API (no GPU): kernel recognition, the plan's
constants, and the initial state of dem_sc_grid against the reference's own output."""
import json
import math
import os

import numpy as np
import pytest

import pairs_gb300 as pairs
from pairs_gb300 import kernels, lattice
import pairs_gb300.dem as pdem
from tests.scripts import dem_script

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_dem_kernels_recognised():
    fam = {f.__name__: kernels.recognize(f).family for f in
           (dem_script.update_mass_and_inertia, dem_script.gravity, dem_script.linear_spring_dashpot,
            dem_script.euler)}
    assert fam == dict(update_mass_and_inertia="dem_setup", gravity="dem_gravity",
                       linear_spring_dashpot="dem_contact", euler="dem_euler")
    m = kernels.recognize(dem_script.linear_spring_dashpot)
    assert m.prop("tsd") == "tangential_spring_displacement"
    assert m.symbol("ln_e") == "lnDryResCoeff" and m.symbol("tc") == "collisionTime_SI"


def test_dem_plan_constants():
    psim = dem_script.build(pairs)
    p = psim.plan
    assert p["program"] == "dem"
    assert p["dt"] == 5e-5 and p["tc"] == 5e-4 and p["pi"] == math.pi
    assert p["kappa"] == 2.0 * (1.0 - 0.22) / (2.0 - 0.22)
    assert p["ln_e"] == math.log(0.1)
    assert p["drho"] == 1550.0 and p["gravity"] == 9.81
    assert p["friction_static"] == [0.0] and p["friction_dynamic"] == [0.5]
    assert p["contact_capacity"] == 20


def test_changed_contact_model_refused():
    import inspect
    src = inspect.getsource(dem_script.linear_spring_dashpot).replace("1e-8", "1e-6")
    with pytest.raises(NotImplementedError):
        kernels.recognize(src, families=pdem.DEM_FAMILIES)


def test_dem_kernel_order_enforced():
    psim = pairs.simulation("dem", [pairs.sphere(), pairs.halfspace()], double_prec=True)
    psim.target(pairs.target_gpu())
    psim.add_position('position')
    psim.setup(dem_script.update_mass_and_inertia, {'infinity': math.inf})
    psim.build_cell_lists(0.0032)
    psim.compute(dem_script.euler, symbols={'dt': 5e-5})
    psim.compute(dem_script.gravity, symbols={})
    with pytest.raises(NotImplementedError):
        psim.generate()


@pytest.mark.parametrize("name", ["dem_small", "dem_dense"])
def test_sc_grid_bit_exact(name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    cfg = json.loads(str(g["cfg"]))
    d = 0.0029
    ds = cfg["domain_size"]
    st = lattice.dem_sc_grid(ds[0], ds[1], ds[2], cfg["spacing"], d, d * 0.9, d * 1.1,
                             cfg.get("initial_velocity", 1.0), 2550, 1)
    n = len(st["uid"])
    assert n == len(g["init_uid"]) - len(cfg["planes"])
    for k in ("uid", "mass", "radius", "pos", "vel", "type"):
        assert np.array_equal(st[k], g["init_" + k][:n]), k


def test_mt19937_known_answer():
    # the C++ standard fixes the 10000th output of a default-constructed mt19937
    assert int(lattice._mt19937_words(10000)[-1]) == 4123659995
