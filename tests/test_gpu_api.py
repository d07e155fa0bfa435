"""Drop-in runs through the reference-style API on the GPU."""
import json
import os

import numpy as np
import pytest

import pairs_gb300 as pairs
from pairs_gb300 import lattice
from tests.scripts import md_script

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def golden_thermo(name):
    return list(np.load(os.path.join(GOLDEN, name + ".npz"))["thermo"])


def test_md_script_prints_reference_thermo():
    psim = md_script.build(pairs, nx=4, timesteps=100)
    psim.run(verbose=False)
    assert psim.thermo_lines == golden_thermo("lj4")


def test_md_script_from_csv_input(tmp_path):
    st = lattice.copper_fcc_lattice(4, 4, 4)
    f = tmp_path / "lattice.input"
    with open(f, "w") as out:
        for k in range(len(st["mass"])):
            p, v = st["pos"][k], st["vel"][k]
            out.write(",".join([str(k), "0", "0", repr(1.0)] + [repr(float(x)) for x in p] +
                               [repr(float(x)) for x in v]) + "\n")
    psim = md_script.build(pairs, nx=4, timesteps=100, input_file=str(f))
    psim.run(verbose=False)
    assert psim.thermo_lines == golden_thermo("lj4")


def test_half_list_script_matches_reference():
    psim = md_script.build(pairs, nx=4, timesteps=100, half=True)
    psim.run(verbose=False)
    assert psim.thermo_lines == golden_thermo("lj4_half")


def test_vtk_output(tmp_path):
    psim = md_script.build(pairs, nx=4, timesteps=10)
    psim.vtk_output(str(tmp_path / "md"), frequency=5)
    psim.run(verbose=False)
    files = sorted(os.listdir(tmp_path))
    assert files == ["md_local_0.vtk", "md_local_10.vtk", "md_local_5.vtk"]
    txt = open(tmp_path / "md_local_5.vtk").read()
    assert "POINTS 256 double" in txt


def test_fused_integration_is_bit_identical_fp64():
    from pairs_gb300.engine import LJEngine
    st = lattice.copper_fcc_lattice(6, 6, 6)
    a = LJEngine(st, sync="reference", fused=True)
    b = LJEngine(st, sync="reference", fused=False)
    a.run(45); b.run(45)
    for x, y in zip(a.state(), b.state()):
        assert np.array_equal(x, y)


def test_mixed_fused_matches_fp64_trajectory():
    from pairs_gb300.engine import LJEngine
    st = lattice.copper_fcc_lattice(6, 6, 6)
    a = LJEngine(st, sync="exact", precision="mixed")
    b = LJEngine(st, sync="exact", precision="fp64")
    for ts in range(41):
        a.step(); b.step()
    pa, va, _ = a.state()
    pb, vb, _ = b.state()
    assert np.abs(pa - pb).max() < 1e-5
    assert np.abs(va - vb).max() < 1e-4
    ta, _ = a.compute_thermo()
    tb, _ = b.compute_thermo()
    assert abs(ta - tb) < 1e-5 * tb
