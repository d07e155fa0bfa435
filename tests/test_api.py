"""The reference-facing Python API: signatures, kernel recognition, plans, I/O."""
import os

import numpy as np
import pytest

import pairs_gb300 as pairs
from pairs_gb300 import io, kernels
from tests.scripts import md_script


def test_md_kernels_recognised():
    assert kernels.recognize(md_script.lennard_jones).family == "lj_pair"
    m = kernels.recognize(md_script.initial_integrate)
    assert m.family == "vv_initial"
    assert m.prop("position") == "position" and m.prop("velocity") == "linear_velocity"
    assert m.symbol("dt") == "dt"
    assert kernels.recognize(md_script.final_integrate).family == "vv_final"


def test_renamed_kernel_still_recognised():
    src = '''
def lj(a, b):
    inv = 1.0 / squared_distance(a, b)
    s6 = inv * inv * inv * sig[a, b]
    apply(frc, delta(a, b) * (48.0 * s6 * (s6 - 0.5) * inv * eps[a, b]))
'''
    m = kernels.recognize(src)
    assert m.family == "lj_pair" and m.prop("force") == "frc" and m.prop("sigma6") == "sig"


@pytest.mark.parametrize("body", [
    # shifted constant: a different potential
    "    apply(force, delta(i, j) * (24.0 * sr6 * (sr6 - 0.5) * sr2 * epsilon[i, j]))",
    # reassociated arithmetic: a different rounding sequence
    "    apply(force, delta(i, j) * (48.0 * sr6 * (sr6 - 0.5) * (sr2 * epsilon[i, j])))",
])
def test_other_kernels_refused(body):
    src = ("def lj(i, j):\n    sr2 = 1.0 / squared_distance(i, j)\n"
           "    sr6 = sr2 * sr2 * sr2 * sigma6[i, j]\n" + body + "\n")
    with pytest.raises(NotImplementedError):
        kernels.recognize(src)


def test_inconsistent_binding_refused():
    # the same template placeholder may not bind two different user names
    src = '''
def f(i):
    linear_velocity[i] += (dt * 0.5) * force[i] / mass[i]
    position[i] += dt * velocity2[i]
'''
    with pytest.raises(NotImplementedError):
        kernels.recognize(src, families=("vv_initial",))


def test_cpu_target_refused():
    psim = pairs.simulation("md", [pairs.point_mass()])
    with pytest.raises(NotImplementedError):
        psim.target(pairs.target_cpu())


def test_plan_of_md_program():
    psim = md_script.build(pairs, nx=4)
    p = psim.plan
    assert p["program"] == "lj"
    assert p["cutoff"] == 2.5 and abs(p["skin"] - 0.3) < 1e-15 and p["dt"] == 0.005
    assert p["ntypes"] == 1 and p["velocity"] == "linear_velocity" and p["force"] == "force"
    assert psim.grid[1][0] == 4 * (4.0 / 0.8442) ** (1.0 / 3.0)
    assert psim.precision == "fp64" and psim.ghost_sync == "reference"


def test_missing_symbol_is_an_error():
    psim = pairs.simulation("md", [pairs.point_mass()], double_prec=True)
    psim.target(pairs.target_gpu())
    psim.add_position('position')
    psim.add_feature('type', 1)
    psim.add_feature_property('type', 'epsilon', pairs.real(), [1.0])
    psim.add_feature_property('type', 'sigma6', pairs.real(), [1.0])
    psim.copper_fcc_lattice(2, 2, 2, 0.8442, 1.44, 1)
    psim.build_neighbor_lists(2.8)
    psim.compute(md_script.initial_integrate, symbols={}, pre_step=True, skip_first=True)
    psim.compute(md_script.lennard_jones, 2.5)
    psim.compute(md_script.final_integrate, symbols={'dt': 0.005}, skip_first=True)
    with pytest.raises(ValueError):
        psim.generate()


def test_read_particle_csv(tmp_path):
    # uid,type,flags,mass,x,y,z,vx,vy,vz  -- one line per particle
    rows = ["0,0,0,1.0,0.5,0.5,0.5,0.1,0.2,0.3",
            "1,0,0,1.0,6.0,1.0,1.0,0.0,0.0,0.0",
            "2,0,0,1.0,9.5,1.0,1.0,0.0,0.0,0.0",        # outside the domain: dropped
            "3,0,4,1.0,9.5,1.0,1.0,0.0,0.0,0.0"]        # fixed: kept although outside
    f = tmp_path / "p.input"
    f.write_text("\n".join(rows) + "\n")
    psim = md_script.build(pairs, nx=4, input_file=str(f))
    st = io.read_particle_data(psim, str(f), ['uid', 'type', 'flags', 'mass', 'position', 'linear_velocity'],
                               pairs.point_mass())
    assert list(st["uid"]) == [0, 1, 3]
    assert np.allclose(st["vel"][0], [0.1, 0.2, 0.3])
    assert list(st["flags"]) == [0, 0, 4]


def test_vtk_format_layout():
    txt = io.format_vtk(np.array([[0.0, 1.0, 2.0], [3.0, 4.0, 5.0], [9, 9, 9]]), np.array([1.0, 2.0, 3.0]),
                        flags=np.array([0, 0, 1]))
    lines = txt.split("\n")
    assert lines[0] == "# vtk DataFile Version 2.0"
    assert "POINTS 2 double" in lines
    assert "0.00000000 1.00000000 2.00000000" in lines
    assert "CELLS 2 4" in lines and "POINT_DATA 2" in lines and "2.00000000" in lines
