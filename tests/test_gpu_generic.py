"""Generated kernels on the GPU against the reference's own program.

The fixtures custom6 / custom6_half come from the reference's generator run on
oracle/ref_custom.py (a force-shifted, capped LJ pair kernel with two atom types and a
damped velocity-Verlet half step that also writes a user property), compiled and run
on CPU.  The same kernels (tests/scripts/custom_script.py) go through this package's
API, are lowered to CUDA by codegen.py and run by GenericEngine with the reference's
ghost refresh; positions, velocities and forces must agree with the reference's at
every stored step, FP64 to round-off, and the thermo lines must be the same strings.
"""
import json
import os

import numpy as np
import pytest

import pairs_gb300 as pairs
from tests.scripts import custom_script

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def rms_rel(a, b):
    return np.abs(a - b).max() / max(np.sqrt((b ** 2).mean()), 1.0)


@pytest.mark.parametrize("name", ["custom6", "custom6_half", "custom_wca"])
def test_generated_kernels_follow_the_reference(name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    cfg = json.loads(str(g["cfg"]))
    psim = custom_script.build(pairs, cfg)
    eng = psim.build_engine()
    from pairs_gb300.generic import GenericEngine
    assert isinstance(eng, GenericEngine)
    every = cfg["thermo_every"]
    thermo = []
    for ts in range(cfg["timesteps"] + 1):
        eng.step()
        if f"step{ts}_pos" in g:
            pos, vel, frc = eng.state()
            assert rms_rel(frc, g[f"step{ts}_force"]) < 1e-12, ts
            assert np.abs(pos - g[f"step{ts}_pos"]).max() < 1e-11, ts
            assert np.abs(vel - g[f"step{ts}_vel"]).max() < 1e-11, ts
        if ts == 0 or (ts + 1) % every == 0:
            thermo.append("%g\t%g" % eng.compute_thermo())
    assert thermo == list(g["thermo"])
    v = eng.property("linear_velocity")
    m = eng.property("mass")
    if cfg.get("program", "capped") == "capped":
        # the user property written by the damped half step: 0.5 m |v|^2 before damping
        kin = eng.property("kinetic")
        s2 = (v ** 2).sum(axis=1)
        undamped = np.where(kin > 0.5 * m * cfg["symbols"]["vmax2"] * (1 - 1e-9), s2 / 0.999 ** 2, s2)
        assert np.allclose(kin, 0.5 * m * undamped, rtol=1e-9, atol=0)
    else:
        # integer and vector user properties of the clamped half step
        assert np.array_equal(eng.property("steps_done"), np.full(len(m), cfg["timesteps"], dtype=np.int32))
        frc = eng.state()[2]
        assert np.allclose(eng.property("accel"), frc / m[:, None], rtol=1e-12, atol=1e-12)


def test_api_run_prints_the_reference_thermo():
    g = np.load(os.path.join(GOLDEN, "custom6.npz"))
    cfg = json.loads(str(g["cfg"]))
    psim = custom_script.build(pairs, cfg)
    psim.run(verbose=False)
    assert psim.thermo_lines == list(g["thermo"])
