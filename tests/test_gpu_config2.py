"""LJ fcc 32^3 (131,072 atoms): the mixed-precision path against FP64.

* Force error.  The FP64 oracle (the reference's loop, pinned to its generated
  program) runs from the lattice; at its rebuild steps 99 and 499 the mixed path is
  started from the oracle's positions and computes one force pass.  Its error over
  the oracle's forces on the same positions is bounded in RMS and in maximum,
  relative to the RMS force (full and half lists).
* Energy drift.  The mixed path (half list, learned schedule, the path the headline
  is quoted on) and the FP64 path (half list, exact guard) each run 1000 steps after
  100 equilibration steps from the lattice; E = KE + PE (FP64 sums) is sampled every
  100 steps, and drift = max |E(t) - E(0)| / |E(0)|.  The mixed path adds no drift of
  its own: the two drifts agree within 1e-4 (both are ~3.5e-4: the reference's
  potential is the truncated, unshifted LJ, whose energy jumps whenever a pair
  crosses the cutoff).
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import lj as olj  # noqa: E402
from pairs_gb300 import lattice  # noqa: E402

pytestmark = pytest.mark.gpu

RMS_TOL = 2e-6        # RMS force error over the RMS force (measured 7e-7)
MAX_TOL = 5e-5        # largest single error over the RMS force (measured 9e-6)
DRIFT_GAP = 1e-4      # |drift(mixed) - drift(FP64)| over 1000 steps


@pytest.fixture(scope="module")
def oracle_states():
    st = olj.fcc_lattice(32, 32, 32)
    sim = olj.Sim(st, every=20, exact_sync=True, nthreads=os.cpu_count() or 1)
    out = {}
    done = 0
    for ts in (99, 499):
        sim.run(ts + 1 - done)
        done = ts + 1
        out[ts] = sim.state()
    return st, out


@pytest.mark.parametrize("ts", [99, 499])
@pytest.mark.parametrize("half", [False, True])
def test_mixed_force_error_against_fp64_oracle(oracle_states, ts, half):
    from pairs_gb300.engine import LJEngine
    st, states = oracle_states
    pos, vel, ref = states[ts]
    eng = LJEngine(dict(st, pos=pos, vel=vel), precision="mixed", half=half, sync="exact", policy="guard")
    assert eng.fixed_point
    eng.rebuild()
    eng.force()
    got = eng.state()[2]
    rms = np.sqrt((ref ** 2).mean())
    err = got - ref
    assert np.sqrt((err ** 2).mean()) / rms < RMS_TOL, np.sqrt((err ** 2).mean()) / rms
    assert np.abs(err).max() / rms < MAX_TOL, np.abs(err).max() / rms


def energy_drift(eng, steps=1000, every=100, equilibrate=100):
    eng.run(equilibrate)
    e0, worst = None, 0.0
    for k in range(0, steps + 1, every):
        if k:
            eng.run(every)
        eng.compute_thermo()
        ke = 0.5 * float(eng.t["thermo"][2].item())
        pe, _ = eng.potential_energy()
        e = ke + pe
        e0 = e if e0 is None else e0
        worst = max(worst, abs(e - e0) / abs(e0))
    return worst


def test_mixed_path_adds_no_energy_drift_over_1000_steps():
    from pairs_gb300.engine import LJEngine
    st = lattice.copper_fcc_lattice(32, 32, 32)
    mixed = LJEngine(st, precision="mixed", half=True, sync="exact", policy="learned")
    d_mixed = energy_drift(mixed)
    del mixed
    fp64 = LJEngine(st, precision="fp64", half=True, sync="exact", policy="guard")
    d_fp64 = energy_drift(fp64)
    assert d_mixed < 1e-3 and d_fp64 < 1e-3, (d_mixed, d_fp64)
    assert abs(d_mixed - d_fp64) < DRIFT_GAP, (d_mixed, d_fp64)
