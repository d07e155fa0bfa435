"""The device VTK writer (pg_vtk_format_rows / pg_vtk_pack_rows) against the host text.

The reference formats every number with std::fixed and 8 decimals (runtime/vtk.hpp:49-53,
79), which is the exact decimal value of the double rounded half to even, as Python's
"%.8f" prints it.  The device text must equal io.format_vtk byte for byte: on random
particle states, on the rounding edge cases (exact ties such as 1/512, -0.0, subnormals,
the largest magnitudes allowed), with infinite particles left out and the CELLS indexes
that name each particle's place among all particles, and through the public API
(vtk_output) on a running LJ simulation.  Values %.8f cannot hold raise PairsError.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from pairs_gb300 import io  # noqa: E402
from pairs_gb300._capi import PairsError  # noqa: E402
from pairs_gb300.types import Flags  # noqa: E402

pytestmark = pytest.mark.gpu

EDGE = [0.0, -0.0, 1.0 / 512, 3.0 / 512, -1.0 / 512, 5.0 / 1024, 0.5e-8, 1.5e-8, 2.5e-8, -2.5e-8, 0.123456785,
        0.999999995, 9.999999995, 1e-300, 5e-324, -5e-324, 1.0 - 2 ** -53, 2.0 ** 36, 123456789.123456789,
        9.1e10, -9.1e10, 0.1, 0.2, 0.3, 1e-8, 1e-9, 4.999999999e-9, 5.000000001e-9, 33.75, 1e10 + 0.5e-8]


def device_text(pos, mass, flags=None, uid=None):
    dev = torch.device("cuda")
    n = len(pos)
    p4 = torch.zeros((n, 4), dtype=torch.float64)
    p4[:, :3] = torch.from_numpy(np.asarray(pos, dtype=np.float64))
    t = lambda a, dt: None if a is None else torch.from_numpy(np.asarray(a)).to(dt).to(dev)
    return io.device_vtk_text(p4.to(dev), t(mass, torch.float64), t(flags, torch.int32), t(uid, torch.int32))


def host_text(pos, mass, flags=None, uid=None):
    order = np.argsort(uid, kind="stable") if uid is not None else np.arange(len(pos))
    f = None if flags is None else np.asarray(flags)[order]
    return io.format_vtk(np.asarray(pos)[order], np.asarray(mass)[order], f).encode()


@pytest.mark.parametrize("n,seed", [(1, 0), (7, 1), (1000, 2), (100003, 3)])
def test_random_states_match_host_text(n, seed):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(-50, 250, (n, 3)) * rng.choice([1e-3, 1.0, 1e3], (n, 1))
    mass = rng.uniform(0.1, 10, n)
    uid = rng.permutation(n).astype(np.int32)
    flags = np.where(rng.random(n) < 0.05, int(Flags.Infinite), 0).astype(np.int32)
    flags |= np.where(rng.random(n) < 0.1, int(Flags.Fixed), 0).astype(np.int32)
    got = device_text(pos, mass, flags, uid)
    assert got == host_text(pos, mass, flags, uid)


def test_rounding_edge_cases_match_host_text():
    v = np.array(EDGE)
    pos = np.stack([v, -v, v[::-1]], axis=1)
    mass = np.abs(v)
    got = device_text(pos, mass)
    want = host_text(pos, mass)
    assert got == want
    assert b"0.00195312 -0.00195312" in got          # 1/512: the tie rounds to even
    assert b"-0.00000000" in got                       # -0.0 keeps its sign, as printf does


def test_all_infinite_and_empty():
    pos = np.zeros((3, 3))
    flags = np.full(3, int(Flags.Infinite), dtype=np.int32)
    assert device_text(pos, np.ones(3), flags) == host_text(pos, np.ones(3), flags)
    assert device_text(np.zeros((0, 3)), np.zeros(0)) == io.format_vtk(np.zeros((0, 3)), np.zeros(0)).encode()


@pytest.mark.parametrize("bad", [9.3e10, -1e12, float("nan"), float("inf")])
def test_values_outside_the_format_raise(bad):
    pos = np.array([[0.0, 1.0, 2.0], [bad, 0.0, 0.0]])
    with pytest.raises(PairsError):
        device_text(pos, np.ones(2))


def test_vtk_output_of_a_running_simulation(tmp_path):
    import pairs_gb300 as pairs
    from tests.scripts import md_script
    psim = md_script.build(pairs, nx=6, timesteps=20)
    psim.vtk_output(str(tmp_path / "md"), frequency=10)
    eng = psim.run(verbose=False)
    assert sorted(os.listdir(tmp_path)) == ["md_local_0.vtk", "md_local_10.vtk", "md_local_20.vtk"]
    pos, _, _ = eng.state()
    got = open(tmp_path / "md_local_20.vtk", "rb").read()
    assert got == io.format_vtk(pos, eng.masses(), eng.flags()).encode()
