"""Lowering of general compute() kernels (pairs_gb300/codegen.py), on CPU.

* a program whose kernels are not the LJ / velocity-Verlet templates is planned as
  generated kernels, and the LJ example still takes the hand-tuned path;
* the lowering finds the modules' roles (pair / particle, pre-step, skip_first),
  the applied, written and partner-read properties;
* the generated source has the reference's operation order for the shown cases and
  compiles for sm_103a with nvcc (no GPU needed);
* constructs outside the supported kernel language raise NotImplementedError.
"""
import json
import os
import shutil

import numpy as np
import pytest

import pairs_gb300 as pairs
from pairs_gb300 import codegen
from tests.scripts import custom_script, md_script

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def custom_sim(name="custom6"):
    cfg = json.loads(str(np.load(os.path.join(GOLDEN, name + ".npz"))["cfg"]))
    return custom_script.build(pairs, cfg)


def test_custom_program_is_planned_as_generated_kernels():
    psim = custom_sim()
    plan = psim.generate()
    assert plan["program"] == "generic" and "capped_lj" in plan["reason"]
    assert md_script.build(pairs, nx=4, timesteps=10).generate()["program"] == "lj"


def test_lowering_finds_roles_and_properties():
    psim = custom_sim()
    mods, layout, src = codegen.lower_program(psim, psim.pre_step_functions + psim.functions)
    roles = [(m.name, m.pair, m.pre_step, m.skip_first) for m in mods]
    assert roles == [("initial_integrate", False, True, True), ("capped_lj", True, False, False),
                     ("damped_final_integrate", False, False, True)]
    pair = mods[1]
    assert pair.applied == ["force"] and pair.read_j == {"type"}
    assert mods[2].written == {"linear_velocity", "kinetic"}
    assert layout.slots == ["force", "kinetic", "steps_done", "accel"]
    # operation order of the reference's generated C (left-associative products,
    # min() as the keyword's select chain, the symbol printed as a literal)
    assert "((((48.0 * v_sr6) * (v_sr6 - 0.5)) * v_sr2)" in src
    assert "((60.0 < v_flj) ? 60.0 : v_flj)" in src
    assert "(-0.039 / v_r)" in src


@pytest.mark.skipif(shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"),
                    reason="nvcc not available")
def test_generated_kernels_compile():
    psim = custom_sim("custom6_half")
    mods, layout, src = codegen.lower_program(psim, psim.pre_step_functions + psim.functions)
    so = codegen.compile_source(src)
    assert os.path.exists(so)


def _unsupported_loop(i):
    for k in range(3):
        linear_velocity[i] += k  # noqa: F821


def _unsupported_function(i, j):
    apply(force, delta(i, j) * exp(squared_distance(i, j)))  # noqa: F821


def _store_in_pair_kernel(i, j):
    force[i] = delta(i, j)  # noqa: F821


@pytest.mark.parametrize("func,pair,what", [(_unsupported_loop, False, "For"),
                                            (_unsupported_function, True, "exp"),
                                            (_store_in_pair_kernel, True, "use apply")])
def test_unsupported_constructs_are_refused(func, pair, what):
    psim = custom_sim()
    entry = dict(func=func, cutoff=2.5 if pair else None, symbols={}, pre_step=False, skip_first=False)
    with pytest.raises(NotImplementedError, match=what):
        codegen.lower_program(psim, [entry])
