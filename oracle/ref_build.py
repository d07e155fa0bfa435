"""Recipe: build the reference's own generated CPU program as a test oracle.

The reference (P4IRS) is a Python code generator: a user script calls
``Simulation.generate()`` (src/pairs/sim/simulation.py:382-452), which prints one
C++ file with a ``main()`` (src/pairs/code_gen/cgen.py:57-117).  That file plus the
runtime sources ``runtime/pairs.cpp``, ``runtime/domain/regular_6d_stencil.cpp`` and
``runtime/devices/dummy.cpp`` is the whole reference CPU program.

This recipe, for one configuration:
  1. runs ``oracle/ref_md.py`` (or ``oracle/ref_dem.py``) with the reference's
     ``src/`` on PYTHONPATH, in ``oracle/_ref/<name>/``; the generator writes
     ``<name>.cpp`` there (a build output, never committed);
  2. inserts two calls into that generated ``main()``: ``oracle_hook_init`` before
     the time loop and ``oracle_hook_step`` after each step's user modules
     (definitions in ``oracle/ref_hooks.hpp``, force-included);
  3. compiles it with the runtime sources where they lie under the reference tree
     and the single-rank ``oracle/mpi_stub/mpi.h``, with ``-ffp-contract=off`` so
     the FP64 arithmetic is exactly the generated expression sequence.

Outputs go only to ``oracle/_ref/`` (git-ignored).  Nothing is copied out of the
reference tree.  Test infrastructure: the product never imports this module.

Usage:  python oracle/ref_build.py <config-name> [--run] [--dump DIR]
Configurations are listed in ``CONFIGS`` below.
"""
import argparse
import json
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference source tree: $PAIRS_REFERENCE, or a checkout named "reference" beside
# this repository.  Only this recipe and the fixture generator read it.
REF = os.environ.get("PAIRS_REFERENCE") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
OUT = os.path.join(HERE, "_ref")

# Parity configurations of the LJ path.  "lj4" is the 4x4x4 fcc case of the
# reference's md example at one atom type; "lj4_half" the same with compute_half();
# "lj8" a larger box (2048 atoms) where ghosts are a minority.
CONFIGS = {
    "lj4": dict(kind="md", n=[4, 4, 4], timesteps=100, ntypes=1, reneighbor_every=20, thermo_every=100),
    "lj4_half": dict(kind="md", n=[4, 4, 4], timesteps=100, ntypes=1, reneighbor_every=20,
                     thermo_every=100, half=True),
    "lj4_t4": dict(kind="md", n=[4, 4, 4], timesteps=100, ntypes=4, reneighbor_every=20, thermo_every=100),
    "lj8": dict(kind="md", n=[8, 8, 8], timesteps=100, ntypes=1, reneighbor_every=20, thermo_every=100),
    "lj6x5x4": dict(kind="md", n=[6, 5, 4], timesteps=60, ntypes=1, reneighbor_every=10, thermo_every=20),
    # kernels outside the LJ / velocity-Verlet templates (oracle/ref_custom.py): a
    # force-shifted, capped LJ pair kernel and a damped velocity-Verlet half step
    "custom6": dict(kind="custom", n=[6, 6, 6], timesteps=60, ntypes=2, reneighbor_every=10, thermo_every=20,
                    epsilon=[1.0, 1.2, 1.2, 0.8], sigma6=[1.0, 1.1, 1.1, 0.9],
                    symbols=dict(dt=0.005, fshift=-0.039, fcap=60.0, vmax2=5.0, damping=0.999)),
    "custom6_half": dict(kind="custom", n=[6, 6, 6], timesteps=60, ntypes=2, reneighbor_every=10,
                         thermo_every=20, half=True, epsilon=[1.0, 1.2, 1.2, 0.8], sigma6=[1.0, 1.1, 1.1, 0.9],
                         symbols=dict(dt=0.005, fshift=-0.039, fcap=60.0, vmax2=5.0, damping=0.999)),
    "custom_wca": dict(kind="custom", program="wca", n=[5, 6, 7], timesteps=40, ntypes=1, reneighbor_every=8,
                       thermo_every=10, rho=0.7, temp=1.2,
                       symbols=dict(dt=0.004, wca_rc2=1.2599210498948732, ksoft=20.0, sigma_s=1.15,
                                    vmax2=4.0, vscale=0.998)),
    # DEM example program (spheres on a simple-cubic grid falling on a bottom wall);
    # "dem_dense" packs the grid tighter so sphere-sphere contacts start early
    "dem_small": dict(kind="dem", timesteps=300, domain_size=[0.03, 0.03, 0.05], spacing=0.005,
                      planes=[[100000, 0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0, 13]]),
    "dem_dense": dict(kind="dem", timesteps=300, domain_size=[0.02, 0.02, 0.03], spacing=0.0034,
                      initial_velocity=0.3,
                      planes=[[100000, 0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0, 13]]),
}


def generate(name, cfg):
    wd = os.path.join(OUT, name)
    os.makedirs(wd, exist_ok=True)
    if cfg["kind"] == "dem":
        with open(os.path.join(wd, "planes.input"), "w") as f:
            for p in cfg["planes"]:
                f.write(",".join(repr(x) if isinstance(x, float) else str(x) for x in p) + "\n")
        cfg = dict(cfg, planes="planes.input")
    env = dict(os.environ)
    env["PYTHONPATH"] = os.path.join(REF, "src")
    full = dict(cfg)
    full["name"] = name
    env["PAIRS_ORACLE_CFG"] = json.dumps(full)
    script = os.path.join(HERE, {"md": "ref_md.py", "custom": "ref_custom.py"}.get(cfg["kind"], "ref_dem.py"))
    subprocess.run([sys.executable, script, "cpu"], cwd=wd, env=env, check=True,
                   stdout=subprocess.DEVNULL)
    return wd, os.path.join(wd, name + ".cpp")


def patch(src_path, cfg):
    """Insert the two hook calls into the generated main()."""
    with open(src_path) as f:
        lines = f.read().split("\n")
    if cfg["kind"] == "dem":
        return patch_dem(src_path, lines)

    # The time loop follows the start of the "all" timer (sim/timestep.py:63-72).
    t0 = next(k for k, l in enumerate(lines) if "pairs::start_timer(pairs, 0);" in l)
    m = re.match(r"\s*for\(int (i\d+) = 0; \1 < (\d+); \1\+\+\) \{", lines[t0 + 1])
    assert m, "time loop not found after the all-timer start"
    ts_var = m.group(1)
    every = cfg.get("reneighbor_every", 20)

    init_call = ("    oracle_hook_init(nlocal, uid, type, flags, mass, position, linear_velocity);")

    # Insert the step hook before the thermo block (the last statement of the body).
    th = next(k for k, l in enumerate(lines) if "pairs::compute_thermo(" in l and k > t0)
    th_if = th - 1
    assert lines[th_if].strip().startswith("if("), lines[th_if]
    box = "{%s}" % ", ".join(repr(float(x)) for x in cfg["_box"])
    step_call = (
        "        { const double __box[3] = %s;\n"
        "          const int __rb = ((((%s + 1) %% %d) == 0) || (%s == 0));\n"
        "          oracle_hook_step(%s, __rb, nlocal, nghost, __box, uid, position, linear_velocity, force,\n"
        "                           numneighs, neighborlists, neighbor_capacity, ncells, cell_sizes, particle_cell); }"
        % (box, ts_var, every, ts_var, ts_var))
    lines.insert(th_if, step_call)
    lines.insert(t0, init_call)
    with open(src_path, "w") as f:
        f.write("\n".join(lines))


def patch_dem(src_path, lines):
    t0 = next(k for k, l in enumerate(lines) if "pairs::start_timer(pairs, 0);" in l)
    m = re.match(r"\s*for\(int (i\d+) = 0; \1 < (\d+); \1\+\+\) \{", lines[t0 + 1])
    assert m, "time loop not found after the all-timer start"
    ts_var = m.group(1)
    cu = next(k for k, l in enumerate(lines) if "clear_unused_contact_history(pairs" in l and k > t0)
    while "stop_timer" in lines[cu + 1]:
        cu += 1
    lines.insert(cu + 1, "        oracle_hook_step_dem(%s, nlocal, uid, position, linear_velocity, angular_velocity, "
                         "force, torque, rotation_quat, num_contacts, contact_lists, is_sticking, "
                         "tangential_spring_displacement, impact_velocity_magnitude, neighbor_capacity);" % ts_var)
    lines.insert(t0, "    oracle_hook_init_dem(nlocal, uid, type, flags, shape, mass, radius, position, "
                     "linear_velocity, normal);")
    with open(src_path, "w") as f:
        f.write("\n".join(lines))


def box_of(cfg):
    if "domain" in cfg:
        lo, hi = cfg["domain"]
        return [hi[d] - lo[d] for d in range(3)]
    if cfg["kind"] == "dem":
        return list(cfg["domain_size"])
    a = pow(4.0 / cfg.get("rho", 0.8442), 1.0 / 3.0)   # sim/copper_fcc_lattice.py:19-22
    return [cfg["n"][d] * a for d in range(3)]


def compile_program(wd, name, src_path):
    exe = os.path.join(wd, name + "_cpu")
    rt = os.path.join(REF, "runtime")
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-w",
           "-I", os.path.join(HERE, "mpi_stub"), "-I", REF,
           "-include", os.path.join(HERE, "ref_hooks.hpp"),
           src_path,
           os.path.join(rt, "pairs.cpp"),
           os.path.join(rt, "domain", "regular_6d_stencil.cpp"),
           os.path.join(rt, "devices", "dummy.cpp"),
           "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


def build(name):
    cfg = dict(CONFIGS[name])
    cfg["_box"] = box_of(cfg)
    wd, src = generate(name, cfg)
    patch(src, cfg)
    return compile_program(wd, name, src), cfg


def run(exe, dump_dir, env_extra=None):
    os.makedirs(dump_dir, exist_ok=True)
    env = dict(os.environ)
    env["PAIRS_ORACLE_DUMP"] = dump_dir
    if env_extra:
        env.update(env_extra)
    res = subprocess.run([exe], cwd=os.path.dirname(exe), env=env, check=True,
                         capture_output=True, text=True)
    return res.stdout


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("names", nargs="*", default=["lj4"])
    ap.add_argument("--run", action="store_true")
    args = ap.parse_args()
    for name in args.names:
        exe, cfg = build(name)
        print("built", exe)
        if args.run:
            out = run(exe, os.path.join(OUT, name, "dump"))
            with open(os.path.join(OUT, name, "stdout.txt"), "w") as f:
                f.write(out)
            print(out[:2000])


if __name__ == "__main__":
    main()
