#!/usr/bin/env python
"""Benchmark: atom-steps/s of the LJ particle path on one GB300.

Workload (default): fcc 64x64x64 unit cells = 1,048,576 atoms, rho 0.8442, T 1.44,
rc 2.5, skin 0.3, dt 0.005, one type, periodic cube.  A "step" is one MD time step of
the reference's loop (integrate, rebuild when due, LJ force, integrate, thermo at
its cadence) over all atoms.  The headline arm is the mixed-precision path (FP32
force on compensated FP32 positions, FP64 integration/guard/reductions); the plain
FP64 path is timed on the same workload and reported beside it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

`--impl reference` times the CPU restatement of the reference's algorithm
(oracle/lj_oracle.c, every host thread) on the same workload.  With N > 1 (torchrun)
each rank runs an independent replica (replicas only: the path does not shard);
value = atoms * steps summed over ranks / max rank time.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "atom-steps/s on 1 GB300: mixed+learned vs plain FP64 at equal energy drift"
UNIT = "atom-steps/s"

WORKLOADS = {
    "lj64": dict(n=(64, 64, 64)),
    "lj32": dict(n=(32, 32, 32)),
    "lj128": dict(n=(128, 128, 128)),
}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.rows, self.proc = [], None
        self.gpu = gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def dist_setup():
    from pairs_gb300.replicas import init_from_env
    return init_from_env(os.environ)


def traffic_from_profiles(kernel, variant, atoms):
    """DRAM bytes per launch of `kernel` in `variant` from a committed ncu summary
    (profiles/traffic.txt lines: kernel variant atoms bytes), scaled to `atoms` by the
    atom count of the capture (the force pass's traffic grows in proportion: list
    entries and records per atom are fixed by the density), or (None, None)."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    try:
        with open(path) as f:
            for line in f:
                parts = line.split()
                if len(parts) >= 4 and parts[0] == kernel and parts[1] == variant:
                    ref_atoms, ref_bytes = int(parts[2]), float(parts[3])
                    return ref_bytes * atoms / ref_atoms, ref_atoms
    except OSError:
        pass
    return None, None


# ------------------------------------------------------------------------------ our arm

def run_ours(args, rank, world, dist):
    import torch
    from pairs_gb300 import _capi as A
    from pairs_gb300 import lattice
    from pairs_gb300.engine import LJEngine

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    wl = WORKLOADS[args.workload]
    st = lattice.copper_fcc_lattice(*wl["n"])
    n = len(st["mass"])
    lib = A.load()

    tiles = {"auto": None, "on": True, "off": False}[args.tiles]   # auto: the engine's default (global lists)

    def make(precision, half, policy):
        return LJEngine(st, precision=precision, half=half, sync="exact", every=20, policy=policy,
                        device=str(dev), tiles=tiles if precision == "mixed" else None, tile_tpa=args.tile_tpa,
                        fixed_point={"auto": None, "on": True, "off": False}[args.fixed_point],
                        pair_lists={"auto": None, "on": True, "off": False}[args.pair_lists]
                        if precision == "mixed" and half else None)

    def kernel_times(eng, k):
        stream = eng.stream
        eng.p.step = eng.device_step(max(eng.ts - 1, 0))
        out = []
        for _ in range(k):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            eng.force()
            b.record(stream)
            out.append((a, b))
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in out[2:]]

    def calibrate(eng):
        """Train the learned schedule on the run's own first rebuild cycles (setup)."""
        t0 = time.perf_counter()
        k = 0
        if eng.schedule is not None:
            while not eng.schedule.trained and k < 2000:
                eng.step()
                k += 1
        torch.cuda.synchronize()
        return k, time.perf_counter() - t0

    def timed(eng, steps, warmup, force_events=True):
        eng.run(warmup)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        stream = eng.stream
        ev = []
        orig_force = eng.force

        def force_timed(energy=False):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            orig_force(energy)
            b.record(stream)
            ev.append((a, b))

        if force_events:
            eng.force = force_timed
        l0 = lib.pg_kernel_launches() + eng.graph_kernels - eng.graph_captured
        c0 = dict(builds=eng.nbuilds, syncs=eng.host_syncs, rewinds=eng.rewinds, skipped=eng.skipped_steps,
                  replays=eng.graph_replays)
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.nvtx.range_push("timed")        # ncu --nvtx-include "timed/" selects these launches
        s0.record(stream)
        eng.run(steps)
        s1.record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        # library kernels that ran: those launched one by one plus those of graph replays
        launches = lib.pg_kernel_launches() + eng.graph_kernels - eng.graph_captured - l0
        eng.force = orig_force
        ms = s0.elapsed_time(s1)
        fms = [a.elapsed_time(b) for a, b in ev]
        counters = {"rebuilds": eng.nbuilds - c0["builds"], "host_syncs": eng.host_syncs - c0["syncs"],
                    "rewinds": eng.rewinds - c0["rewinds"], "skipped_steps": eng.skipped_steps - c0["skipped"],
                    "graph_replays": eng.graph_replays - c0["replays"]}
        return ms, fms, launches, counters

    prec, half = {"mixed-half": ("mixed", True), "mixed-full": ("mixed", False),
                  "fp64-half": ("fp64", True), "fp64-full": ("fp64", False)}[args.variant]
    eng = make(prec, half, args.policy)
    calib_steps, calib_s = calibrate(eng)
    clocks = ClockSampler(dev.index or 0)
    clocks.start()
    ms, _, launches, counters = timed(eng, args.steps, args.warmup, force_events=False)
    clk = clocks.stop()
    # whole job: the atoms all replicas advanced over the slowest rank's time
    from pairs_gb300.replicas import job_throughput
    value, ms = job_throughput(n * args.steps, ms, dist, device=dev)
    # force-kernel time for the roofline: a speculative policy issues passes that the
    # device skips after a guard trip, so time the kernel on its own on the settled
    # state (same stream, CUDA events around each launch)
    eng.settle()
    fms = kernel_times(eng, 20)
    pairs_total, entries_total = eng.list_size()

    def build_times(eng, k):
        """The Verlet build alone (the last binning's cells, current positions), CUDA
        events around each call; the list it leaves is valid for these positions."""
        out = []
        for _ in range(k):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(eng.stream)
            A.call("pg_build_neighbor_lists", C.byref(eng.box), C.byref(eng.p), C.byref(eng.cells),
                   C.byref(eng.list), eng.r_list2, eng.status_ptr, eng.sh)
            b.record(eng.stream)
            out.append((a, b))
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in out[1:]]

    build_ms = statistics.median(build_times(eng, 6))
    # algorithmic bytes of one force launch: own position (16 fixed point, 32 FP32 hi+lo
    # or FP64 x,y,z,pad), neighbour count (4 per particle; a pair-cluster list reads a
    # count and a table word per cluster slot), force write (16 FP32 / 32 FP64), each
    # stored list entry once (4 bytes global, 2 bytes tile-local; a pair-cluster entry
    # carries one or two pairs); a half list adds one reaction write per particle (b_F)
    b_f = 16 if prec == "mixed" else 32
    b_entry = 2 if eng.list.nbr16 else 4
    b_pos = 16 if (prec == "mixed" and eng.fixed_point) else 32     # fixed point: one int4
    b_count = 8 * eng.list.stride if eng.pair_lists else 4 * n
    b_force = n * (b_pos + b_f) + b_count + b_entry * entries_total + (n * b_f if eng.list.half else 0)
    # the mixed path's force pass: pair-cluster lists (k_pc_lj), packed pair arithmetic
    # on fixed-point positions (k_lj_packed), one pair at a time on compensated
    # positions (k_lj_mixed)
    kname = ("k_tile_lj" if eng.list.nbr16 else "k_pc_lj" if eng.pair_lists else
             (("k_lj_packed" if eng.fixed_point else "k_lj_mixed") if prec == "mixed" else "k_lj_fp64"))
    f_avg = statistics.mean(fms) if fms else float("nan")
    pk, pk_kind = peaks()
    achieved = b_force / (f_avg / 1e3) / 1e9
    traffic, traffic_atoms = traffic_from_profiles(kname, args.variant, n)
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": round(achieved / pk["hbm_gbs"], 4), "peak_kind": pk_kind,
                "traffic": traffic, "kernel": "%s (%s)" % (kname, args.variant),
                "kernel_ms": round(f_avg, 4), "algorithmic_bytes": b_force, "list_pairs": pairs_total,
                "list_entries": entries_total, "list_bytes": b_entry * entries_total,
                "build_ms": round(build_ms, 4)}
    if traffic is not None and traffic_atoms != n:
        roofline["traffic_scaled_from_atoms"] = traffic_atoms
    schedule = dict(counters, policy=args.policy, calibration_steps=calib_steps,
                    calibration_s=round(calib_s, 3),
                    mean_cycle=round(args.steps / max(1, counters["rebuilds"]), 2))
    if args.only_headline:
        print(json.dumps({"variant": args.variant, "policy": args.policy, "value": value,
                          "ms_per_step": ms / args.steps, "roofline": roofline, "schedule": schedule,
                          "gpu_launches": launches, "clocks": clk}))
        return

    # energy drift over --drift-steps (untimed): E = KE + PE, sampled every 100 steps,
    # both methods started from the same state after 100 equilibration steps
    def drift(eng_d, steps, every=100):
        eng_d.run(max(0, 100 - eng_d.ts))
        e0 = None
        worst = 0.0
        for k in range(0, steps + 1, every):
            if k:
                eng_d.run(every)
            t, _ = eng_d.compute_thermo()
            ke = 0.5 * float(eng_d.t["thermo"][2].item())
            pe, _ = eng_d.potential_energy()
            e = ke + pe
            e0 = e if e0 is None else e0
            worst = max(worst, abs(e - e0) / abs(e0))
        return worst

    drift_headline = None
    if args.drift_steps:
        ed = make(prec, half, args.policy)
        calibrate(ed)
        drift_headline = drift(ed, args.drift_steps)
        del ed

    # force error of the mixed path against the FP64 path (which matches the FP64
    # oracle to 1e-12) on one equilibrated state: RMS and maximum error over the RMS
    # force, both engines rebuilt from the same positions
    def force_error():
        eq = make(prec, half, "guard")
        eq.run(100)
        pos, vel, _ = eq.state()
        del eq
        st2 = dict(st, pos=pos, vel=vel)
        out = {}
        for p_ in (prec, "fp64"):
            e_ = LJEngine(st2, precision=p_, half=half, sync="exact", every=20, policy="fixed", device=str(dev))
            e_.rebuild()
            e_.force()
            out[p_] = e_.state()[2]
            del e_
        ref = out["fp64"]
        err = out[prec] - ref
        rms = float(np.sqrt((ref ** 2).mean()))
        return {"rms_rel": float(np.sqrt((err ** 2).mean())) / rms, "max_rel": float(np.abs(err).max()) / rms,
                "state": "after 100 steps from the lattice"}

    ferr = force_error() if prec == "mixed" else None

    # plain FP64 path on the same workload, with rebuild schedules that keep the list
    # valid (the exact guard read after every step, alone or with the reference's
    # every-20 rule): at 1M atoms the guard trips every ~6 steps, so the reference's
    # every-20 rule alone would miss pairs and is not a valid comparator
    fp64 = {}
    k64 = max(100, args.steps)
    for half64, pol in ((True, "guard"), (False, "guard"), (True, "fixed+guard")):
        e64 = make("fp64", half64, pol)
        ms64, _, _, c64 = timed(e64, k64, max(args.warmup, 3), force_events=False)
        f64ms = kernel_times(e64, 6)
        fp64[f"{'half' if half64 else 'full'}_{pol}"] = {
            "value": n * k64 / (ms64 / 1e3), "steps": k64, "force_ms": round(statistics.mean(f64ms), 4),
            "rebuilds": c64["rebuilds"]}
        del e64
    best64 = max(v["value"] for v in fp64.values())
    drift64 = None
    if args.drift_steps:
        e64 = make("fp64", True, "guard")
        drift64 = drift(e64, args.drift_steps)
        del e64

    # rebuild schedules on the same path and workload (mixed, same list kind): the
    # learned schedule against the reference's fixed every-20 schedule with the exact
    # guard on (a trip forces the rebuild; the host reads the guard after every step),
    # the guard alone, and a fixed interval of 7 steps checked by the guard
    schedules = {}
    if prec == "mixed":
        ks = max(100, min(args.steps, 800))
        for pol in (args.policy, "ema", "fixed+guard", "guard", "interval:7"):
            if pol in schedules:
                continue
            es = make(prec, half, pol)
            cs, _ = calibrate(es)
            mss, _, _, cnt = timed(es, ks, max(args.warmup, 100 - cs), force_events=False)
            schedules[pol] = {"ms_per_step": round(mss / ks, 4), "value": n * ks / (mss / 1e3), "steps": ks,
                              "rebuilds": cnt["rebuilds"], "host_syncs": cnt["host_syncs"],
                              "rewinds": cnt["rewinds"]}
            del es

    # end to end through the public engine API from pinned host buffers, on the state
    # the timed loop ended with (downloaded once, untimed): every chunk uploads that
    # state, advances `chunk` steps, and downloads positions, velocities and thermo
    chunk = min(100, args.steps)
    nchunks = max(3, args.steps // chunk)
    eng.settle()
    eng.flush()
    host = {k: eng.t[k][:n].cpu().pin_memory() for k in ("pos", "vel", "mass", "type", "uid")}
    out_pos = torch.empty((n, 4), dtype=torch.float64).pin_memory()
    out_vel = torch.empty((n, 4), dtype=torch.float64).pin_memory()
    torch.cuda.synchronize()
    h2d = d2h = 0
    t0 = time.perf_counter()
    for _ in range(nchunks):
        eng.upload(host["pos"], host["vel"], host["mass"], host["type"], host["uid"])
        h2d += sum(v.numel() * v.element_size() for v in host.values())
        eng.run(chunk)
        eng.flush()
        out_pos.copy_(eng.t["pos"][:n], non_blocking=True)
        out_vel.copy_(eng.t["vel"][:n], non_blocking=True)
        eng.compute_thermo()
        d2h += 2 * n * 32 + 24
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    e2e = {"value": n * chunk * nchunks / el, "unit": UNIT, "h2d_bytes_per_step": h2d // (chunk * nchunks),
           "d2h_bytes_per_step": d2h // (chunk * nchunks), "chunks": nchunks,
           "definition": f"public engine API on the state the timed loop ended with: per call upload the full "
                         f"particle state from pinned host, advance {chunk} MD steps (the first a rebuild), "
                         f"download positions+velocities and thermo; {nchunks} calls"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(st, args.cpu_steps)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 force / f64 integrate",
        "data": "synthetic (fcc lattice, Park-Miller velocities as the reference)",
        "config": {"workload": f"LJ fcc {wl['n'][0]}x{wl['n'][1]}x{wl['n'][2]} = {n} atoms, rho 0.8442, T 1.44, "
                               f"rc 2.5, skin 0.3, dt 0.005, {args.variant}, rebuild policy {args.policy} "
                               "(exact FP64 displacement guard)",
                   "atoms": n, "parallelism": "replicas" if world > 1 else "single",
                   "l2": "inputs larger than L2 (per step: Verlet list %.0f MB, FP64 positions and "
                         "velocities %.0f MB)" % (b_entry * entries_total / 1e6, 64 * n / 1e6)},
        "roofline": roofline, "schedule": schedule,
        "energy_drift_1000": {"headline": drift_headline, "fp64_guard": drift64, "steps": args.drift_steps},
        "force_error_vs_fp64": ferr,
        "fp64": {"best_value": best64, **fp64, "speedup_headline_vs_fp64": value / world / best64},
        "schedules": schedules,
        "e2e": e2e, "gpu_launches": launches, "clocks": clk, "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line))


def cpu_baseline(st, steps):
    """The oracle port (C restatement of the reference's loop) on every host thread."""
    from oracle import lj as olj
    nth = os.cpu_count() or 1
    sim = olj.Sim(st, every=20, exact_sync=True, nthreads=nth)
    t0 = time.perf_counter()
    sim.run(steps)
    el = time.perf_counter() - t0
    n = len(st["mass"])
    return {"value": n * steps / el, "unit": UNIT, "cores": nth, "kind": "port",
            "sample": f"{steps} MD steps of the full {n}-atom system (incl. rebuilds every 20) "
                      f"with oracle/lj_oracle.c, OpenMP {nth} threads"}


# ------------------------------------------------------------------------------ ensemble

def run_ensemble(args, rank, world, dist):
    """Batched ensemble (512 replicas, 500..32000 atoms each, rho U[0.6,0.9],
    T U[0.7,1.5], mixed precision): aggregate atom-steps/s of the batched path (one
    launch per phase, CUDA-graph chunks, autotuned layout) against the same replicas
    advanced one by one with the single-system engine."""
    import torch
    from pairs_gb300 import _capi as A
    from pairs_gb300 import lattice
    from pairs_gb300.engine import LJEngine
    from pairs_gb300.ensemble import Ensemble, autotune
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    cfgs = lattice.ensemble_configs(count=args.replicas)
    reps = [lattice.trimmed_fcc(**c) for c in cfgs]
    natoms = sum(len(r["mass"]) for r in reps)
    steps = args.steps
    if args.ensemble_layout:
        # a fixed layout "tpa,block,reach,half" instead of the autotuner's choice (half:
        # 0 full lists, 1 half lists, 2 pair-cluster half lists)
        tpa, block, reach, half = (int(v) for v in args.ensemble_layout.split(","))
        half, table = ("pairs" if half == 2 else bool(half)), []
    else:
        (tpa, block, reach, half), table = autotune(reps)
    pairs = half == "pairs"
    ens = Ensemble(reps, tpa=tpa, block=block, reach=reach, half=True if pairs else half, pair_lists=pairs,
                   persistent=args.ensemble_persistent, partial=not args.ensemble_full_rebuilds,
                   select=args.ensemble_select)
    ens.run(args.warmup)
    ens.synchronize()
    clocks = ClockSampler(dev.index or 0)
    clocks.start()
    lib = A.load()
    l0 = lib.pg_kernel_launches() + ens.graph_kernels - ens.graph_captured
    b0, s0, a0 = ens.nbuilds, ens.host_syncs, ens.rebuilt_atoms
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("timed")            # ncu --nvtx-include "timed/" selects these launches
    e0.record(ens.stream)
    ens.run(steps)
    e1.record(ens.stream)
    ens.synchronize()
    torch.cuda.nvtx.range_pop()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    # library kernels that ran: launched one by one, plus those of graph replays
    launches = lib.pg_kernel_launches() + ens.graph_kernels - ens.graph_captured - l0
    value = natoms * steps / (ms / 1e3)
    # one by one: every replica with the single-system mixed engine (guard policy)
    one_steps = args.one_by_one_steps
    one_s, one_value = 0.0, None
    if one_steps > 0:
        t0 = time.perf_counter()
        for st in reps:
            eng = LJEngine(st, precision="mixed", half=ens.half, tiles=False, policy="guard", sync="exact")
            eng.run(one_steps + 1)
            del eng
        torch.cuda.synchronize()
        one_s = time.perf_counter() - t0
        one_value = natoms * one_steps / one_s
    line = {
        "metric": "aggregate atom-steps/s of a batched LJ ensemble on 1 GB300", "value": value,
        "unit": UNIT, "n_gpus": 1, "steps": steps, "warmup": args.warmup, "ms_per_step": ms / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 force / f64 integrate",
        "data": "synthetic (trimmed fcc lattices, reference velocity rule, seed 2024)",
        "config": {"workload": f"{len(reps)} LJ replicas, {natoms} atoms total, sizes log-uniform 500..32000, "
                               "rho U[0.6,0.9], T U[0.7,1.5], rc 2.5, skin 0.3, dt 0.005, mixed, "
                               f"{'pair-cluster half' if pairs else ('half' if ens.half else 'full')} lists, "
                               f"guard rebuilds ({'selected replicas' if ens.partial else 'every replica'}), CUDA-graph chunks",
                   "replicas": len(reps), "atoms": natoms,
                   "autotuned": {"tpa": tpa, "block": block, "reach": reach, "half_lists": bool(half),
                                 "pair_lists": pairs}},
        "autotune_table": table,
        "one_by_one": {"value": one_value, "steps": one_steps, "seconds": one_s,
                       "definition": f"each replica alone through LJEngine (mixed, {'half' if ens.half else 'full'} "
                                     "list, guard), "
                                     "wall time including its setup"},
        "speedup_vs_one_by_one": value / one_value if one_value else None,
        "schedule": {"rebuilds": ens.nbuilds - b0, "host_syncs": ens.host_syncs - s0,
                     "partial": ens.partial, "select": args.ensemble_select,
                     "rebuilt_atoms_per_step": (ens.rebuilt_atoms - a0) / steps},
        "gpu_launches": launches, "clocks": clk,
    }
    print(json.dumps(line))


# ------------------------------------------------------------------------------ DEM

def granular_workload(count, seed=7):
    """The granular DEM workload: `count` spheres, radii U[0.4, 0.6] mm, 2500 kg/m^3,
    random non-overlapping positions (jittered lattice of spacing 1.2615 mm) in a
    1:1:4 box periodic in x and y over a rigid plane at z = 0 (82 x 82 x 328 mm for
    1M spheres, ~25% solid fraction), at rest under gravity."""
    import math
    from pairs_gb300 import lattice
    s = 0.082 / 65
    nx = 65 if count == 1000000 else int(math.ceil((count / 4.0) ** (1.0 / 3.0))) + 1
    a = nx * s
    box = (a, a, 4 * a)
    st = lattice.dem_random_packing(count, box, 4e-4, 6e-4, 2500, seed=seed, spacing=s)
    plane = dict(pos=np.zeros((1, 3)), vel=np.zeros((1, 3)), mass=np.ones(1), radius=np.zeros(1),
                 type=np.zeros(1, np.int32), uid=np.array([count + 1], np.int32), flags=np.array([13], np.int32),
                 shape=np.ones(1, np.int32), normal=np.array([[0.0, 0.0, 1.0]]))
    state = {k: np.concatenate([st[k] if k in st else np.zeros((count, 3)), plane[k]]) for k in plane}
    e, nu = 0.7, 0.22
    consts = dict(dt=1e-6, kappa=2.0 * (1.0 - nu) / (2.0 - nu), ln_e=math.log(e), tc=5e-4, drho=2500.0,
                  gravity=9.81, mu=0.5, kn=1e5)
    return box, state, consts


def dense_workload(count, seed=7):
    """The dense DEM workload: `count` spheres, radii U[0.4, 0.6] mm, 2500 kg/m^3, on
    an fcc lattice of 1 mm nearest-neighbour distance (a compressed packing: about 6
    of the 12 neighbours overlap), periodic in x and y, between a plane at z = 0
    (normal +z) and a plane at the top (normal -z), at rest under gravity.  The same
    contact model and time step as the granular workload."""
    import math
    from pairs_gb300 import lattice
    st, box = lattice.dem_compressed_fcc(count, 4e-4, 6e-4, 2500, 1e-3, seed=seed)
    planes = dict(pos=np.array([[0.0, 0.0, 0.0], [0.0, 0.0, box[2]]]), vel=np.zeros((2, 3)), mass=np.ones(2),
                  radius=np.zeros(2), type=np.zeros(2, np.int32), uid=np.array([count + 1, count + 2], np.int32),
                  flags=np.array([13, 13], np.int32), shape=np.ones(2, np.int32),
                  normal=np.array([[0.0, 0.0, 1.0], [0.0, 0.0, -1.0]]))
    state = {k: np.concatenate([st[k] if k in st else np.zeros((count, 3)), planes[k]]) for k in planes}
    e, nu = 0.7, 0.22
    consts = dict(dt=1e-6, kappa=2.0 * (1.0 - nu) / (2.0 - nu), ln_e=math.log(e), tc=5e-4, drho=2500.0,
                  gravity=9.81, mu=0.5, kn=1e5)
    return box, state, consts


def run_dem(args, rank, world, dist):
    """Granular DEM workload on one GB300: mixed precision (FP64 contact geometry,
    FP32 contact model, FP64 integration) against the FP64 path, particle-steps/s."""
    import torch
    from pairs_gb300 import _capi as A
    from pairs_gb300.dem import DEMEngine, dem_params
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    count = args.dem_spheres
    dense = args.workload == "dem-dense"
    builder = dense_workload if dense else granular_workload
    box, state, c = builder(count)
    nplanes = int((np.asarray(state["shape"]) != 0).sum())
    prm = lambda: dem_params(c["dt"], c["kappa"], c["ln_e"], c["tc"], c["drho"], c["gravity"], [0.0], [c["mu"]],
                             kn=c["kn"])
    lib = A.load()

    def timed(precision, steps):
        eng = DEMEngine(state, lo=[0, 0, 0], hi=box, periodic=(True, True, False), params=prm(),
                        precision=precision, skin=1e-4)
        eng.run(args.warmup)
        torch.cuda.synchronize()
        l0, b0 = lib.pg_kernel_launches(), eng.nbuilds
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        eng.run(steps)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        ncont = int(eng.sets[0]["ccount"][:eng.n].sum().item())
        # the contact kernel on its own (CUDA events on the engine's stream), on the
        # state the run ended with
        fev = []
        eng.d.guard = None                      # time every pass, whatever the guard says
        for _ in range(5):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(eng.stream)
            eng._force(eng.ts)
            b.record(eng.stream)
            fev.append((a, b))
        torch.cuda.synchronize()
        force_ms = statistics.median([a.elapsed_time(b) for a, b in fev[1:]])
        out = dict(value=(count + nplanes) * steps / (ms / 1e3), ms_per_step=ms / steps, steps=steps,
                   rebuilds=eng.nbuilds - b0, launches=lib.pg_kernel_launches() - l0, contacts_at_end=ncont,
                   contacts_per_sphere=round(ncont / count, 3), contact_kernel_ms=round(force_ms, 4),
                   contact_capacity=eng.ccap)
        del eng
        torch.cuda.empty_cache()
        return out

    clocks = ClockSampler(dev.index or 0)
    clocks.start()
    mixed = timed("mixed", args.steps)
    clk = clocks.stop()
    fp64 = timed("fp64", max(10, args.steps // 5))
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import dem as odem
        n_cpu = 20000
        cbox, cstate, _ = builder(n_cpu)
        spheres = {k: cstate[k][:n_cpu] for k in ("uid", "type", "mass", "radius", "pos", "vel")}
        p = dict(dt=c["dt"], kappa=c["kappa"], ln_e=c["ln_e"], tc=c["tc"], rho_p=2500, rho_f=0,
                 gravity=c["gravity"], mu=c["mu"], cell=1.01 * 1.2e-3)
        planes = [[int(cstate["uid"][k]), 0, 1.0] + list(cstate["pos"][k]) + list(cstate["normal"][k]) + [13]
                  for k in range(n_cpu, len(cstate["uid"]))]
        sim = odem.Sim(cbox, planes, p, spheres=spheres, kn=c["kn"], ccap=64 if dense else 20)
        sim.run(5)
        k = 100
        t0 = time.perf_counter()
        sim.run(k)
        el = time.perf_counter() - t0
        cpu = {"value": (n_cpu + 1) * k / el, "unit": "particle-steps/s", "cores": 1, "kind": "port",
               "sample": f"{k} steps of a {n_cpu}-sphere version of the workload with oracle/dem_oracle.c "
                         "(the reference's DEM program restated: every step rebins and scans 27 cells)"}
    line = {
        "metric": f"particle-steps/s of the {'dense' if dense else 'granular'} DEM workload on 1 GB300",
        "value": mixed["value"],
        "unit": "particle-steps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": mixed["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64 geometry + f32 contact model / f64 integrate",
        "data": ("synthetic (seeded radii on an fcc lattice of 1 mm nearest-neighbour distance: a "
                 "compressed packing, at rest)" if dense else
                 "synthetic (seeded random non-overlapping spheres, at rest)"),
        "config": {"workload": f"{count} spheres r U[0.4,0.6] mm, 2500 kg/m^3, box {box[0]*1e3:.1f} x "
                               f"{box[1]*1e3:.1f} x {box[2]*1e3:.1f} mm periodic x,y, "
                               f"{'planes z=0 and z=top' if dense else 'plane z=0'}, gravity, kn 1e5 N/m, "
                               "e 0.7, kt = kappa kn (nu 0.22), Coulomb mu 0.5 with history, dt 1e-6 s",
                   "spheres": count},
        "mixed": mixed, "fp64": fp64, "speedup_mixed_vs_fp64": mixed["value"] / fp64["value"],
        "gpu_launches": mixed["launches"], "clocks": clk, "cpu_baseline": cpu,
    }
    print(json.dumps(line))


# ------------------------------------------------------------------------------ reference arm

def run_reference(args, rank, world, dist):
    if rank != 0:
        return
    from pairs_gb300 import lattice
    wl = WORKLOADS[args.workload]
    st = lattice.copper_fcc_lattice(*wl["n"])
    n = len(st["mass"])
    from oracle import lj as olj
    nth = os.cpu_count() or 1
    sim = olj.Sim(st, every=20, exact_sync=True, nthreads=nth)
    sim.run(args.warmup)
    budget = args.reference_budget_s
    t0 = time.perf_counter()
    done = 0
    while done < args.steps:
        sim.step()
        done += 1
        if time.perf_counter() - t0 > budget:
            break
    el = time.perf_counter() - t0
    v = n * done / el
    line = {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": done, "warmup": args.warmup,
        "ms_per_step": el * 1e3 / done, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (fcc lattice, Park-Miller velocities as the reference)",
        "config": {"workload": f"LJ fcc {wl['n'][0]}x{wl['n'][1]}x{wl['n'][2]} = {n} atoms, rho 0.8442, T 1.44, "
                               "rc 2.5, skin 0.3, dt 0.005, reference CPU algorithm (FP64, ghosts), "
                               "rebuild every 20", "atoms": n},
        "impl": "reference",
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": nth, "kind": "port",
                         "sample": f"{done} MD steps of the full system, oracle/lj_oracle.c, OpenMP {nth} threads"
                                   + (f", stopped at the {budget:.0f} s budget" if done < args.steps else "")},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["ensemble", "dem", "dem-dense"], default="lj64")
    ap.add_argument("--dem-spheres", type=int, default=1000000, help="dem workload: number of spheres")
    ap.add_argument("--replicas", type=int, default=512, help="ensemble workload: number of replicas")
    ap.add_argument("--ensemble-layout", default="",
                    help="ensemble workload: fixed layout 'tpa,block,reach,half' (half 0 full, 1 half, "
                         "2 pair-cluster half lists) instead of the autotuner's")
    ap.add_argument("--ensemble-full-rebuilds", action="store_true",
                    help="ensemble workload: rebuild every replica at each trip (default: the selected ones)")
    ap.add_argument("--ensemble-select", type=float, default=0.6,
                    help="ensemble workload: partial rebuilds take the replicas displaced by this x skin/2")
    ap.add_argument("--ensemble-persistent", action="store_true",
                    help="ensemble workload: each chunk's plain steps in one persistent launch")
    ap.add_argument("--one-by-one-steps", type=int, default=100,
                    help="ensemble workload: steps per replica of the one-by-one comparison")
    ap.add_argument("--cpu-steps", type=int, default=40)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--reference-budget-s", type=float, default=120.0)
    ap.add_argument("--variant", choices=["mixed-half", "mixed-full", "fp64-half", "fp64-full"],
                    default="mixed-half")
    ap.add_argument("--policy", default="learned", help="rebuild policy: learned | guard | fixed | interval:k")
    ap.add_argument("--drift-steps", type=int, default=1000)
    ap.add_argument("--tiles", choices=["auto", "on", "off"], default="auto",
                    help="mixed path, full lists: 16-bit shared-memory tile lists or global lists (auto = off)")
    ap.add_argument("--tile-tpa", type=int, default=2, choices=[1, 2, 4],
                    help="threads per atom of the tile force kernel")
    ap.add_argument("--pair-lists", choices=["auto", "on", "off"], default="auto",
                    help="pair-cluster half lists on the mixed fixed-point path (auto: the engine's default)")
    ap.add_argument("--fixed-point", choices=["auto", "on", "off"], default="auto",
                    help="FP32 position layout: fixed point (2^32 units per box length, one 16-byte record "
                         "per partner) or compensated hi/lo pairs (auto = fixed point where the box allows)")
    ap.add_argument("--only-headline", action="store_true",
                    help="time the headline arm only (profiling runs)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    dist, rank, world, _ = dist_setup()
    if args.impl == "reference":
        run_reference(args, rank, world, dist)
    elif args.workload == "ensemble":
        run_ensemble(args, rank, world, dist)
    elif args.workload in ("dem", "dem-dense"):
        run_dem(args, rank, world, dist)
    else:
        run_ours(args, rank, world, dist)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
