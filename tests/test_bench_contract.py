"""bench.py on CPU: the roofline's DRAM traffic comes from the committed ncu summary
(profiles/traffic.txt), scaled to the workload by its atom count."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def load_bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_traffic_of_the_headline_kernel_is_recorded_and_scales():
    bench = load_bench()
    t1, ref = bench.traffic_from_profiles("k_lj_mixed", "mixed-half", 1048576)
    assert ref == 1048576 and t1 is not None and t1 > 0
    t8, _ = bench.traffic_from_profiles("k_lj_mixed", "mixed-half", 8 * 1048576)
    assert t8 == pytest.approx(8 * t1)
    assert bench.traffic_from_profiles("k_lj_mixed", "no-such-variant", 1048576) == (None, None)


def test_every_recorded_traffic_line_is_well_formed():
    with open(os.path.join(ROOT, "profiles", "traffic.txt")) as f:
        lines = [l.split() for l in f if l.strip()]
    assert lines
    for parts in lines:
        assert len(parts) == 4, parts
        assert int(parts[2]) > 0 and float(parts[3]) > 0
