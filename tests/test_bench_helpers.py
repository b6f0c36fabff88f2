"""bench.py's host-side helpers on the CPU: the per-FMM-step roofline of a
workload (the reference's flop split and algorithmic bytes) and the peaks it
divides by."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_phase_roofline_single_vector():
    sys.path.insert(0, REPO)
    import bench

    N, maxs = 1 << 20, 64
    wl = bench.Workload("single", N, maxs, 1)
    L, s = 12, 64
    Nb = (2 << L) - (L + 2)
    phases = {k: {"ms_per_step": 0.1, "launches_per_step": 2.0}
              for k in ("gather", "near", "leaf_up", "tree_up", "far", "tree_down", "leaf_down")}
    r = bench.phase_roofline(wl, L, s, Nb, phases, 1.0, 6800.0, 0)
    assert set(r) == set(phases)
    # the step's flops add up to the reference's count for L2C + C2L
    K = 2 * ((2 << (L - 1)) - 1)
    total = sum(v["fp64_tflops"] for v in r.values()) * 1e12 * 0.1e-3
    assert total > 2 * 4 * K * s * 18  # leaf products alone
    # the far-field step reads its A blocks (60.7 B per coefficient) once per call
    assert r["far"]["alg_gbs"] * 1e9 * 0.1e-3 >= 2 * 3 * Nb * 324 * 8
    # nodal trees cost four times the modal ones
    rn = bench.phase_roofline(wl, L, s, Nb, phases, 1.0, 6800.0, 1)
    assert rn["tree_up"]["fp64_tflops"] == pytest.approx(4 * r["tree_up"]["fp64_tflops"], rel=1e-3)


def test_hbm_peak_source():
    sys.path.insert(0, REPO)
    import bench

    v, src = bench.hbm_peak_gbs()
    assert v > 1000 and ("measured" in src or "fallback" in src)


def test_autotune_record():
    """autotune_plan tunes each direction the workload calls once and reports
    the choices and timings the plan gives back."""
    sys.path.insert(0, REPO)
    import bench

    class FakePlan:
        def __init__(self):
            self.tuned = []

        def autotune(self, d, count, dist, stride):
            self.tuned.append((d, count, dist, stride))
            return 0.5 + d

        def tuned_config(self, d, count, dist, stride):
            return ("tuned", f"overlap=1 dir={d}", 0.5 + d, 0.6 + d)

    p = FakePlan()
    calls = [(0, "u", "o0"), (1, "o0", "o1"), (0, "u", "o2")]
    rec = bench.autotune_plan(p, calls, 4096, 1024)
    assert p.tuned == [(0, 4096, 1024, 1), (1, 4096, 1024, 1)]
    assert rec["shapes"]["L2C"] == {"choices": "overlap=1 dir=0", "ms_per_call": 0.5,
                                    "ms_per_call_default": 0.6}
    assert rec["shapes"]["C2L"]["ms_per_call"] == 1.5 and rec["seconds"] >= 0
