"""The reference arm of bench.py times whole model evaluations, not a sample.

Its timed steps split the 220 triplets round robin: --steps 20 (the driver's run) cover
every triplet exactly once, so the reported rate is one measured evaluation per measured
time; other step counts cover whole passes where they can.  CPU only.
"""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_twenty_steps_cover_every_triplet_once():
    parts = bench.reference_steps(220, 20)
    assert len(parts) == 20
    flat = sorted(sum(parts, []))
    assert flat == list(range(220))
    assert {len(p) for p in parts} == {11}


def test_other_step_counts():
    for steps in (1, 3, 7, 220):
        parts = bench.reference_steps(220, steps)
        assert len(parts) == steps
        assert sorted(sum(parts, [])) == list(range(220))
    parts = bench.reference_steps(220, 300)  # more steps than triplets: passes repeat
    assert len(parts) == 300 and all(len(p) == 1 for p in parts)


def test_parity_summary():
    f64 = np.zeros(4, dtype=[("val", "f8"), ("neval", "u8"), ("status", "i4")])
    f64["val"] = [1.0, 2.0, -3.0, 4.0]
    f64["neval"] = [10, 20, 30, 40]
    mx = f64.copy()
    mx["val"] = [1.0, 2.0 * (1 + 2e-4), -3.0, 4.0 * (1 - 1e-6)]
    p = bench.parity(mx, f64)
    assert p["terms_over_1e-4"] == 1 and abs(p["max_rel"] - 2e-4) < 1e-12
    assert p["neval_identical"] and p["status_ok"]
    mx["neval"][2] += 1
    assert not bench.parity(mx, f64)["neval_identical"]
