"""Time-to-relMSE bookkeeping of nuray_gb300/convergence.py (CPU only)."""
import math

from nuray_gb300 import convergence as C


def test_crossing_interpolates_between_the_bracketing_checkpoints():
    # relMSE falling as 1 / time: the log-log interpolation is exact
    curve = [(t, int(t), 10.0 / t) for t in (1000.0, 2000.0, 4000.0, 8000.0)]
    x = C.crossing(curve, 10.0 / 3000.0)
    assert math.isclose(x, 3000.0, rel_tol=1e-12)
    # a checkpoint exactly on the target is its own crossing
    assert math.isclose(C.crossing(curve, 10.0 / 4000.0), 4000.0, rel_tol=1e-12)


def test_crossing_absent_when_the_curve_stays_above_or_starts_below():
    curve = [(100.0, 64, 2e-3), (200.0, 128, 1.5e-3)]
    assert C.crossing(curve, 1e-3) is None
    assert C.crossing([(100.0, 64, 5e-4), (200.0, 128, 4e-4)], 1e-3) is None


def test_summary_keeps_the_checkpoint_time_and_adds_the_crossing():
    curve = [(7803.01, 4160, 1.028e-3), (8036.57, 4288, 1.008e-3), (8270.03, 4416, 0.9897e-3)]
    s = C.summary(curve, 8270.03)
    assert s["ms_to_target"] == 8270.0 and s["spp"] == 4416
    assert 8036.57 < s["ms_to_target_interp"] < 8270.03
    assert C.summary(curve[:2], None)["ms_to_target_interp"] is None
