"""Host-side pieces of bench.py that need no GPU: the outcome figures computed from a step's rows."""
import numpy as np

from coarseair_gb300 import _lib


def test_outcome_summary():
    import bench
    rows = np.zeros(6, dtype=_lib.RESULT_DTYPE)
    rows["iste"] = [8, 10, 300, 7, 500, 9]
    rows["irej"] = [2, 0, 5, 3, 0, 2]        # attempts 10, 10, 305, 10, 500, 11
    rows["status"] = [0, 1, 0, 0, 0, 0]
    rows["ipes"] = [0, 0, 1, 1, 2, 2]
    out = bench.outcome_summary(rows, 10)
    assert out["first_check_fraction"] == 2 / 6     # rows 0 and 3: finished at the first check
    assert out["per_surface"]["1"] == {"trajectories": 2, "attempts_per_trajectory": 157.5,
                                       "converged_fraction": 1.0}
    assert out["per_surface"]["0"]["converged_fraction"] == 0.5
    assert "per_surface" not in bench.outcome_summary(rows[:2], 10)
