"""The full 1,000,000-trajectory N2 + N configuration (the benchmark workload) through the public host
entry point, checked by properties that do not depend on size (the oracle cannot follow a million
trajectories): every trajectory ends at the end of the collision and conserves energy, every initial
point analyses back to its work item's level, the statistics count every row once, and each item's
cross sections add up to pi bmax^2 exactly (the total probability)."""
import os
import sys

import numpy as np
import pytest

from coarseair_gb300 import api

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_million_trajectories_properties(gpu_lib):
    sys.path.insert(0, ROOT)
    import bench
    table, items = bench.workload(1000000)
    cfg = bench.config()
    H = api.Handle(cfg)
    rows = api.RunTrajectories(H).run(table, items)
    assert len(rows) == 1000000
    assert np.all(rows["status"] == 0)
    assert np.max(np.abs(rows["dH"])) <= cfg.ham_abs_tol
    # initial points: the item's (v, J) and the target pair
    J, v, arr = api.histogram_assign(rows["j_i"], rows["v_i"], rows["arr_i"])
    lv = table[items["ilevel"][rows["item"]]]
    agree = (J == lv["jqn"]) & (v == lv["vqn"]) & (arr // 16 == 1)   # pair 1-2, bound or quasi-bound
    print("initial (v, J) recovered on %.5f of 1M trajectories" % agree.mean())
    assert agree.mean() >= 0.999
    st = api.Statistics(H, pres_even_odd=(1, 0, 0)).compute(items, rows)
    for i in range(len(items)):
        g = st[st["run"] == i]
        assert g["count"].sum() == g["nrows"][0] == items["ntraj"][i]
        assert g["cross"].sum() == pytest.approx(np.pi * items["bmax"][i] ** 2, rel=1e-12)
    H.close()
