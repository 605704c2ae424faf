"""GPU test of the replicas' statistics entry points (cair_statistics_items / cair_statistics_counts and
the host cair_statistics_finish): the rows of one queue run split into two "replicas" -- one holding
every row of an item -- summed through the three steps give the lines of all rows together.
Collected after the validated test files (a newest GPU path)."""
import numpy as np
import pytest

from coarseair_gb300 import api, systems

pytestmark = pytest.mark.gpu


def test_replica_steps_on_the_gpu_give_the_statistics_of_all_rows(gpu_lib, oracle_lib):
    cfg = systems.n3_config(rmax=16.0)
    H = api.Handle(cfg)
    lv = systems.load_levels("N2")
    table = api.level_table(lv[[5, 300]])
    items = api.work_items([(0, 0, 200, api.process_seed(7, 1), 10000.0, 7.0, 15.0),
                            (0, 0, 200, api.process_seed(7, 2), 10000.0, 7.0, 15.0),
                            (1, 0, 200, api.process_seed(7, 3), 20000.0, 7.0, 15.0)])
    rows = api.RunTrajectories(H).run(table, items)
    runs = [0, 0, 1]
    st = api.Statistics(H, pres_even_odd=(1, 0, 0))
    part = [rows[(rows["item"] == 0) | ((rows["item"] == 2) & (np.arange(len(rows)) % 2 == 0))],
            rows[(rows["item"] == 1) | ((rows["item"] == 2) & (np.arange(len(rows)) % 2 == 1))]]
    totals = [st.replica_items(len(items), p) for p in part]
    ir = totals[0][0] + totals[1][0]
    ii = np.minimum(totals[0][1], totals[1][1])
    cs = [st.replica_counts(items, p, ir, ii, runs) for p in part]
    got = api.statistics_finish(st.params, items, ir, ii, np.concatenate([c[0] for c in cs]), cs[0][1] + cs[1][1],
                                runs)
    ref = st.compute(items, rows, runs=runs)
    assert len(got) == len(ref) and len(ref) > 0
    for f in ("run", "fin", "ini", "nrings", "count", "nrows"):
        assert np.array_equal(got[f], ref[f]), f
    for f in ("cross", "cross_sd", "rate", "rate_sd"):
        assert np.allclose(got[f], ref[f], rtol=1e-14, atol=0), f
    H.close()
