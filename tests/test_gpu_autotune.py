"""GPU test of the project's autotuner (cair_autotune): it measures every launch shape of the
persistent integrator on a capped sample of the job's own work items, keeps the fastest on the
handle, and the job's results do not depend on the shape (each trajectory's integration is its own
thread's, whatever block it runs in).  Also the warp timeline that measures the queue's tail."""
import numpy as np
import pytest

from coarseair_gb300 import api, systems

pytestmark = pytest.mark.gpu


def test_autotune_measures_every_shape_and_keeps_results(gpu_lib):
    torch = pytest.importorskip("torch")
    cfg = systems.n3_config(rmax=16.0)
    H = api.Handle(cfg)
    lv = systems.load_levels("N2")
    table = api.level_table(lv[[5, 300, 2000]])
    items = api.work_items([(k, 0, 800, api.process_seed(6, k + 1), T, 7.0, 15.0)
                            for k, T in ((0, 10000.0), (1, 5000.0), (2, 20000.0))])
    wt = torch.zeros(4 * 4096, dtype=torch.int64, device="cuda")
    H.check(H.lib.cair_set_warp_timeline(H.h, wt.data_ptr(), 4096), "cair_set_warp_timeline")
    before = api.RunTrajectories(H).run(table, items, max_attempts=4000)
    nw = int(H.lib.cair_warp_timeline_count(H.h))
    H.check(H.lib.cair_set_warp_timeline(H.h, None, 0), "cair_set_warp_timeline")
    t = wt[:4 * nw].cpu().numpy().reshape(-1, 4)
    assert nw == 2 * ((2400 + 63) // 64) and np.all(t[:, 1] >= t[:, 0]) and np.all(t[:, 0] > 0)
    # lane-blocks: at most 32 per block, and every trajectory's blocks are counted once
    att = before["iste"].astype(np.int64) + before["irej"]
    assert np.all(t[:, 2] <= 32 * t[:, 3]) and int(t[:, 2].sum()) == int(np.sum((att + cfg.ncall - 1) // cfg.ncall))
    (block, per_sm), pts = api.autotune(H, table, items, sample=1200, cap_attempts=100)
    print("autotune: chose block %d x %d per SM; points:" % (block, per_sm),
          [(int(p["block"]), int(p["per_sm"]), round(float(p["attempts_per_s"]) / 1e6, 2)) for p in pts])
    shapes = {(int(p["block"]), int(p["per_sm"])) for p in pts}
    assert {(32, 1), (64, 1), (128, 1)} <= shapes and len(shapes) == len(pts)
    best = pts[np.argmax(pts["attempts_per_s"])]
    assert (block, per_sm) == (int(best["block"]), int(best["per_sm"]))
    after = api.RunTrajectories(H).run(table, items, max_attempts=4000)
    for f in ("status", "iste", "irej"):
        assert np.array_equal(before[f], after[f]), f
    for f in ("j_f", "v_f", "arr_f", "t", "dH"):
        assert np.array_equal(before[f], after[f]), f
    H.close()
