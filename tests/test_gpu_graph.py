"""The queue path captured as a CUDA graph (cair_queue_graph_*): two replays write the same rows as
a direct cair_run_queue_dev call on the same inputs (the path is deterministic), and a replay after
the work items are rewritten in place runs the new batch."""
import ctypes

import numpy as np
import pytest

from coarseair_gb300 import _lib, api, systems

pytestmark = pytest.mark.gpu


def test_graph_replays_match_direct_call(gpu_lib):
    torch = pytest.importorskip("torch")
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    cfg = systems.n3_config(rmax=16.0)
    H = api.Handle(cfg)
    lib = H.lib
    lv = systems.load_levels("N2")
    table = api.level_table(lv[[7, 900]])
    items = api.work_items([(0, 0, 300, api.process_seed(6, 1), 10000.0, 7.0, 15.0),
                            (1, 0, 212, api.process_seed(6, 2), 20000.0, 7.0, 15.0)])
    n = int(items["ntraj"].sum())
    d_lv = torch.from_numpy(table.view(np.uint8).copy()).to(dev)
    d_it = torch.from_numpy(items.view(np.uint8).copy()).to(dev)
    size = n * _lib.RESULT_DTYPE.itemsize
    ws = torch.empty(int(lib.cair_queue_workspace_bytes(n)) + 256, dtype=torch.uint8, device=dev)
    wsp = (ws.data_ptr() + 255) & ~255
    stream = torch.cuda.current_stream().cuda_stream
    ref = torch.empty(size, dtype=torch.uint8, device=dev)
    H.check(lib.cair_run_queue_dev(H.h, len(table), d_lv.data_ptr(), len(items), d_it.data_ptr(), n,
                                   cfg.max_attempts, ref.data_ptr(), wsp, stream), "cair_run_queue_dev")
    torch.cuda.synchronize()
    ref_rows = np.frombuffer(ref.cpu().numpy().tobytes(), dtype=_lib.RESULT_DTYPE)
    out = torch.zeros(size, dtype=torch.uint8, device=dev)
    g = ctypes.c_void_p()
    H.check(lib.cair_queue_graph_create(H.h, len(table), d_lv.data_ptr(), len(items), d_it.data_ptr(), n,
                                        cfg.max_attempts, out.data_ptr(), wsp, ctypes.byref(g)),
            "cair_queue_graph_create")
    try:
        for _ in range(2):
            out.zero_()
            H.check(lib.cair_queue_graph_launch(H.h, g, stream), "cair_queue_graph_launch")
            torch.cuda.synchronize()
            rows = np.frombuffer(out.cpu().numpy().tobytes(), dtype=_lib.RESULT_DTYPE)
            assert rows.tobytes() == ref_rows.tobytes()
        # new seeds written into the captured work-item buffer: the replay runs the new batch
        items2 = items.copy()
        items2["seed"] = [api.process_seed(6, 3), api.process_seed(6, 4)]
        d_it.copy_(torch.from_numpy(items2.view(np.uint8).copy()).to(dev))
        H.check(lib.cair_queue_graph_launch(H.h, g, stream), "cair_queue_graph_launch")
        torch.cuda.synchronize()
        rows2 = np.frombuffer(out.cpu().numpy().tobytes(), dtype=_lib.RESULT_DTYPE)
        assert np.all(rows2["status"] == 0) and not np.array_equal(rows2["b"], ref_rows["b"])
    finally:
        lib.cair_queue_graph_destroy(g)
    with pytest.raises(api.CairError, match="workspace required"):
        H.check(lib.cair_queue_graph_create(H.h, len(table), d_lv.data_ptr(), len(items), d_it.data_ptr(), n,
                                            cfg.max_attempts, out.data_ptr(), None, ctypes.byref(g)),
                "cair_queue_graph_create")
    H.close()
