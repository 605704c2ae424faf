"""The allocation-free queue entry point (cair_run_queue_static_dev).

Callers that cannot allocate device memory while they run -- a host whose GPU memory is handed out
by its own pool at start-up, or code that must not trigger cudaMalloc's implicit synchronisation --
use this variant: its batch state lives in a static device array inside the library.  This test
calls it twice in a row through the C ABI and checks both results against the regular entry point
(cair_run_queue_dev) on the same work items, with the tolerance of the other GPU tests (exact
integers, 1e-12 relative for the floating-point fields; the kernels are the same, so the rows are
expected to be identical).  It also checks that a batch beyond the static capacity is rejected.
Collected after the other tests (only the N4 PIPNN file follows it) so that a run that stops at the first
failure has run them.
"""

import numpy as np
import pytest

from coarseair_gb300 import _lib, api, systems

pytestmark = pytest.mark.gpu


def _device_inputs(torch, table, items, n):
    dev = torch.device("cuda", 0)
    d_lv = torch.from_numpy(table.view(np.uint8).copy()).to(dev)
    d_it = torch.from_numpy(items.view(np.uint8).copy()).to(dev)
    return d_lv, d_it, dev


def _rows(torch_buf):
    return np.frombuffer(torch_buf.cpu().numpy().tobytes(), dtype=_lib.RESULT_DTYPE)


def _assert_same(a, b):
    for f in ("idx", "item", "ipes", "status", "iste", "irej"):
        np.testing.assert_array_equal(a[f], b[f])
    for f in ("bmax", "b", "j_i", "v_i", "arr_i", "j_f", "v_f", "arr_f", "t", "dH"):
        assert np.allclose(a[f], b[f], rtol=1e-12, atol=1e-300), f


def test_static_queue_matches_regular_entry_point(gpu_lib):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    torch.cuda.set_device(0)
    cfg = systems.n3_config(rmax=16.0)
    H = api.Handle(cfg)
    lib = H.lib
    lv = systems.load_levels("N2")
    table = api.level_table(lv[[5, 300]])
    items = api.work_items([(0, 0, 700, api.process_seed(4, 1), 10000.0, 7.0, 15.0),
                            (1, 0, 500, api.process_seed(4, 2), 5000.0, 7.0, 15.0)])
    n = int(items["ntraj"].sum())
    d_lv, d_it, dev = _device_inputs(torch, table, items, n)
    size = n * _lib.RESULT_DTYPE.itemsize
    ref_buf = torch.empty(size, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    H.check(lib.cair_run_queue_dev(H.h, len(table), d_lv.data_ptr(), len(items), d_it.data_ptr(), n,
                                   cfg.max_attempts, ref_buf.data_ptr(), None, stream), "cair_run_queue_dev")
    torch.cuda.synchronize()
    ref = _rows(ref_buf)
    assert np.all(ref["status"] == 0)
    for call in range(2):
        out_buf = torch.zeros(size, dtype=torch.uint8, device=dev)
        H.check(lib.cair_run_queue_static_dev(H.h, len(table), d_lv.data_ptr(), len(items), d_it.data_ptr(), n,
                                              cfg.max_attempts, out_buf.data_ptr(), stream),
                "cair_run_queue_static_dev (call %d)" % (call + 1))
        torch.cuda.synchronize()
        _assert_same(_rows(out_buf), ref)
    # beyond the static capacity: a clear error, nothing launched
    big = _lib.CAIR_STATIC_QUEUE_MAX_TRAJ + 1
    rc = lib.cair_run_queue_static_dev(H.h, len(table), d_lv.data_ptr(), len(items), d_it.data_ptr(), big,
                                       cfg.max_attempts, out_buf.data_ptr(), stream)
    assert rc == 1 and b"static workspace" in lib.cair_last_error(H.h)
    H.close()
