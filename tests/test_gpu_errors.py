"""Error paths of the C ABI on a GPU: malformed systems are refused at cair_create with a message,
bad work items are refused before any launch, and a handle keeps working after a refused call
(the reference's print-and-stop becomes an error code the caller can act on)."""
import ctypes as C

import numpy as np
import pytest

from coarseair_gb300 import _lib, api, systems

pytestmark = pytest.mark.gpu


def _create(cfg, mutate):
    """cair_create on a system description that `mutate` edits; returns (rc, message)."""
    lib = _lib.load()
    desc, keep = api.system_desc(cfg)
    mutate(desc)
    h = C.c_void_p()
    rc = lib.cair_create(C.byref(h), C.byref(desc))
    msg = lib.cair_last_error(h).decode() if h.value else ""
    if h.value:
        lib.cair_destroy(h)
    return rc, msg


def test_malformed_systems_are_refused(gpu_lib):
    cfg = systems.o3nn_config()
    rc, _ = _create(cfg, lambda d: setattr(d.pes[0], "ncoef", d.pes[0].ncoef - 1))
    assert rc == 1
    rc, _ = _create(systems.n3_config(), lambda d: setattr(d, "natoms", 4))
    assert rc == 1
    rc, _ = _create(systems.n3_config(), lambda d: setattr(d, "abi_version", 1))
    assert rc == 1
    rc, _ = _create(systems.n3_config(), lambda d: setattr(d, "npes", 17))
    assert rc == 1


def test_bad_items_are_refused_and_the_handle_survives(gpu_lib):
    cfg = systems.n3_config(rmax=16.0)
    H = api.Handle(cfg)
    lv = systems.load_levels("N2")
    table = api.level_table(lv[[3]])
    bad_level = api.work_items([(1, 0, 10, 3, 10000.0, 7.0, 15.0)])
    with pytest.raises(api.CairError, match="level out of range"):
        api.RunTrajectories(H).run(table, bad_level)
    too_wide = api.work_items([(0, 0, 10, 3, 10000.0, 16.0, 15.0)])
    with pytest.raises(api.CairError, match="Dinit"):
        api.RunTrajectories(H).run(table, too_wide)
    bad_pes = api.work_items([(0, 2, 10, 3, 10000.0, 7.0, 15.0)])
    with pytest.raises(api.CairError, match="surface out of range"):
        api.RunTrajectories(H).run(table, bad_pes)
    ok = api.work_items([(0, 0, 16, 3, 10000.0, 7.0, 15.0)])
    rows = api.RunTrajectories(H).run(table, ok)
    assert np.all(rows["status"] == 0) and len(rows) == 16
    st = api.Statistics(H, qn_max=2)            # every J >= 2 is beyond QuantumNumberMax
    with pytest.raises(api.CairError, match="qn_max"):
        st.compute(ok, rows)
    H.close()
