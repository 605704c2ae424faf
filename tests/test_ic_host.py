"""The initial-condition stream code of the library (item_draws and impact_parameter in
coarseair_gb300/csrc/cair_ic.cuh, which k_ic_draws and the sampling kernels run on the GPU) run on
the host through an internal hook: every trajectory's impact parameter -- which depends on the
position of its draw in the stream -- equals the oracle's for impact-parameter rings of every strata
type, a fixed-b ring that draws nothing, and the earlier rings skipped, for diatom + atom and
diatom + diatom."""
import ctypes as C

import numpy as np
import pytest

from coarseair_gb300 import _lib, api, systems

RINGS = ([-2.0, -4.5, 3.0, -7.0], [1, 2, 1, 3])


def _host_b(path, natoms, table, items):
    L = C.CDLL(path)
    f = L.cair_internal_ic_draws
    f.restype = C.c_int
    f.argtypes = [C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                  C.c_void_p]
    ntot = int(items["ntraj"].sum())
    draws = np.zeros(10 * ntot)
    item_of = np.zeros(ntot, np.int32)
    b = np.zeros(ntot)
    assert f(natoms, len(table), table.ctypes.data, len(items), items.ctypes.data, ntot, draws.ctypes.data,
             item_of.ctypes.data, b.ctypes.data) == 0
    return b, item_of


def _oracle_levels(rows):
    out = np.zeros(len(rows), dtype=[(c, "f8") for c in ("vqn", "jqn", "eint", "egam", "rmin", "rmax", "vmin", "vmax",
                                                          "tau", "ri", "ro", "rlim")])
    for c in out.dtype.names:
        out[c] = rows[c] if c in rows.dtype.names else 0.0
    return out


@pytest.mark.parametrize("strata", ["Circles", "Rings", "Segments"])
def test_rings_continue_one_stream_diatom_atom(gpu_lib, oracle_lib, strata):
    from oracle import Oracle
    cfg = systems.n3_config()
    o = Oracle(cfg)
    rows = systems.load_levels("N2")[[17]]
    n, seed = 71, api.process_seed(4, 1)
    items = api.work_items(api.ring_entries(0, 0, n, seed, 1e4, 15.0, *RINGS, strata=strata))
    b, item_of = _host_b(gpu_lib, 3, api.level_table(rows), items)
    ref = o.sample_ics(n, _oracle_levels(rows), seed=seed, ttra=1e4, dinit=15.0,
                       rings=(RINGS[0], RINGS[1], api.STRATA[strata]))
    assert list(item_of) == list(np.repeat(np.arange(4), [11, 20, 10, 30]))
    assert np.allclose(b, ref["b"], rtol=1e-14, atol=1e-300)
    assert np.all(b[31:41] == 3.0)


def test_rings_continue_one_stream_diatom_diatom(gpu_lib, oracle_lib):
    from oracle import Oracle
    cfg = systems.o4_config()
    o = Oracle(cfg)
    lv = systems.load_levels("O2")
    rows = lv[[0, 40]]
    n, seed = 60, api.process_seed(2, 1)
    items = api.work_items(api.ring_entries(0, 1, n, seed, 1e4, 18.0, [-3.0, -8.0], [1, 2], strata="Rings",
                                            ilevel2=1))
    b, _ = _host_b(gpu_lib, 4, api.level_table(rows), items)
    ref = o.sample_ics4(n, _oracle_levels(rows)[0], _oracle_levels(rows)[1], ttra=1e4, dinit=18.0, seed=seed,
                        rings=([-3.0, -8.0], [1, 2], 1))
    assert np.allclose(b, ref["b"], rtol=1e-14, atol=1e-300)
    assert np.all(b[:20] <= 3.0) and np.all((b[20:] >= 3.0) & (b[20:] <= 8.0))


def test_one_ring_stream_matches_the_plain_path(gpu_lib, oracle_lib):
    """skip = 0, Circles, bmax > 0: the stream the queue tests and the bench use."""
    from oracle import Oracle
    o = Oracle(systems.o3_config())
    rows = systems.load_levels("O2")[[0, 1]]
    items = api.work_items([(0, 0, 30, api.process_seed(3, 1), 5000.0, 7.0, 15.0),
                            (1, 0, 25, api.process_seed(3, 2), 20000.0, 6.0, 15.0)])
    b, _ = _host_b(gpu_lib, 3, api.level_table(rows), items)
    r0 = o.sample_ics(30, _oracle_levels(rows[:1]), seed=api.process_seed(3, 1), ttra=5000.0, bmax=7.0, dinit=15.0)
    r1 = o.sample_ics(25, _oracle_levels(rows[1:]), seed=api.process_seed(3, 2), ttra=20000.0, bmax=6.0, dinit=15.0)
    assert np.allclose(b, np.concatenate([r0["b"], r1["b"]]), rtol=1e-14, atol=1e-300)
