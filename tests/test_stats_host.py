"""The device statistics' logic on the CPU, without a GPU.  The two device passes are restated here in
numpy from Statistics_Class.F90 -- IdentifyInitialStates (591-680), AddFinState's Histogram codes
(935-1282) and its ring assignment.  The library's own per-row device code (stats_counted,
stats_codes, stats_key, run on the host through an internal hook) must give the same codes, rings
and keys, and the counted (run, final state, ring) keys go through the library's host half
(coarseair_gb300/csrc/cair_stats_host.cpp: SetRings per run, key decoding, WriteFinStateProbabilities
over the rings); the lines must equal the oracle's statistics of each run's rows.  The same rows as
the GPU statistics tests, plus pooled runs."""
import ctypes as C

import numpy as np
import pytest

from coarseair_gb300 import _lib, systems

MAXR = 64
_P, _I32, _I64 = C.c_void_p, C.c_int32, C.c_int64


def _load(path):
    """The library with the host half's two internal entry points declared."""
    L = C.CDLL(path)
    L.cair_internal_stats_rings.restype = C.c_int
    L.cair_internal_stats_rings.argtypes = [C.POINTER(_lib.StatsParams), _I32, _P, _P, _P, _P, _P, _P,
                                            C.POINTER(_I32), C.POINTER(_I32), C.c_char_p, C.c_int]
    L.cair_internal_stats_rows.restype = C.c_int
    L.cair_internal_stats_rows.argtypes = [C.POINTER(_lib.StatsParams), _I32, _P, _P, _P, _P, _I64, _P, _P, _P, _P,
                                           _P, _P]
    L.cair_internal_stats_finish.restype = C.c_int
    L.cair_internal_stats_finish.argtypes = [C.POINTER(_lib.StatsParams), _I32, _P, _P, _P, _P, _I64, _P, _P, _P, _P,
                                             _I64, C.POINTER(_I64), C.c_char_p, C.c_int]
    return L


def _nint(x):
    return np.where(x >= 0, np.floor(x + 0.5), np.ceil(x - 0.5)).astype(np.int64)


def _codes(qi, qf, iskip, pres, qnmax):
    """Initial- and final-state codes of every row (Fortran nint, mod with the dividend's sign)."""
    qi, qf = qi.astype(np.float64).copy(), qf.astype(np.float64).copy()
    nc = qi.shape[1]
    ipi = np.trunc((qi[:, -1] - 0.49) / 16).astype(np.int64)
    ipf = np.trunc((qf[:, -1] - 0.49) / 16).astype(np.int64)
    ini_code = np.zeros(len(qi), np.int64)
    fin_code = np.zeros(len(qi), np.int64)
    ifact = 1
    for c in range(nc):
        ini = _nint(qi[:, c] - 0.5)
        raw = qf[:, c].copy()
        q = qf[:, c] - 0.5
        if pres[c]:
            m = ipi == ipf
            odd = m & (np.fmod(ini, 2) == 1)
            q = np.where(odd, q - 1.0, q)
            q = np.where(odd & (_nint(q * 0.5) < 0) & (raw > 0.0), q + 2.0, q)
            q = np.where(m, q * 0.5, q)
        ini_code += (ini + 2 if iskip[c] else 2) * ifact
        iquse = _nint(q) * iskip[c]
        iquse = np.where(iquse + 2 > qnmax, 0, iquse)
        if iskip[c] or c == nc - 1:
            fin_code += (iquse + 2) * ifact
        ifact *= qnmax
    return ini_code, fin_code


def _host_statistics(L, P, items, rows, runs, keep, nc):
    """Restated device passes + the library's host half."""
    names = ("j", "v", "arr") if nc == 3 else ("j", "v", "j2", "v2", "arr")
    qi = np.stack([rows[n + "_i"] for n in names], 1)
    qf = np.stack([rows[n + "_f"] for n in names], 1)
    ic, fc = _codes(qi, qf, list(P.iskip)[:nc], list(P.pres_even_odd)[:nc], P.qn_max)
    nitems = len(items)
    it = rows["item"]
    item_rows = np.bincount(it[keep], minlength=nitems).astype(np.uint64)
    item_ini = np.full(nitems, np.iinfo(np.int64).max, np.int64)
    np.minimum.at(item_ini, it[keep], ic[keep])
    run_arr = None if runs is None else np.ascontiguousarray(runs, np.int32)
    run_of = np.arange(nitems) if runs is None else np.asarray(runs)
    ring_b = np.zeros(nitems * MAXR)
    nring = np.zeros(nitems, np.int32)
    R, nruns = C.c_int32(), C.c_int32()
    err = C.create_string_buffer(256)
    itc = np.ascontiguousarray(items, dtype=_lib.ITEM_DTYPE)
    assert L.cair_internal_stats_rings(C.byref(P), nitems, itc.ctypes.data,
                                       None if run_arr is None else run_arr.ctypes.data, item_rows.ctypes.data,
                                       item_ini.ctypes.data, ring_b.ctypes.data, nring.ctypes.data, C.byref(R),
                                       C.byref(nruns), err, 256) == 0, err.value
    R, nruns = R.value, nruns.value
    rr = run_of[it]
    ring = np.zeros(len(rows), np.int64)
    for k in np.flatnonzero(keep):
        e = ring_b[rr[k] * MAXR: rr[k] * MAXR + nring[rr[k]]]
        for q in range(len(e) - 1):
            if not (rows["b"][k] > e[q + 1] or rows["b"][k] <= e[q]):
                ring[k] = q + 1
                break
    # the library's per-row device code (run on the host) gives the same codes, rings and keys
    rws = np.ascontiguousarray(rows, dtype=_lib.RESULT_DTYPE)
    d_cnt, d_ic, d_fc = np.zeros(len(rows), np.int32), np.zeros(len(rows), np.int64), np.zeros(len(rows), np.int64)
    d_ring, d_key = np.zeros(len(rows), np.int32), np.zeros(len(rows), np.uint64)
    assert L.cair_internal_stats_rows(C.byref(P), nitems, itc.ctypes.data,
                                      None if run_arr is None else run_arr.ctypes.data, item_rows.ctypes.data,
                                      item_ini.ctypes.data, len(rws), rws.ctypes.data, d_cnt.ctypes.data,
                                      d_ic.ctypes.data, d_fc.ctypes.data, d_ring.ctypes.data, d_key.ctypes.data) == 0
    full_key = (fc * nruns + rr) * R + ring
    assert np.array_equal(d_cnt.astype(bool), keep)
    assert np.array_equal(d_ic[keep], ic[keep]) and np.array_equal(d_fc[keep], fc[keep])
    assert np.array_equal(d_ring[keep], ring[keep])
    assert np.array_equal(d_key[keep], full_key[keep].astype(np.int64).view(np.uint64))
    key = full_key[keep]
    uk, cnt = np.unique(key, return_counts=True)
    ring_rows = np.bincount((rr * MAXR + ring)[keep], minlength=nruns * MAXR).astype(np.uint64)
    ukc = np.ascontiguousarray(uk.astype(np.int64).view(np.uint64))
    cntc = np.ascontiguousarray(cnt.astype(np.uint64))
    out = np.zeros(max(64, len(rows)), dtype=_lib.FINAL_STATE_DTYPE)
    n = C.c_int64()
    assert L.cair_internal_stats_finish(C.byref(P), nitems, itc.ctypes.data,
                                        None if run_arr is None else run_arr.ctypes.data, item_rows.ctypes.data,
                                        item_ini.ctypes.data, len(ukc), ukc.ctypes.data, cntc.ctypes.data,
                                        ring_rows.ctypes.data, out.ctypes.data, len(out), C.byref(n), err, 256) == 0, \
        err.value
    return out[:n.value]


def _params(nc, pres, xmu, qn=300):
    p = _lib.StatsParams()
    p.qn_max, p.ncond = qn, nc
    for i in range(5):
        p.iskip[i] = 1 if i < nc else 0
        p.pres_even_odd[i] = int(pres[i]) if i < nc else 0
    p.ham_abs_tol, p.xmu = 1e-5, xmu
    return p


def _check(L, items, rows, pres, nc, xmu, runs=None):
    import oracle
    P = _params(nc, pres, xmu)
    keep = (rows["status"] == 0) & (np.abs(rows["dH"]) <= P.ham_abs_tol)
    got = _host_statistics(L, P, items, rows, runs, keep, nc)
    assert np.all(got["fin"][:, nc:] == 0) and np.all(got["ini"][:, nc:] == 0)
    names = ("j", "v", "arr") if nc == 3 else ("j", "v", "j2", "v2", "arr")
    run_of = np.arange(len(items)) if runs is None else np.asarray(runs)
    rr = run_of[rows["item"]]
    for run in np.unique(run_of):
        sel = keep & (rr == run)
        g = got[got["run"] == run]
        if sel.sum() == 0:
            assert len(g) == 0
            continue
        ref, ini = oracle.statistics(rows["bmax"][sel], rows["b"][sel],
                                     np.stack([rows[n + "_i"][sel] for n in names], 1),
                                     np.stack([rows[n + "_f"][sel] for n in names], 1),
                                     iskip=(1,) * nc, pres=pres[:nc], cap=max(64, int(sel.sum())))
        assert len(g) == len(ref)
        gd = {tuple(int(x) for x in r["fin"][:nc]): r for r in g}
        vel = oracle.mean_velocity(items["ttra"][run_of == run][0], xmu)
        for fs, n, cross, sd in ref:
            r = gd[fs]
            assert tuple(int(x) for x in r["ini"][:nc]) == ini
            assert r["count"] == n and r["nrows"] == sel.sum() and r["nrings"] == len(np.unique(rows["bmax"][sel]))
            assert r["cross"] == pytest.approx(cross, rel=1e-14)
            assert r["cross_sd"] == pytest.approx(sd, rel=1e-14, abs=1e-300)
            assert r["rate"] == pytest.approx(cross * vel, rel=1e-13)
    return got


def _xmu(masses):
    mt, mp = masses[0] + masses[1], sum(masses[2:])
    return mt * mp / (mt + mp)


def test_three_conditions_one_run_per_item(gpu_lib, oracle_lib):
    L = _load(gpu_lib)
    rng = np.random.default_rng(21)
    n, nitems = 20000, 5
    rows = np.zeros(n, dtype=_lib.RESULT_DTYPE)
    rows["item"] = rng.integers(0, nitems, n)
    rows["j_i"] = 10.5 + 2.0 * rows["item"]
    rows["v_i"] = 0.5 + rows["item"] % 2
    rows["arr_i"] = 16.5
    rows["j_f"] = rng.uniform(0.0, 60.0, n)
    rows["v_f"] = rng.uniform(-1.5, 12.0, n)
    rows["arr_f"] = rng.choice([16.5, 17.5, 18.5, 32.5, 48.5], n)
    rows["b"] = rng.uniform(0.0, 6.0, n)
    rows["bmax"] = 6.0
    rows["status"] = np.where(rng.uniform(size=n) < 0.01, 1, 0)
    rows["dH"] = np.where(rng.uniform(size=n) < 0.01, 1.0, 1e-9)
    items = np.zeros(nitems, dtype=_lib.ITEM_DTYPE)
    items["bmax"] = 6.0
    items["ttra"] = [5000.0, 10000.0, 15000.0, 20000.0, 8000.0]
    xmu = _xmu(systems.o3_config().masses)
    _check(L, items, rows, (1, 0, 0, 0, 0), 3, xmu)
    _check(L, items, rows, (0, 0, 0, 0, 0), 3, xmu)


def test_five_conditions_with_clusters(gpu_lib, oracle_lib):
    L = _load(gpu_lib)
    rng = np.random.default_rng(33)
    n, nitems = 20000, 4
    rows = np.zeros(n, dtype=_lib.RESULT_DTYPE)
    rows["item"] = rng.integers(0, nitems, n)
    rows["j_i"] = 1.5 + 2.0 * rows["item"]
    rows["v_i"] = 0.5
    rows["j2_i"] = 3.5 + 4.0 * (rows["item"] % 2)
    rows["v2_i"] = 0.5 + (rows["item"] >= 2)
    rows["arr_i"] = 26.5
    arr = rng.choice([26.5, 42.5, 58.5, 22.5, 18.5, 17.5, -65.5], n)
    for c in ("j_f", "v_f", "j2_f", "v2_f"):
        rows[c] = np.where(arr == -65.5, -0.5, rng.uniform(-1.0, 40.0 if c[0] == "j" else 8.0, n))
    rows["arr_f"] = arr
    rows["b"] = rng.uniform(0.0, 8.0, n)
    rows["bmax"] = 8.0
    rows["status"] = np.where(rng.uniform(size=n) < 0.01, 1, 0)
    rows["dH"] = 1e-9
    items = np.zeros(nitems, dtype=_lib.ITEM_DTYPE)
    items["bmax"] = 8.0
    items["ttra"] = [5000.0, 10000.0, 15000.0, 20000.0]
    xmu = _xmu(systems.o4_config().masses)
    got = _check(L, items, rows, (1, 0, 1, 0, 0), 5, xmu)
    assert np.any(got["fin"][:, 4] < 0)
    _check(L, items, rows, (0, 0, 0, 0, 0), 5, xmu)


def test_pooled_runs_with_rings_and_an_empty_ring(gpu_lib, oracle_lib):
    """Run 0: items with bmax 2, 4, 6 (Circles: each samples its whole disc) where the 4-bohr item
    has no counted rows, so its ring is not one of the run's; run 1: two items of one bmax."""
    L = _load(gpu_lib)
    rng = np.random.default_rng(5)
    bm = [2.0, 4.0, 6.0, 5.0, 5.0]
    counts = [3000, 4000, 6000, 3000, 3000]
    n = sum(counts)
    rows = np.zeros(n, dtype=_lib.RESULT_DTYPE)
    rows["item"] = np.repeat(np.arange(5), counts)
    rows["bmax"] = np.repeat(bm, counts)
    rows["b"] = rows["bmax"] * np.sqrt(rng.uniform(size=n))
    rows["j_i"], rows["v_i"], rows["arr_i"] = 20.5, 0.5, 16.5
    rows["j_f"] = rng.uniform(0.0, 45.0, n)
    rows["v_f"] = rng.uniform(-0.5, 6.0, n)
    rows["arr_f"] = rng.choice([16.5, 17.5, 32.5, 48.5], n)
    rows["dH"] = np.where(rows["item"] == 1, 1.0, 1e-9)
    items = np.zeros(5, dtype=_lib.ITEM_DTYPE)
    items["bmax"] = bm
    items["ttra"] = 10000.0
    got = _check(L, items, rows, (1, 0, 0, 0, 0), 3, _xmu(systems.n3_config().masses), runs=[0, 0, 0, 1, 1])
    assert set(got[got["run"] == 0]["nrings"]) == {2} and set(got[got["run"] == 1]["nrings"]) == {1}


def test_items_of_a_run_must_share_the_temperature(gpu_lib):
    L = _load(gpu_lib)
    items = np.zeros(2, dtype=_lib.ITEM_DTYPE)
    items["bmax"], items["ttra"] = 5.0, [1e4, 2e4]
    P = _params(3, (0,) * 5, 1.0)
    err = C.create_string_buffer(256)
    z = np.zeros(2, np.uint64)
    ini = np.zeros(2, np.int64)
    ring_b, nring, R, nr = np.zeros(2 * MAXR), np.zeros(2, np.int32), C.c_int32(), C.c_int32()
    runs = np.zeros(2, np.int32)
    rc = L.cair_internal_stats_rings(C.byref(P), 2, items.ctypes.data, runs.ctypes.data, z.ctypes.data, ini.ctypes.data,
                                     ring_b.ctypes.data, nring.ctypes.data, C.byref(R), C.byref(nr), err, 256)
    assert rc == 1  # CAIR_EINVAL
    assert b"temperature" in err.value


def test_no_counted_rows(gpu_lib, oracle_lib):
    """Every row HNotCons or unfinished: no lines, no error."""
    L = _load(gpu_lib)
    rows = np.zeros(50, dtype=_lib.RESULT_DTYPE)
    rows["j_i"], rows["v_i"], rows["arr_i"] = 1.5, 0.5, 16.5
    rows["arr_f"] = 16.5
    rows["status"] = np.where(np.arange(50) % 2 == 0, 1, 0)
    rows["dH"] = 1.0
    items = np.zeros(2, dtype=_lib.ITEM_DTYPE)
    items["bmax"], items["ttra"] = 6.0, 1e4
    rows["item"] = np.arange(50) % 2
    P = _params(3, (0,) * 5, 1.0)
    keep = (rows["status"] == 0) & (np.abs(rows["dH"]) <= P.ham_abs_tol)
    assert not keep.any()
    assert len(_host_statistics(L, P, items, rows, None, keep, 3)) == 0


def numpy_passes(gpu_lib, P, nc):
    """The two device passes of the replicas' statistics restated in numpy (the rings from the library's
    host half): items_pass(nitems, rows) and counts_pass(items, rows, item_rows, item_ini, runs)."""
    L = _load(gpu_lib)
    names = ("j", "v", "arr") if nc == 3 else ("j", "v", "j2", "v2", "arr")

    def codes(rows):
        qi = np.stack([rows[n + "_i"] for n in names], 1)
        qf = np.stack([rows[n + "_f"] for n in names], 1)
        keep = (rows["status"] == 0) & (np.abs(rows["dH"]) <= P.ham_abs_tol)
        ic, fc = _codes(qi, qf, list(P.iskip)[:nc], list(P.pres_even_odd)[:nc], P.qn_max)
        return keep, ic, fc

    def items_pass(nitems, rows):
        keep, ic, _ = codes(rows)
        item_rows = np.bincount(rows["item"][keep], minlength=nitems).astype(np.uint64)
        item_ini = np.full(nitems, 0x7f7f7f7f7f7f7f7f, np.int64)
        np.minimum.at(item_ini, rows["item"][keep], ic[keep])
        return item_rows, item_ini

    def counts_pass(items, rows, item_rows, item_ini, runs):
        nitems = len(items)
        keep, ic, fc = codes(rows)
        itc = np.ascontiguousarray(items, dtype=_lib.ITEM_DTYPE)
        run_arr = None if runs is None else np.ascontiguousarray(runs, np.int32)
        ring_b, nring = np.zeros(nitems * MAXR), np.zeros(nitems, np.int32)
        R, nruns = C.c_int32(), C.c_int32()
        ir, ii = np.ascontiguousarray(item_rows, np.uint64), np.ascontiguousarray(item_ini, np.int64)
        assert L.cair_internal_stats_rings(C.byref(P), nitems, itc.ctypes.data,
                                           None if run_arr is None else run_arr.ctypes.data, ir.ctypes.data,
                                           ii.ctypes.data, ring_b.ctypes.data, nring.ctypes.data, C.byref(R),
                                           C.byref(nruns), None, 0) == 0
        run_of = np.arange(nitems) if runs is None else np.asarray(runs)
        rr = run_of[rows["item"]]
        ring = np.zeros(len(rows), np.int64)
        for k in np.flatnonzero(keep):
            e = ring_b[rr[k] * MAXR: rr[k] * MAXR + nring[rr[k]]]
            for q in range(len(e) - 1):
                if not (rows["b"][k] > e[q + 1] or rows["b"][k] <= e[q]):
                    ring[k] = q + 1
                    break
        trip = np.stack([rr[keep], ring[keep], fc[keep]], 1)
        u, cnt = np.unique(trip, axis=0, return_counts=True)
        out = np.zeros(len(u), dtype=_lib.STATS_COUNT_DTYPE)
        out["run"], out["ring"], out["code"], out["count"] = u[:, 0], u[:, 1], u[:, 2], cnt
        ring_rows = np.zeros((nruns.value, MAXR), np.uint64)
        np.add.at(ring_rows, (rr[keep], ring[keep]), 1)
        return out, ring_rows

    return items_pass, counts_pass


def _ring_rows_two_runs():
    rng = np.random.default_rng(8)
    bm = [2.0, 4.0, 6.0, 5.0, 5.0]
    counts = [3000, 4000, 6000, 3000, 3000]
    n = sum(counts)
    rows = np.zeros(n, dtype=_lib.RESULT_DTYPE)
    rows["item"] = np.repeat(np.arange(5), counts)
    rows["bmax"] = np.repeat(bm, counts)
    rows["b"] = rows["bmax"] * np.sqrt(rng.uniform(size=n))
    rows["j_i"], rows["v_i"], rows["arr_i"] = 20.5, 0.5, 16.5
    rows["j_f"] = rng.uniform(0.0, 45.0, n)
    rows["v_f"] = rng.uniform(-0.5, 6.0, n)
    rows["arr_f"] = rng.choice([16.5, 17.5, 32.5, 48.5], n)
    rows["dH"] = 1e-9
    items = np.zeros(5, dtype=_lib.ITEM_DTYPE)
    items["bmax"], items["ttra"] = bm, 10000.0
    return items, rows, [0, 0, 0, 1, 1]


def test_replicas_sum_to_the_statistics_of_all_rows(gpu_lib, oracle_lib):
    """Two replicas with disjoint rows -- the first holds every row of the 4-bohr item, the second none,
    so the rings only agree through the summed totals -- through the three steps of the replicas'
    statistics: the lines equal the oracle's and the one-replica lines of all rows."""
    from coarseair_gb300 import api
    L = _load(gpu_lib)
    items, rows, runs = _ring_rows_two_runs()
    P = _params(3, (1, 0, 0, 0, 0), _xmu(systems.n3_config().masses))
    items_pass, counts_pass = numpy_passes(gpu_lib, P, 3)
    part = [rows[(rows["item"] == 1) | (np.arange(len(rows)) % 2 == 0)],
            rows[(rows["item"] != 1) & (np.arange(len(rows)) % 2 == 1)]]
    totals = [items_pass(len(items), p) for p in part]
    ir = sum(t[0] for t in totals)
    ii = np.minimum(totals[0][1], totals[1][1])
    cs = [counts_pass(items, p, ir, ii, runs) for p in part]
    got = api.statistics_finish(P, items, ir, ii, np.concatenate([c[0] for c in cs]), cs[0][1] + cs[1][1], runs)
    keep = (rows["status"] == 0) & (np.abs(rows["dH"]) <= P.ham_abs_tol)
    one = _host_statistics(L, P, items, rows, runs, keep, 3)
    assert np.array_equal(got, one)
    _check(L, items, rows, (1, 0, 0, 0, 0), 3, P.xmu, runs=runs)
    with pytest.raises(api.CairError, match="outside the runs and rings"):
        bad = np.concatenate([c[0] for c in cs])
        bad["ring"][0] = 7
        api.statistics_finish(P, items, ir, ii, bad, cs[0][1] + cs[1][1], runs)


def _kernels_on_host(P, items, rows, runs):
    from test_pes_host import _harness
    L = _harness()
    it = np.ascontiguousarray(items, dtype=_lib.ITEM_DTYPE)
    rw = np.ascontiguousarray(rows, dtype=_lib.RESULT_DTYPE)
    rn = None if runs is None else np.ascontiguousarray(runs, np.int32)
    out = np.zeros(max(64, len(rw)), dtype=_lib.FINAL_STATE_DTYPE)
    n = C.c_int64()
    rc = L.stats_host_run(C.addressof(P), len(it), it.ctypes.data, None if rn is None else rn.ctypes.data, len(rw),
                          rw.ctypes.data, out.ctypes.data, len(out), C.byref(n))
    assert rc == 0, rc
    return out[:n.value]


def test_statistics_kernels_run_on_the_host(gpu_lib, oracle_lib):
    """k_stats_items, k_stats_count and k_stats_compact themselves (host build of cair_stats.cuh, a 1 x 1
    grid, atomics emulated) in cair_statistics_dev's order with the library's host half: the same lines
    as the restated passes, on pooled multi-ring runs (3 conditions) and on diatom + diatom rows with
    clusters (5 conditions)."""
    L = _load(gpu_lib)
    items, rows, runs = _ring_rows_two_runs()
    P = _params(3, (1, 0, 0, 0, 0), _xmu(systems.n3_config().masses))
    keep = (rows["status"] == 0) & (np.abs(rows["dH"]) <= P.ham_abs_tol)
    assert np.array_equal(_kernels_on_host(P, items, rows, runs), _host_statistics(L, P, items, rows, runs, keep, 3))
    rng = np.random.default_rng(4)
    n = 6000
    r5 = np.zeros(n, dtype=_lib.RESULT_DTYPE)
    r5["item"] = rng.integers(0, 2, n)
    r5["j_i"], r5["v_i"], r5["j2_i"], r5["v2_i"], r5["arr_i"] = 1.5, 0.5, 3.5, 0.5, 26.5
    arr = rng.choice([26.5, 42.5, 18.5, -65.5], n)
    for c in ("j_f", "v_f", "j2_f", "v2_f"):
        r5[c] = np.where(arr == -65.5, -0.5, rng.uniform(-1.0, 30.0 if c[0] == "j" else 6.0, n))
    r5["arr_f"] = arr
    r5["b"] = rng.uniform(0.0, 8.0, n)
    r5["bmax"] = 8.0
    r5["dH"] = 1e-9
    it5 = np.zeros(2, dtype=_lib.ITEM_DTYPE)
    it5["bmax"], it5["ttra"] = 8.0, 1e4
    P5 = _params(5, (1, 0, 1, 0, 0), _xmu(systems.o4_config().masses))
    keep5 = np.ones(n, bool)
    assert np.array_equal(_kernels_on_host(P5, it5, r5, None), _host_statistics(L, P5, it5, r5, None, keep5, 5))
