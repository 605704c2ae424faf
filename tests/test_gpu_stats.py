"""GPU statistics (cair_statistics: final-state counts on the device, cross sections and rates)
against the oracle's restatement of Statistics_Class.F90 on the same rows: identical final states
and counts, cross sections and their standard deviations to 1e-14 relative, rates = cross
sections x the Boltzmann mean velocity."""
import numpy as np
import pytest

from coarseair_gb300 import _lib, api, systems

pytestmark = pytest.mark.gpu


def _conds(rows, sel, natoms, which):
    names = ("j", "v", "arr") if natoms == 3 else ("j", "v", "j2", "v2", "arr")
    return np.stack([rows[nm + "_" + which][sel] for nm in names], 1)


def _compare(H, items, rows, pres, st, runs=None):
    """Device statistics against the oracle's on the counted rows of each run (in row order)."""
    import oracle
    cfg = H.cfg
    m = cfg.masses
    nc = 3 if cfg.natoms == 3 else 5
    mt, mp = m[0] + m[1], sum(m[2:])
    xmu = mt * mp / (mt + mp)
    got = st.compute(items, rows, runs=runs)
    assert np.all(got["fin"][:, nc:] == 0) and np.all(got["ini"][:, nc:] == 0)
    run_of = np.arange(len(items)) if runs is None else np.asarray(runs)
    row_run = run_of[rows["item"]]
    keep = (rows["status"] == 0) & (np.abs(rows["dH"]) <= cfg.ham_abs_tol)
    for run in np.unique(run_of):
        sel = keep & (row_run == run)
        g = got[got["run"] == run]
        if sel.sum() == 0:
            assert len(g) == 0
            continue
        ref, ini = oracle.statistics(rows["bmax"][sel], rows["b"][sel],
                                     _conds(rows, sel, cfg.natoms, "i"), _conds(rows, sel, cfg.natoms, "f"),
                                     iskip=(1,) * nc, pres=pres, cap=max(64, int(sel.sum())))
        assert len(g) == len(ref)
        gd = {tuple(int(x) for x in r["fin"][:nc]): r for r in g}
        vel = oracle.mean_velocity(items["ttra"][run_of == run][0], xmu)
        nrings = len(np.unique(rows["bmax"][sel]))
        for fs, n, cross, sd in ref:
            r = gd[fs]
            assert tuple(int(x) for x in r["ini"][:nc]) == ini
            assert r["count"] == n and r["nrows"] == sel.sum() and r["nrings"] == nrings
            assert r["cross"] == pytest.approx(cross, rel=1e-14)
            assert r["cross_sd"] == pytest.approx(sd, rel=1e-14, abs=1e-300)
            assert r["rate"] == pytest.approx(cross * vel, rel=1e-13)
            assert r["rate_sd"] == pytest.approx(sd * vel, rel=1e-13, abs=1e-300)
    return got


def test_statistics_of_a_queue_run(gpu_lib, oracle_lib):
    cfg = systems.n3_config(rmax=16.0)
    H = api.Handle(cfg)
    lv = systems.load_levels("N2")
    table = api.level_table(lv[[5, 300, 2000]])
    items = api.work_items([(0, 0, 400, api.process_seed(7, 1), 10000.0, 7.0, 15.0),
                            (1, 0, 300, api.process_seed(7, 2), 20000.0, 7.0, 15.0),
                            (2, 0, 300, api.process_seed(7, 3), 5000.0, 7.0, 15.0)])
    rows = api.RunTrajectories(H).run(table, items)
    got = _compare(H, items, rows, (1, 0, 0), api.Statistics(H, pres_even_odd=(1, 0, 0)))
    # every counted row is in exactly one final state
    for i in range(len(items)):
        g = got[got["run"] == i]
        assert g["count"].sum() == g["nrows"][0]
    H.close()


def test_statistics_on_synthetic_rows(gpu_lib, oracle_lib):
    """100k rows over 5 items with scattered continuous quantum numbers (many final states,
    arrangement changes, dissociated rows, a few HNotCons and capped rows)."""
    cfg = systems.o3_config()
    H = api.Handle(cfg)
    rng = np.random.default_rng(21)
    n, nitems = 100000, 5
    rows = np.zeros(n, dtype=_lib.RESULT_DTYPE)
    rows["item"] = rng.integers(0, nitems, n)
    rows["j_i"] = 10.5 + 2.0 * rows["item"]
    rows["v_i"] = 0.5 + rows["item"] % 2
    rows["arr_i"] = 16.5
    rows["j_f"] = rng.uniform(0.0, 60.0, n)
    rows["v_f"] = rng.uniform(-1.5, 12.0, n)
    rows["arr_f"] = rng.choice([16.5, 17.5, 18.5, 32.5, 48.5], n)
    rows["b"] = rng.uniform(0.0, 6.0, n)
    rows["status"] = np.where(rng.uniform(size=n) < 0.01, 1, 0)
    rows["dH"] = np.where(rng.uniform(size=n) < 0.01, 1.0, 1e-9)
    items = np.zeros(nitems, dtype=_lib.ITEM_DTYPE)
    items["bmax"] = 6.0
    items["ttra"] = [5000.0, 10000.0, 15000.0, 20000.0, 8000.0]
    rows["bmax"] = items["bmax"][rows["item"]]      # a row carries its item's ring bound, as the queue writes it
    _compare(H, items, rows, (1, 0, 0), api.Statistics(H, pres_even_odd=(1, 0, 0)))
    _compare(H, items, rows, (0, 0, 0), api.Statistics(H))
    # a table that cannot hold every final state is an error, not a truncation
    with pytest.raises(api.CairError, match="cap too small"):
        api.Statistics(H).compute(items, rows, cap=8)
    H.close()


def test_statistics_with_zero_bmax_are_probabilities(gpu_lib, oracle_lib):
    """Rows whose bMax is 0 make one ring of area 0, which SetRings turns into area 1
    (Statistics_Class.F90:578-581): the cross sections are the final states' probabilities, on the
    device as in the oracle."""
    cfg = systems.o3_config()
    H = api.Handle(cfg)
    rng = np.random.default_rng(22)
    n, nitems = 20000, 2
    rows = np.zeros(n, dtype=_lib.RESULT_DTYPE)
    rows["item"] = rng.integers(0, nitems, n)
    rows["j_i"] = 10.5
    rows["v_i"] = 0.5 + rows["item"]
    rows["arr_i"] = 16.5
    rows["j_f"] = rng.uniform(0.0, 30.0, n)
    rows["v_f"] = rng.uniform(-1.0, 6.0, n)
    rows["arr_f"] = rng.choice([16.5, 32.5, 48.5], n)
    rows["bmax"] = 0.0
    rows["b"] = 0.0
    items = np.zeros(nitems, dtype=_lib.ITEM_DTYPE)
    items["bmax"] = 0.0
    items["ttra"] = [10000.0, 20000.0]
    got = _compare(H, items, rows, (0, 0, 0), api.Statistics(H))
    assert np.all(got["nrings"] == 1)
    for i in range(nitems):
        g = got[got["run"] == i]
        assert g["cross"].sum() == pytest.approx(1.0, rel=1e-12)
        assert np.allclose(g["cross"], g["count"] / g["nrows"][0], rtol=1e-14, atol=0.0)
    H.close()


def test_statistics_refuse_rows_ringed_apart_from_their_item(gpu_lib):
    """The device rings each run by its items' bmax.  A counted row whose bmax differs from its
    item's by 1e-3 or more would be ringed differently by SetRings, which reads the rows' bMax, so
    the statistics refuse it; a difference below SetRings' 1e-3 is one ring and is accepted."""
    cfg = systems.o3_config()
    H = api.Handle(cfg)
    n = 1000
    rows = np.zeros(n, dtype=_lib.RESULT_DTYPE)
    rows["j_i"], rows["v_i"], rows["arr_i"] = 10.5, 0.5, 16.5
    rows["j_f"], rows["v_f"], rows["arr_f"] = 12.5, 0.5, 16.5
    rows["b"] = np.linspace(0.0, 6.0, n)
    items = np.zeros(1, dtype=_lib.ITEM_DTYPE)
    items["bmax"], items["ttra"] = 6.0, 10000.0
    rows["bmax"] = 6.0 + 5e-4
    got = api.Statistics(H).compute(items, rows)
    assert got["count"].sum() == n
    rows["bmax"][17] = 6.0 + 2e-3
    with pytest.raises(api.CairError, match="bmax"):
        api.Statistics(H).compute(items, rows)
    H.close()


def test_statistics_on_synthetic_diatom_diatom_rows(gpu_lib, oracle_lib):
    """Five conditions (J1, v1, J2, v2, arrangement) as for O2 + O2: 100k rows over 4 items with
    exchange arrangements, one-molecule dissociation and four-atom clusters (arrangement -65.5,
    a negative final-state code), against the oracle with and without even/oddness preserved."""
    cfg = systems.o4_config()
    H = api.Handle(cfg)
    rng = np.random.default_rng(33)
    n, nitems = 100000, 4
    rows = np.zeros(n, dtype=_lib.RESULT_DTYPE)
    rows["item"] = rng.integers(0, nitems, n)
    rows["j_i"] = 1.5 + 2.0 * rows["item"]
    rows["v_i"] = 0.5
    rows["j2_i"] = 3.5 + 4.0 * (rows["item"] % 2)
    rows["v2_i"] = 0.5 + (rows["item"] >= 2)
    rows["arr_i"] = 16.0 + 2.0 + 4.0 * 2.0 + 0.5       # iPair 1, both molecules bound (itype 2)
    rows["j_f"] = rng.uniform(-1.0, 40.0, n)
    rows["v_f"] = rng.uniform(-1.0, 8.0, n)
    rows["j2_f"] = rng.uniform(-1.0, 40.0, n)
    rows["v2_f"] = rng.uniform(-1.0, 8.0, n)
    arr = rng.choice([26.5, 42.5, 58.5, 22.5, 18.5, 17.5, -65.5], n)
    rows["arr_f"] = arr
    for c in ("j_f", "v_f", "j2_f", "v2_f"):
        rows[c] = np.where(arr == -65.5, -0.5, rows[c])
    rows["b"] = rng.uniform(0.0, 8.0, n)
    rows["status"] = np.where(rng.uniform(size=n) < 0.01, 1, 0)
    rows["dH"] = np.where(rng.uniform(size=n) < 0.01, 1.0, 1e-9)
    items = np.zeros(nitems, dtype=_lib.ITEM_DTYPE)
    items["bmax"] = 8.0
    items["ttra"] = [5000.0, 10000.0, 15000.0, 20000.0]
    rows["bmax"] = items["bmax"][rows["item"]]
    got = _compare(H, items, rows, (1, 0, 1, 0, 0), api.Statistics(H, pres_even_odd=(1, 0, 1, 0, 0)))
    assert np.any(got["fin"][:, 4] < 0)
    _compare(H, items, rows, (0, 0, 0, 0, 0), api.Statistics(H))
    H.close()


def test_statistics_of_an_o2_o2_queue_run(gpu_lib, oracle_lib):
    """Rows of a real O2 + O2 queue run (two items, two of the O4 surfaces) through the device
    statistics and through the oracle's: identical final states, counts and cross sections."""
    cfg = systems.o4_config()
    H = api.Handle(cfg)
    lv = systems.load_levels("O2")
    il = [int(np.flatnonzero((lv["vqn"] == 0) & (lv["jqn"] == j))[0]) for j in (1, 3)]
    table = api.level_table(lv[il])
    items = api.work_items([(0, 0, 48, api.process_seed(5, 1), 10000.0, 8.0, 18.0, 1),
                            (1, 1, 48, api.process_seed(5, 2), 20000.0, 8.0, 18.0, 0)])
    rows = api.RunTrajectories(H).run(table, items)
    got = _compare(H, items, rows, (0, 0, 0, 0, 0), api.Statistics(H))
    for i in range(len(items)):
        g = got[got["run"] == i]
        assert g["count"].sum() == g["nrows"][0]
    H.close()


def test_rate_coefficients_within_two_sigma_of_the_oracle_path(gpu_lib, oracle_lib):
    """The same 600 initial conditions (one N2 + N run) propagated and analysed by the GPU path and
    by the oracle: every final state's rate coefficient agrees within twice the combined Monte-Carlo
    standard deviation (the acceptance criterion for rates), and the totals match."""
    import os
    import oracle
    from oracle import Oracle
    cfg = systems.n3_config(rmax=16.0)
    H = api.Handle(cfg)
    o = Oracle(cfg)
    lv = systems.load_levels("N2")
    rows_lv = lv[[300]]
    table = api.level_table(rows_lv)
    nt, seed, T = 600, api.process_seed(9, 1), 10000.0
    items = api.work_items([(0, 0, nt, seed, T, 7.0, 15.0)])
    rows = api.RunTrajectories(H).run(table, items)
    # oracle path on the same stream
    lvo = np.zeros(1, dtype=[(c, "f8") for c in ("vqn", "jqn", "eint", "egam", "rmin", "rmax", "vmin", "vmax", "tau",
                                                   "ri", "ro", "rlim")])
    for c in lvo.dtype.names:
        lvo[c] = rows_lv[c] if c in rows_lv.dtype.names else 0.0
    ic = o.sample_ics(nt, lvo, seed=seed, ttra=T, bmax=7.0, dinit=15.0)
    res = o.integrate(ic["paq"], ic["erra"], procs=min(16, os.cpu_count() or 1))
    fi = o.analyze(ic["paq0"])
    ff = o.analyze(o.apply_transformation(res["paq"]))
    keep = (res["status"] == 0) & (np.abs(res["H"] - ic["H0"]) <= cfg.ham_abs_tol)
    col = lambda fs, k: np.array([f[k] for f in fs])
    qi = np.stack([col(fi, "angmom"), col(fi, "viba"), 16 * col(fi, "ipair") + col(fi, "itype") + 0.5], 1)
    qf = np.stack([col(ff, "angmom"), col(ff, "viba"), 16 * col(ff, "ipair") + col(ff, "itype") + 0.5], 1)
    ref, _ = oracle.statistics(np.full(keep.sum(), 7.0), ic["b"][keep], qi[keep], qf[keep], pres=(1, 0, 0),
                               cap=nt)
    m = cfg.masses
    vel = oracle.mean_velocity(T, (m[0] + m[1]) * m[2] / sum(m))
    got = api.Statistics(H, pres_even_odd=(1, 0, 0)).compute(items, rows)
    g = {tuple(int(x) for x in r["fin"][:3]): (r["rate"], r["rate_sd"]) for r in got}
    r = {fs: (cross * vel, sd * vel) for fs, n, cross, sd in ref}
    worst = 0.0
    for fs in set(g) | set(r):
        kg, sg = g.get(fs, (0.0, 0.0))
        ko, so = r.get(fs, (0.0, 0.0))
        sig = np.hypot(sg, so)
        if sig == 0.0:
            assert kg == ko
            continue
        worst = max(worst, abs(kg - ko) / sig)
    tot_g, tot_o = sum(v[0] for v in g.values()), sum(v[0] for v in r.values())
    print("rates: %d final states (GPU) / %d (oracle), worst |dk|/sigma %.3f, total %.6e vs %.6e" %
          (len(g), len(r), worst, tot_g, tot_o))
    assert worst <= 2.0
    assert tot_g == pytest.approx(tot_o, rel=1e-12)
    H.close()


_CONFIG1_REF = {}


def _config1_oracle_rates(o, cfg, row, nt, seed, T):
    """The oracle's rates of config 1 (computed once for both integrator modes)."""
    import os
    import oracle
    if "ref" not in _CONFIG1_REF:
        lvo = np.zeros(1, dtype=[(c, "f8") for c in ("vqn", "jqn", "eint", "egam", "rmin", "rmax", "vmin", "vmax",
                                                       "tau", "ri", "ro", "rlim")])
        for c in lvo.dtype.names:
            lvo[c] = row[c] if c in row.dtype.names else 0.0
        ic = o.sample_ics(nt, lvo, seed=seed, ttra=T, bmax=6.0, dinit=15.0)
        res = o.integrate(ic["paq"], ic["erra"], procs=min(16, os.cpu_count() or 1))
        fi, ff = o.analyze(ic["paq0"]), o.analyze(o.apply_transformation(res["paq"]))
        keep = (res["status"] == 0) & (np.abs(res["H"] - ic["H0"]) <= cfg.ham_abs_tol)
        col = lambda fs, k: np.array([f[k] for f in fs])
        qi = np.stack([col(fi, "angmom"), col(fi, "viba"), 16 * col(fi, "ipair") + col(fi, "itype") + 0.5], 1)
        qf = np.stack([col(ff, "angmom"), col(ff, "viba"), 16 * col(ff, "ipair") + col(ff, "itype") + 0.5], 1)
        _CONFIG1_REF["ref"], _ = oracle.statistics(np.full(keep.sum(), 6.0), ic["b"][keep], qi[keep], qf[keep], cap=nt)
    return _CONFIG1_REF["ref"]


@pytest.mark.parametrize("mode", ["thread", "warp"])
def test_o2_o_ground_state_rates_within_two_sigma(gpu_lib, oracle_lib, mode):
    """O2(v=0, J=1) + O on UMN_11A1 in full -- 10,000 trajectories, seed 1,
    10,000 K, b = 6 sqrt(U) bohr, Dinit 15 bohr, rmax 16 bohr -- through the GPU queue (a lane per
    trajectory, and a warp per trajectory, the mode a job of this size runs in) and through the oracle
    from the same stream: every final state's rate agrees within twice the combined Monte-Carlo
    standard deviation."""
    import oracle
    from oracle import Oracle
    cfg = systems.o3_config(dinit=15.0, bmax=6.0, rmax=16.0)
    H = api.Handle(cfg)
    H.integrator_mode = mode
    o = Oracle(cfg)
    lv = systems.load_levels("O2")
    row = lv[(lv["vqn"] == 0) & (lv["jqn"] == 1)]
    nt, seed, T = 10000, api.process_seed(1, 1), 10000.0
    items = api.work_items([(0, 0, nt, seed, T, 6.0, 15.0)])
    rows = api.RunTrajectories(H).run(api.level_table(row), items)
    ref = _config1_oracle_rates(o, cfg, row, nt, seed, T)
    m = cfg.masses
    vel = oracle.mean_velocity(T, (m[0] + m[1]) * m[2] / sum(m))
    got = api.Statistics(H).compute(items, rows)
    g = {tuple(int(x) for x in r["fin"][:3]): (r["rate"], r["rate_sd"]) for r in got}
    r = {fs: (cross * vel, sd * vel) for fs, n, cross, sd in ref}
    dev = []
    for fs in set(g) | set(r):
        kg, sg = g.get(fs, (0.0, 0.0))
        ko, so = r.get(fs, (0.0, 0.0))
        sig = np.hypot(sg, so)
        dev.append(0.0 if sig == 0.0 else abs(kg - ko) / sig)
    print("O2(0,1) + O rates (%s integrator): %d final states (GPU) / %d (oracle), worst |dk|/sigma %.3f" %
          (mode, len(g), len(r), max(dev)))
    assert max(dev) <= 2.0
    H.close()
