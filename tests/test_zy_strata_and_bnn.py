"""GPU tests of the O3 BNN surface and of stratified impact parameters.

* The O3 BNN (BNN_PES_Class.F90) with its 50 posterior samples as 50 surfaces of one handle, as the
  reference's stochastic-PES input runs them ("Nb of PESs Samples = 50", each sample read from
  CalibratedParams/<name>.csv.<i>): every sample against the oracle at the same points; the parity
  checks of test_gpu_parity on one sample; a queue run in per-sample blocks whose final states and
  pooled statistics match the oracle's.
* Impact-parameter rings (ImpactParameter_Class.F90, Collision_Class.F90:1276-1296): one stream
  split into rings of every strata type through the queue, and statistics runs pooling rings.

Collected after every other test file, so that a run that stops at the first failure has run the
rest: these are the newest GPU paths.
"""
import os

import numpy as np
import pytest

from coarseair_gb300 import _lib, api, systems
from test_gpu_parity import test_final_state_analysis_parity_on_identical_points as _final_states
from test_gpu_parity import test_phase_space_after_1000_attempts as _phase_space
from test_gpu_parity import test_rhs_and_hamiltonian_parity as _rhs
from test_gpu_parity import test_surface_energy_and_gradient_parity as _surface
from test_gpu_queue import _oracle_levels
from test_gpu_queue import _setup as _queue_setup
from test_gpu_stats import _compare

pytestmark = pytest.mark.gpu
PROCS = min(16, os.cpu_count() or 1)


def test_bnn_sample_surface_parity(gpu_lib, oracle_lib):
    _surface(gpu_lib, oracle_lib, "O3BNN")


def test_bnn_sample_rhs_and_hamiltonian_parity(gpu_lib, oracle_lib):
    _rhs(gpu_lib, oracle_lib, "O3BNN")


def test_bnn_sample_phase_space_after_1000_attempts(gpu_lib, oracle_lib):
    _phase_space(gpu_lib, oracle_lib, "O3BNN")


def test_bnn_sample_final_state_analysis(gpu_lib, oracle_lib):
    _final_states(gpu_lib, oracle_lib, "O3BNN")


def _bnn_setup():
    from oracle import Oracle
    cfg = systems.o3bnn_config()
    o = Oracle(cfg)
    return cfg, o, api.Handle(cfg, tpq=o.tpq)


def test_fifty_samples_match_the_oracle(gpu_lib, oracle_lib):
    from test_gpu_o3mix import o_k
    from test_gpu_parity import _check_rounding_level, _geometries
    cfg, o, H = _bnn_setup()
    assert len(cfg.surfaces) == 50
    R, Qall = _geometries(o, 50 * 24, 41)
    ip = np.arange(len(R), dtype=np.int32) % 50
    for k in range(50):
        sel = ip == k
        V_o, g_o, _ = o.compute(R[sel], Qall[sel], ipes=ip[sel])
        V_g, g_g, _ = api.PES(H).Compute(R[sel], Qall[sel], ipes=ip[sel])
        _check_rounding_level(o_k(o, k), R[sel], V_o, g_o, [(V_g, g_g)], "BNN sample %d" % (k + 1))
        Ve = api.PES(H).Potential(R[sel], Qall[sel], ipes=ip[sel])
        Vp_o = o.potential(R[sel], ipes=ip[sel])
        _check_rounding_level(o_k(o, k), R[sel], Vp_o, g_o, [(Ve, None)], "BNN sample %d Potential" % (k + 1))
    H.close()


def test_sample_blocks_through_the_queue_and_pooled_statistics(gpu_lib, oracle_lib):
    """100 trajectories in 50 per-sample blocks of one stream each, capped at 20,000 BS attempts on
    both sides (the cap keeps a trapped O3 complex from holding the GPU): final states against the
    oracle where both finished, then the finished rows of all 50 samples pooled into one run."""
    import oracle
    cfg, o, H = _bnn_setup()
    lv = systems.load_levels("O2")
    row = lv[(lv["vqn"] == 0) & (lv["jqn"] == 1)]
    table = api.level_table(row)
    counts = api.degeneracy_blocks(100, cfg.degeneracy)
    assert counts == [2] * 50
    seed, cap = api.process_seed(3, 1), 20000
    items = api.work_items([(0, k, n, seed, 20000.0, 6.0, 15.0) for k, n in enumerate(counts)])
    res = api.RunTrajectories(H).run(table, items, max_attempts=cap)
    assert list(np.bincount(res["ipes"], minlength=50)) == counts
    lvo = np.zeros(1, dtype=[(c, "f8") for c in ("vqn", "jqn", "eint", "egam", "rmin", "rmax", "vmin", "vmax", "tau",
                                                   "ri", "ro", "rlim")])
    for c in lvo.dtype.names:
        lvo[c] = row[c] if c in row.dtype.names else 0.0
    ic = o.sample_ics(2, lvo, seed=seed, ttra=20000.0, bmax=6.0, dinit=15.0)
    paq = np.tile(ic["paq"], (50, 1))
    erra = np.tile(ic["erra"], (50, 1))
    ipv = np.repeat(np.arange(50, dtype=np.int32), 2)
    a = o.integrate(paq, erra, ipes=ipv, max_attempts=cap, procs=PROCS)
    b = o.integrate(paq * (1 + 1e-14), erra, ipes=ipv, max_attempts=cap, procs=PROCS)

    def qn(paqs):
        fs = o.analyze(o.apply_transformation(paqs))
        return api.histogram_assign(np.array([f["angmom"] for f in fs]), np.array([f["viba"] for f in fs]),
                                    np.array([16 * f["ipair"] + f["itype"] + 0.5 for f in fs]))

    fa, fb = qn(a["paq"]), qn(b["paq"])
    fg = api.histogram_assign(res["j_f"], res["v_f"], res["arr_f"])
    done = (res["status"] == 0) & (a["status"] == 0) & (b["status"] == 0)
    same = (fa[0] == fg[0]) & (fa[1] == fg[1]) & (fa[2] == fg[2])
    stable = done & (fa[0] == fb[0]) & (fa[1] == fb[1]) & (fa[2] == fb[2])
    print("O3 BNN 50 samples: %d of 100 finished; GPU vs oracle %.4f on oracle-stable (%d stable)" %
          (int(done.sum()), same[stable].mean() if stable.any() else float("nan"), int(stable.sum())))
    assert stable.sum() >= 20
    assert same[stable].mean() >= 0.995
    # the finished rows of the 50 samples pooled into one run (the reference's statistics read every
    # PES's rows); the Hamiltonian comes from Potential, so HNotCons is decided by a wide tolerance here
    st = api.Statistics(H, ham_abs_tol=1.0e6)
    got = st.compute(items, res, runs=[0] * 50)
    ok = res["status"] == 0
    qi = np.stack([res["j_i"], res["v_i"], res["arr_i"]], 1)[ok]
    qf = np.stack([res["j_f"], res["v_f"], res["arr_f"]], 1)[ok]
    ref, ini = oracle.statistics(res["bmax"][ok], res["b"][ok], qi, qf, cap=200)
    assert len(got) == len(ref)
    gd = {tuple(int(x) for x in r["fin"][:3]): r for r in got}
    for fs, n, cross, sd in ref:
        assert gd[fs]["count"] == n and gd[fs]["nrows"] == int(ok.sum())
        assert gd[fs]["cross"] == pytest.approx(cross, rel=1e-14)
    H.close()


@pytest.mark.parametrize("strata", ["Circles", "Rings", "Segments"])
def test_stratified_rings_continue_one_stream(gpu_lib, oracle_lib, strata):
    """One stream split into impact-parameter rings (ImpactParameter_Class.F90:55-221), one work item
    per ring from api.ring_entries: every trajectory's initial condition equals the oracle's at the
    same stream position, the third ring's positive input value is a fixed b that draws no random
    number, and the rows are numbered along the stream with each ring's |b| as bmax."""
    cfg, o, H, lv = _queue_setup("N3")
    rows = lv[[17]]
    bring, ntring, n, seed = [-2.0, -4.5, 3.0, -7.0], [1, 2, 1, 3], 71, api.process_seed(4, 1)
    entries = api.ring_entries(0, 0, n, seed, 10000.0, 15.0, bring, ntring, strata)
    assert [e[2] for e in entries] == [11, 20, 10, 30] and [e[10] for e in entries] == [0, 11, 31, 41]
    items = api.work_items(entries)
    table = api.level_table(rows)
    ic = api.InitialConditions(H).sample(table, items)
    ref = o.sample_ics(n, _oracle_levels(rows), seed=seed, ttra=10000.0, dinit=15.0,
                       rings=(bring, ntring, api.STRATA[strata]))
    for key in ("paq", "paq0", "erra"):
        sc = np.abs(ref[key]).max(axis=1, keepdims=True)
        assert np.all(np.abs(ic[key] - ref[key]) <= 1e-10 * sc), key
    assert np.allclose(ic["b"], ref["b"], rtol=1e-14, atol=0)
    assert np.all(ic["b"][31:41] == 3.0)
    res = api.RunTrajectories(H).run(table, items, max_attempts=2000)  # the rows' numbering and b only
    assert list(res["idx"]) == list(range(1, n + 1))
    assert np.array_equal(res["bmax"], np.repeat([2.0, 4.5, 3.0, 7.0], [11, 20, 10, 30]))
    # the row's b is the analysed impact parameter of the initial point (TrajIni%b), a magnitude; Segments
    # strata after a sampled ring draw negative b
    assert np.allclose(res["b"], np.abs(ref["b"]), rtol=1e-13, atol=0)
    H.close()


def test_statistics_pool_rings_and_skip_empty_ones(gpu_lib, oracle_lib):
    """Impact-parameter rings (SetRings and the ring assignment of AddFinState): 60k synthetic rows in
    two runs.  Run 0 has items with bmax 2, 4 and 6 bohr (Circles: each samples its whole disc, so
    rows fall in inner rings too), and the 4-bohr item's rows are all HNotCons, so its ring is not a
    ring of the statistics; run 1 pools two items of one bmax (two surfaces).  Cross sections sum
    ring area x probability over the rings, against the oracle on the same rows."""
    cfg = systems.n3_config()
    H = api.Handle(cfg)
    rng = np.random.default_rng(5)
    bm = [2.0, 4.0, 6.0, 5.0, 5.0]
    counts = [8000, 12000, 20000, 10000, 10000]
    items = api.work_items([(0, 0, c, 1, 10000.0, b, 15.0) for c, b in zip(counts, bm)])
    n = sum(counts)
    rows = np.zeros(n, dtype=_lib.RESULT_DTYPE)
    rows["item"] = np.repeat(np.arange(5), counts)
    rows["bmax"] = np.repeat(bm, counts)
    rows["b"] = rows["bmax"] * np.sqrt(rng.uniform(size=n))
    rows["j_i"], rows["v_i"], rows["arr_i"] = 20.5, 0.5, 16.5
    rows["j_f"] = rng.uniform(0.0, 45.0, n)
    rows["v_f"] = rng.uniform(-0.5, 6.0, n)
    rows["arr_f"] = rng.choice([16.5, 17.5, 32.5, 48.5], n)
    rows["status"] = 0
    rows["dH"] = np.where(rows["item"] == 1, 1.0, 1e-9)
    runs = [0, 0, 0, 1, 1]
    got = _compare(H, items, rows, (1, 0, 0), api.Statistics(H, pres_even_odd=(1, 0, 0)), runs=runs)
    assert set(got[got["run"] == 0]["nrings"]) == {2} and set(got[got["run"] == 1]["nrings"]) == {1}
    # items of one run must share the temperature
    bad = items.copy()
    bad["ttra"][2] = 20000.0
    with pytest.raises(api.CairError, match="temperature"):
        api.Statistics(H).compute(bad, rows, runs=runs)
    H.close()
