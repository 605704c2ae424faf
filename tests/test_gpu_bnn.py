"""O2 + O on the O3 BNN (BNN_PES_Class.F90) with its 50 posterior samples as 50 surfaces of one
handle, as the reference's stochastic-PES input runs them ("Nb of PESs Samples = 50", each sample
read from CalibratedParams/<name>.csv.<i>): every sample against the oracle at the same points, and
a queue run in per-sample blocks whose final states and pooled statistics match the oracle's."""
import os

import numpy as np
import pytest

from coarseair_gb300 import api, systems

pytestmark = pytest.mark.gpu
PROCS = min(16, os.cpu_count() or 1)


def _setup():
    from oracle import Oracle
    cfg = systems.o3bnn_config()
    o = Oracle(cfg)
    return cfg, o, api.Handle(cfg, tpq=o.tpq)


def test_fifty_samples_match_the_oracle(gpu_lib, oracle_lib):
    from test_gpu_o3mix import o_k
    from test_gpu_parity import _check_rounding_level, _geometries
    cfg, o, H = _setup()
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
    cfg, o, H = _setup()
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
