"""GPU parity of N2 + N2 on the N4 UMN surface (the N4 PIP on all six pairs) against the oracle:
surface energies and gradients, right-hand side and Hamiltonian (1e-12 relative or the rounding-level
bound of a chain of 2 x 101 + 276 + 10 operations), 1000 fixed attempts on non-chaotic trajectories,
and the queue path's final states."""
import os

import numpy as np
import pytest

from coarseair_gb300 import api, systems

pytestmark = pytest.mark.gpu
PROCS = min(16, os.cpu_count() or 1)
ROUND_N4 = 2 * 488 * 1.1102230246251565e-16


def _setup():
    from oracle import Oracle
    cfg = systems.n4_config()
    o = Oracle(cfg)
    return cfg, o, api.Handle(cfg, tpq=o.tpq)


def _check(err, ref, cs, floor, name):
    b = np.maximum(1e-12 * np.maximum(ref, floor), ROUND_N4 * cs)
    print("%s: worst/bound %.2e, %.4f within 1e-12" % (name, (err / b).max(), np.mean(err <= 1e-12 * np.maximum(ref, floor))))
    assert np.all(err <= b)


def test_n4_surface_rhs_and_attempts(gpu_lib, oracle_lib):
    from test_gpu_o4 import _collision_points, _geometries
    cfg, o, H = _setup()
    R, Qall = _geometries(o, 384, 41)
    V_o, g_o, m_o = o.compute(R, Qall)
    V_g, g_g, m_g = api.PES(H).Compute(R, Qall)
    cs = o.condition_scale(R)
    _check(np.abs(V_g - V_o), np.abs(V_o), cs[:, 0], 0.1, "N4 V")
    _check(np.abs(api.PES(H).Potential(R, Qall) - V_o), np.abs(V_o), cs[:, 0], 0.1, "N4 V (energy only)")
    _check(np.abs(g_g - g_o), np.abs(g_o).max(axis=1, keepdims=True), cs[:, 1:], 1e-2, "N4 dV/dR")
    y, erra = _collision_points(o, cfg, 48, 42, sep=7.0, ekin=0.05)
    yp_o, yp_g = o.rhs(y), api.Collision(H).EvaluateRHS(y)
    cy = o.condition_scale(o.rp(y[:, 9:])[0])
    _check(np.abs(yp_g - yp_o), np.abs(yp_o).max(axis=1, keepdims=True), cy[:, 1:].max(axis=1, keepdims=True), 1e-12,
           "N4 RHS")
    h_o, _ = o.hamiltonian(y)
    h_g, _ = api.Collision(H).Hamiltonian(y)
    _check(np.abs(h_g - h_o), np.abs(h_o), cy[:, 0], 0.1, "N4 H")
    n = 24
    t0, dt0 = np.zeros(n), np.full(n, cfg.dt0)
    a, _, _ = o.bs_attempts(y[:n], t0, dt0, erra[:n], 1000)
    b, _, _ = o.bs_attempts(y[:n] * (1 + 1e-14), t0, dt0, erra[:n], 1000)
    ok = np.abs(a - b).max(axis=1) / np.abs(a).max(axis=1) < 1e-11
    tr = api.Trajectories.start(y[:n], erra[:n], cfg.dt0)
    api.ODE(H).Integrate(tr, 1000)
    rel = np.abs(tr.paq - a).max(axis=1) / np.abs(a).max(axis=1)
    print("N4 1000 attempts: %d non-chaotic, max rel %.2e" % (ok.sum(), rel[ok].max() if ok.any() else 0.0))
    assert ok.sum() >= 4 and np.all(rel[ok] < 1e-9)
    H.close()


def test_n4_queue_matches_oracle(gpu_lib, oracle_lib):
    from test_gpu_o4 import _fs_tuple
    cfg, o, H = _setup()
    lv = systems.load_levels("N2")
    rows = lv[[0, 30, 200]]
    table = api.level_table(rows)
    entries = [(0, 0, 12, api.process_seed(5, 1), 20000.0, 8.0, 23.0, 1),
               (1, 0, 12, api.process_seed(5, 2), 20000.0, 8.0, 23.0, 2)]
    items = api.work_items(entries)
    res = api.RunTrajectories(H).run(table, items)
    assert np.all(res["status"] == 0)
    assert np.max(np.abs(res["dH"])) < cfg.ham_abs_tol
    qn = lambda x: (np.sign(x) * np.floor(np.abs(x) + 0.5)).astype(int)
    same, stable = [], []
    for i, (il, ipes, nt, seed, T, bmax, dinit, il2) in enumerate(entries):
        ref = o.sample_ics4(nt, rows[il], rows[il2], ttra=T, bmax=bmax, dinit=dinit, seed=seed)
        a = o.integrate(ref["paq"], ref["erra"], procs=PROCS)
        b = o.integrate(ref["paq"] * (1 + 1e-14), ref["erra"], procs=PROCS)
        fa = [_fs_tuple(f) for f in o.analyze(o.apply_transformation(a["paq"]))]
        fb = [_fs_tuple(f) for f in o.analyze(o.apply_transformation(b["paq"]))]
        r = res[int(items["first"][i]):int(items["first"][i]) + nt]
        fg = [tuple(int(x) for x in t) for t in zip(qn(r["j_f"] - 0.5), qn(r["v_f"] - 0.5), qn(r["j2_f"] - 0.5),
                                                     qn(r["v2_f"] - 0.5), qn(r["arr_f"] - 0.5))]
        same += [x == y for x, y in zip(fg, fa)]
        stable += [x == y for x, y in zip(fa, fb)]
    same, stable = np.array(same), np.array(stable)
    print("N4 queue: GPU vs oracle %.4f overall, %.4f on oracle-stable (%d of %d stable)" %
          (same.mean(), same[stable].mean(), stable.sum(), len(stable)))
    assert stable.sum() >= len(stable) // 2 and same[stable].mean() >= 0.995
    H.close()
