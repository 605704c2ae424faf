"""GPU parity of N2 + N2 on the N4 UMN PIPNN surface (N4_UMN_PIPNN_PES_Class.F90) against the oracle.

Compute through cair_pes_eval: V and dVdR (the reference's central differences) within 2048 units of
the oracle's rounding scale for this surface (the magnitudes its output cancels, ~200 Eh; the host
build of the same device code is within 60 units without fused multiply-adds and 150 with them), dVdQ
zero.  Hamilton's equations feel no force (dp/dt = -0, the momenta never change); the Hamiltonian and
40 fixed attempts as the oracle's; the queue path's initial states equal to the oracle's and its final
states on >= 99.5 % of the trajectories whose oracle outcome a 1e-14 perturbation leaves unchanged
(the motion is force-free, so that is nearly all).  On the GB300 the surface came within 68 units (V)
and 106 (dV/dR) of the scale."""
import numpy as np
import pytest

from coarseair_gb300 import api, systems

pytestmark = pytest.mark.gpu
U = 1.1102230246251565e-16
UNITS = 2048


def _setup(**kw):
    from oracle import Oracle
    cfg = systems.n4pipnn_config(**kw)
    o = Oracle(cfg)
    return cfg, o, api.Handle(cfg, tpq=o.tpq)


def test_pipnn_surface_rhs_hamiltonian_and_attempts(gpu_lib, oracle_lib):
    from test_gpu_o4 import _collision_points, _geometries
    cfg, o, H = _setup()
    R, Qall = _geometries(o, 256, 43)
    V_o, g_o, m_o = o.compute(R, Qall)
    V_g, g_g, m_g = api.PES(H).Compute(R, Qall)
    cs = o.condition_scale(R)
    print("PIPNN: V %.1f, dV/dR %.1f units of the scale" %
          (np.max(np.abs(V_g - V_o) / (U * cs[:, 0])), np.max(np.abs(g_g - g_o) / (U * cs[:, 1:]))))
    assert np.all(np.abs(V_g - V_o) <= UNITS * U * cs[:, 0])
    assert np.all(np.abs(g_g - g_o) <= UNITS * U * cs[:, 1:])
    assert np.all(m_g == 0.0)
    assert np.all(np.abs(api.PES(H).Potential(R, Qall) - V_o) <= UNITS * U * cs[:, 0])
    y, erra = _collision_points(o, cfg, 32, 44, sep=7.0, ekin=0.05)
    yp_o, yp_g = o.rhs(y), api.Collision(H).EvaluateRHS(y)
    assert np.all(yp_g[:, :9] == 0.0) and np.all(yp_o[:, :9] == 0.0)
    assert np.allclose(yp_g[:, 9:], yp_o[:, 9:], rtol=1e-13, atol=1e-13 * np.abs(yp_o).max())
    h_o, _ = o.hamiltonian(y)
    h_g, _ = api.Collision(H).Hamiltonian(y)
    cy = o.condition_scale(o.rp(y[:, 9:])[0])
    assert np.all(np.abs(h_g - h_o) <= UNITS * U * cy[:, 0] + 1e-13 * np.abs(h_o))
    # Free flight lets every accepted attempt grow the step by (1.5 + relax) / (1 + relax): after ~80 attempts the
    # coordinates' rounding exceeds the error scale and the step control follows the rounding, so fixed attempts
    # are compared over 40 (a real trajectory meets rmax or tmax within ~35).
    n, na = 16, 40
    t0, dt0 = np.zeros(n), np.full(n, cfg.dt0)
    a, ta, _ = o.bs_attempts(y[:n], t0, dt0, erra[:n], na)
    tr = api.Trajectories.start(y[:n], erra[:n], cfg.dt0)
    api.ODE(H).Integrate(tr, na)
    assert np.array_equal(tr.paq[:, :9], y[:n, :9])
    rel = np.abs(tr.paq - a).max(axis=1) / np.abs(a).max(axis=1)
    print("PIPNN %d attempts: max rel %.2e" % (na, rel.max()))
    assert np.all(rel < 1e-12) and np.allclose(tr.t, ta, rtol=1e-14)
    H.close()


def test_pipnn_queue_matches_oracle(gpu_lib, oracle_lib):
    from test_gpu_o4 import _fs_tuple
    cfg, o, H = _setup()
    lv = systems.load_levels("N2")
    rows = lv[[0, 30, 200]]
    entries = [(0, 0, 16, api.process_seed(9, 1), 20000.0, 8.0, 23.0, 1),
               (1, 0, 16, api.process_seed(9, 2), 10000.0, 8.0, 23.0, 2)]
    items = api.work_items(entries)
    res = api.RunTrajectories(H).run(api.level_table(rows), items)
    assert np.all(res["status"] == 0)
    qn = lambda x: (np.sign(x) * np.floor(np.abs(x) + 0.5)).astype(int)
    same, stable, same_i = [], [], []
    for i, (il, ipes, nt, seed, T, bmax, dinit, il2) in enumerate(entries):
        ref = o.sample_ics4(nt, rows[il], rows[il2], ttra=T, bmax=bmax, dinit=dinit, seed=seed)
        a = o.integrate(ref["paq"], ref["erra"])
        b = o.integrate(ref["paq"] * (1 + 1e-14), ref["erra"])
        fa = [_fs_tuple(f) for f in o.analyze(o.apply_transformation(a["paq"]))]
        fb = [_fs_tuple(f) for f in o.analyze(o.apply_transformation(b["paq"]))]
        fi = [_fs_tuple(f) for f in o.analyze(ref["paq0"])]
        r = res[int(items["first"][i]):int(items["first"][i]) + nt]
        fg = [tuple(int(x) for x in t) for t in zip(qn(r["j_f"] - 0.5), qn(r["v_f"] - 0.5), qn(r["j2_f"] - 0.5),
                                                     qn(r["v2_f"] - 0.5), qn(r["arr_f"] - 0.5))]
        gi = [tuple(int(x) for x in t) for t in zip(qn(r["j_i"] - 0.5), qn(r["v_i"] - 0.5), qn(r["j2_i"] - 0.5),
                                                     qn(r["v2_i"] - 0.5), qn(r["arr_i"] - 0.5))]
        print("PIPNN queue item %d: final states %s" % (i, sorted(set(fg))))
        same += [x == y for x, y in zip(fg, fa)]
        stable += [x == y for x, y in zip(fa, fb)]
        same_i += [x == y for x, y in zip(gi, fi)]
    same, stable = np.array(same), np.array(stable)
    assert all(same_i) and stable.mean() >= 0.9 and same[stable].mean() >= 0.995
    H.close()
