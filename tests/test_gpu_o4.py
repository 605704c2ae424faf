"""GPU parity of the four-atom path (O2 + O2 on the O4 UMN surfaces) against the oracle.

Same criteria as the three-atom tests: surface energies and gradients to 1e-12 relative or the
rounding-level bound of the evaluation, whichever is larger; right-hand side and Hamiltonian
likewise; phase-space points after 1000 fixed Bulirsch-Stoer attempts to 1e-9 on trajectories that
the oracle itself shows to be non-chaotic.  The O4 PIP is 95 products deep over 430 basis terms,
so its longest gradient chain is about 2 x 95 + 430 + 10 = 630 operations.
"""
import os

import numpy as np
import pytest

from coarseair_gb300 import api, systems

pytestmark = pytest.mark.gpu
PROCS = min(16, os.cpu_count() or 1)
ROUND_O4 = 2 * 630 * 1.1102230246251565e-16
SURFACES = ("UMN_Singlet", "UMN_Triplet", "UMN_Quintet")


def _setup():
    from oracle import Oracle
    cfg = systems.o4_config()
    o = Oracle(cfg)
    H = api.Handle(cfg, tpq=o.tpq)
    return cfg, o, H


def _geometries(o, n, seed):
    rng = np.random.default_rng(seed)
    out = []
    while sum(len(x) for x in out) < n:
        Q = rng.uniform(-3.5, 3.5, size=(4 * n, 9))
        R, Qall = o.rp(Q)
        keep = np.all((R > 1.6) & (R < 10.0), axis=1)
        out.append(Qall[keep])
    Qall = np.concatenate(out)[:n]
    return o.rp(Qall[:, :9])


def _collision_points(o, cfg, n, seed, sep=9.0, ekin=0.03):
    """O2 + O2 phase points: both bonds near 2.28 bohr, random orientations and small rotations,
    centres `sep` bohr apart approaching with relative kinetic energy `ekin` Eh; p = Tqp qdot."""
    rng = np.random.default_rng(seed)
    m = np.asarray(cfg.masses)
    pts = []
    for _ in range(n):
        X = np.zeros((4, 3))
        Vv = np.zeros((4, 3))
        for k, c in enumerate((np.array([0.0, 0.0, -sep / 2]), np.array([rng.uniform(-2, 2), 0.0, sep / 2]))):
            u = rng.normal(size=3)
            u /= np.linalg.norm(u)
            r = 2.28 + rng.uniform(-0.05, 0.05)
            X[2 * k] = c + 0.5 * r * u
            X[2 * k + 1] = c - 0.5 * r * u
            w = np.cross(u, rng.normal(size=3)) * 2e-4
            Vv[2 * k] = w
            Vv[2 * k + 1] = -w
        mu = (m[0] + m[1]) * (m[2] + m[3]) / (m.sum())
        vrel = np.sqrt(2 * ekin / mu)
        Vv[:2, 2] += vrel * (m[2] + m[3]) / m.sum()
        Vv[2:, 2] -= vrel * (m[0] + m[1]) / m.sum()
        X -= (m[:, None] * X).sum(0) / m.sum()
        Vv -= (m[:, None] * Vv).sum(0) / m.sum()
        q, qd = X[:3].ravel(), Vv[:3].ravel()
        p = o.tqp @ qd
        pts.append(np.concatenate([p, q]))
    y = np.array(pts)
    ep = cfg.eps * np.sqrt(np.mean(y[:, :9] ** 2, axis=1))   # SetErrorFactor: momenta RMS for both halves
    erra = np.repeat(ep[:, None], 18, axis=1)
    return y, erra


def _bound_check(err, ref_scale, cs, floor, name):
    b = np.maximum(1e-12 * np.maximum(ref_scale, floor), ROUND_O4 * cs)
    frac = np.mean(err <= 1e-12 * np.maximum(ref_scale, floor))
    print("%s: worst/bound %.2e, %.4f within 1e-12" % (name, (err / b).max(), frac))
    assert np.all(err <= b)


@pytest.mark.parametrize("ipes", [0, 1, 2])
def test_o4_surface_parity(gpu_lib, oracle_lib, ipes):
    cfg, o, H = _setup()
    R, Qall = _geometries(o, 384, 5 + ipes)
    ip = np.full(len(R), ipes, np.int32)
    V_o, g_o, m_o = o.compute(R, Qall, ipes=ip)
    V_g, g_g, m_g = api.PES(H).Compute(R, Qall, ipes=ip)
    Ve = api.PES(H).Potential(R, Qall, ipes=ip)
    cs = o.condition_scale(R, ipes=ip)
    _bound_check(np.abs(V_g - V_o), np.abs(V_o), cs[:, 0], 0.1, "O4 %s V" % SURFACES[ipes])
    _bound_check(np.abs(Ve - V_o), np.abs(V_o), cs[:, 0], 0.1, "O4 %s V (energy only)" % SURFACES[ipes])
    gs = np.abs(g_o).max(axis=1, keepdims=True)
    _bound_check(np.abs(g_g - g_o), gs, cs[:, 1:], 1e-2, "O4 %s dV/dR" % SURFACES[ipes])
    ms = np.abs(m_o).max(axis=1, keepdims=True)
    _bound_check(np.abs(m_g - m_o), ms, cs[:, 1:].max(axis=1, keepdims=True), 1e-2, "O4 %s dV/dQ" % SURFACES[ipes])


def test_o4_rhs_and_hamiltonian_parity(gpu_lib, oracle_lib):
    cfg, o, H = _setup()
    y, _ = _collision_points(o, cfg, 96, 11)
    ip = np.arange(len(y), dtype=np.int32) % 3
    yp_o = o.rhs(y, ipes=ip)
    yp_g = api.Collision(H).EvaluateRHS(y, ipes=ip)
    R, _ = o.rp(y[:, 9:])
    cs = o.condition_scale(R, ipes=ip)
    _bound_check(np.abs(yp_g - yp_o), np.abs(yp_o).max(axis=1, keepdims=True),
                 cs[:, 1:].max(axis=1, keepdims=True), 1e-12, "O4 RHS")
    h_o, r_o = o.hamiltonian(y, ipes=ip)
    h_g, r_g = api.Collision(H).Hamiltonian(y, ipes=ip)
    _bound_check(np.abs(h_g - h_o), np.abs(h_o), cs[:, 0], 0.1, "O4 H")
    assert np.allclose(r_g, r_o, rtol=4e-16, atol=0)


def test_o4_phase_space_after_1000_attempts(gpu_lib, oracle_lib):
    cfg, o, H = _setup()
    y, erra = _collision_points(o, cfg, 24, 12)
    ip = np.arange(len(y), dtype=np.int32) % 3
    n, nattempts = len(y), 1000
    t0, dt0 = np.zeros(n), np.full(n, cfg.dt0)
    a, _, _ = o.bs_attempts(y, t0, dt0, erra, nattempts, ipes=ip)
    b, _, _ = o.bs_attempts(y * (1 + 1e-14), t0, dt0, erra, nattempts, ipes=ip)
    ok = np.abs(a - b).max(axis=1) / np.abs(a).max(axis=1) < 1e-11
    assert ok.sum() >= 4, "too few non-chaotic trajectories in the sample"
    tr = api.Trajectories.start(y, erra, cfg.dt0, ipes=ip)
    api.ODE(H).Integrate(tr, nattempts)
    rel = np.abs(tr.paq - a).max(axis=1) / np.abs(a).max(axis=1)
    print("O4 1000 attempts: %d non-chaotic, max rel %.2e" % (ok.sum(), rel[ok].max()))
    assert np.all(rel[ok] < 1e-9), rel[ok]


def test_o4_integrate_to_end(gpu_lib, oracle_lib):
    """Whole collisions: both sides finish every trajectory; on the trajectories whose oracle
    outcome is stable under a 1e-14 perturbation, the final points agree to 1e-6."""
    cfg, o, H = _setup()
    y, erra = _collision_points(o, cfg, 32, 13)
    ip = np.arange(len(y), dtype=np.int32) % 3
    ref = o.integrate(y, erra, ipes=ip, procs=PROCS)
    pert = o.integrate(y * (1 + 1e-14), erra, ipes=ip, procs=PROCS)
    tr = api.Trajectories.start(y, erra, cfg.dt0, ipes=ip)
    api.Integrator(H).Integrate(tr)
    assert np.all(tr.status == 0) and np.all(ref["status"] == 0)
    scale = np.abs(ref["paq"]).max(axis=1)
    stable = np.abs(pert["paq"] - ref["paq"]).max(axis=1) / scale < 1e-9
    rel = np.abs(tr.paq - ref["paq"]).max(axis=1) / scale
    print("O4 to the end: %d of %d stable, max rel on stable %.2e" % (stable.sum(), len(y), rel[stable].max()))
    assert stable.sum() >= 4
    assert np.all(rel[stable] < 1e-6)
    h_o, _ = o.hamiltonian(tr.paq, ipes=ip)
    assert np.max(np.abs(tr.H - h_o)) < 1e-9
    assert np.max(np.abs(tr.H - o.hamiltonian(y, ipes=ip)[0])) < cfg.ham_abs_tol


def _o4_items(lv):
    from coarseair_gb300 import api as _api
    rows = lv[[0, 40, 120]]
    table = _api.level_table(rows)
    entries = [(0, 0, 12, _api.process_seed(3, 1), 10000.0, 8.0, 18.0, 1),
               (1, 1, 12, _api.process_seed(3, 2), 10000.0, 8.0, 18.0, 2),
               (2, 2, 12, _api.process_seed(3, 3), 10000.0, 8.0, 18.0, 0)]
    return rows, table, entries, _api.work_items(entries)


def test_o4_device_initial_conditions_match_oracle(gpu_lib, oracle_lib):
    """SetIniCondForward for diatom + diatom on the device against the oracle's stream."""
    cfg, o, H = _setup()
    lv = systems.load_levels("O2")
    rows, table, entries, items = _o4_items(lv)
    ic = api.InitialConditions(H).sample(table, items)
    for i, e in enumerate(entries):
        il, ipes, nt, seed, T, bmax, dinit, il2 = e
        ref = o.sample_ics4(nt, rows[il], rows[il2], ttra=T, bmax=bmax, dinit=dinit, seed=seed)
        sl = slice(int(items["first"][i]), int(items["first"][i] + nt))
        for key in ("paq", "paq0", "erra"):
            sc = np.abs(ref[key]).max(axis=1, keepdims=True)
            assert np.all(np.abs(ic[key][sl] - ref[key]) <= 1e-10 * sc), key
        # H0 on the item's surface
        h_ref, _ = o.hamiltonian(ref["paq"], ipes=np.full(nt, ipes))
        assert np.all(np.abs(ic["H0"][sl] - h_ref) <= 1e-11 * np.maximum(np.abs(h_ref), 0.1))
        assert np.allclose(ic["b"][sl], ref["b"], rtol=1e-14, atol=0)


def _fs_tuple(f):
    qn = lambda x: int(np.sign(x) * np.floor(abs(x) + 0.5))
    return (qn(f["angmom"] - 0.5), qn(f["viba"] - 0.5), qn(f["angmom1"] - 0.5), qn(f["viba1"] - 0.5),
            16 * f["ipair"] + f["itype"] + 4 * f["itype1"])


def test_o4_final_state_analysis_on_identical_points(gpu_lib, oracle_lib):
    cfg, o, H = _setup()
    y, erra = _collision_points(o, cfg, 16, 17)
    ip = np.arange(len(y), dtype=np.int32) % 3
    res = o.integrate(y, erra, ipes=ip, procs=PROCS)
    pts = np.concatenate([o.apply_transformation(y), o.apply_transformation(res["paq"])])
    fo = o.analyze(pts)
    fg = api.MolecularState(H).FindState(pts)
    for k, f in enumerate(fo):
        g = fg[k]
        gd = dict(angmom=g["angmom0"], viba=g["viba0"], angmom1=g["angmom1"], viba1=g["viba1"],
                  ipair=g["ipair0"], itype=g["itype0"], itype1=g["itype1"])
        assert _fs_tuple(gd) == _fs_tuple(f)
        assert g["ipair1"] == f["ipair1"]
        assert np.allclose([g["viba0"], g["viba1"]], [f["viba"], f["viba1"]], rtol=1e-9, atol=1e-12)
        assert np.allclose([g["angmom0"], g["angmom1"]], [f["angmom"], f["angmom1"]], rtol=1e-12, atol=1e-12)


def test_o4_run_queue_matches_oracle(gpu_lib, oracle_lib):
    """cair_run_queue for O2 + O2 on the three surfaces: final (J1, v1, J2, v2, arrangement) equal
    to the oracle's on the trajectories whose oracle outcome is stable under a 1e-14 perturbation."""
    cfg, o, H = _setup()
    lv = systems.load_levels("O2")
    rows, table, entries, items = _o4_items(lv)
    res = api.RunTrajectories(H).run(table, items)
    assert np.all(res["status"] == 0)
    assert np.max(np.abs(res["dH"])) < cfg.ham_abs_tol
    same, stable = [], []
    for i, e in enumerate(entries):
        il, ipes, nt, seed, T, bmax, dinit, il2 = e
        ref = o.sample_ics4(nt, rows[il], rows[il2], ttra=T, bmax=bmax, dinit=dinit, seed=seed)
        ipv = np.full(nt, ipes, np.int32)
        a = o.integrate(ref["paq"], ref["erra"], ipes=ipv, procs=PROCS)
        b = o.integrate(ref["paq"] * (1 + 1e-14), ref["erra"], ipes=ipv, procs=PROCS)
        fa = [_fs_tuple(f) for f in o.analyze(o.apply_transformation(a["paq"]))]
        fb = [_fs_tuple(f) for f in o.analyze(o.apply_transformation(b["paq"]))]
        sl = slice(int(items["first"][i]), int(items["first"][i] + nt))
        r = res[sl]
        qn = lambda x: (np.sign(x) * np.floor(np.abs(x) + 0.5)).astype(int)
        fg = list(zip(qn(r["j_f"] - 0.5), qn(r["v_f"] - 0.5), qn(r["j2_f"] - 0.5), qn(r["v2_f"] - 0.5),
                      qn(r["arr_f"] - 0.5)))
        same += [tuple(int(x) for x in g) == f for g, f in zip(fg, fa)]
        stable += [x == y for x, y in zip(fa, fb)]
        fi = [_fs_tuple(f) for f in o.analyze(ref["paq0"])]
        gi = list(zip(qn(r["j_i"] - 0.5), qn(r["v_i"] - 0.5), qn(r["j2_i"] - 0.5), qn(r["v2_i"] - 0.5),
                      qn(r["arr_i"] - 0.5)))
        assert [tuple(int(x) for x in g) for g in gi] == fi
    same, stable = np.array(same), np.array(stable)
    print("O4 queue: GPU vs oracle %.4f overall, %.4f on oracle-stable (%d of %d stable)" %
          (same.mean(), same[stable].mean(), stable.sum(), len(stable)))
    assert stable.sum() >= len(stable) // 2
    assert same[stable].mean() >= 0.995
