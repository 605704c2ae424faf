"""N4 UMN PIPNN (N4_UMN_PIPNN_PES_Class.F90) and its N2 UMN_PIPNN_ForN4 diatomic on the CPU.

The oracle is pinned on the reference's own numbers: the three networks evaluated at infinite
separation (every basis function zero) give the VInfSurface constants the reference subtracts
(N4_UMN_PIPNN_PES_Class.F90:96), to 2e-13 kcal/mol.  Its energy is checked against a numpy
restatement of getpot; its Compute against the reference's central differences and dVdQ = 0.  The
loader reads Weights.dat / Biases.dat with the reference's record rules and parameter count.  The
device code (cair_device.cuh, through the host harness of test_pes_host) is held to the oracle: the
surface at random N2 + N2 geometries, the diatomic, fixed Bulirsch-Stoer attempts (no force: the
momenta stay as they are), and the whole queue pipeline for two N2 levels.

The surface's output is a cancellation: 23.0605 times a network output of ~1e5 kcal/mol summed from
terms of both signs, de-normalised, comes to tens of kcal/mol.  Its rounding scale (the oracle's
condition_scale: the magnitudes summed at the top, times the cancellation below them) is ~200 Eh, and
the tolerances are units of that scale: the host code without fused multiply-adds is within 60 of
them, with them (an FMA build of the same harness) within 150."""
import ctypes as C

import numpy as np
import pytest

from coarseair_gb300 import api, systems
from test_pes_host import U, _harness, _host_eval, _levels_for_oracle, _points, _queue_host, _setup

VINF = (-0.021346263746904, -0.196886061330806, -0.030606048118131)   # N4_UMN_PIPNN_PES_Class.F90:96
HOST_UNITS = 512


def _oracle(model="UMN_PIPNN", **kw):
    from oracle import Oracle
    cfg = systems.n4pipnn_config(model, **kw)
    return cfg, Oracle(cfg)


def test_loader_reads_the_three_networks():
    s = systems.load_n4_pipnn()
    c = s.coef
    assert s.model == systems.PES_N4_PIPNN and c.size == 8 + 3 * 2570
    assert list(c[:8]) == [1, 1, 1, 1, 276, 5, 90, 1]
    for k in range(3):
        net = c[8 + 2570 * k: 8 + 2570 * (k + 1)]
        pdel, pavg = net[:277], net[277:554]
        assert np.all(pdel > 0) and np.all(np.isfinite(net))
        # the shipped fit normalises every input by its own mean: pdel = pavg for the 276 inputs
        assert np.array_equal(pdel[:276], pavg[:276]) and pdel[276] != pavg[276]
    for name, use in systems.PIPNN_VARIANTS.items():
        assert tuple(systems.load_n4_pipnn(name).coef[:3]) == use


def test_networks_at_infinite_separation_give_the_reference_vinf(oracle_lib):
    """At infinite separation every basis function is zero; each network's value there, in kcal/mol, is
    the constant the reference subtracts for it."""
    L = oracle_lib.lib()
    c = np.ascontiguousarray(systems.load_n4_pipnn().coef)
    zero = np.zeros(276)
    for k in range(3):
        v = L.orc_pipnn_net(oracle_lib.dp(c), k, oracle_lib.dp(zero)) * 23.0605
        assert abs(v - VINF[k]) < 2e-13, (k, v, VINF[k])


def _numpy_net(net, ifunc, b):
    pdel, pavg = net[:277], net[277:554]
    W1 = net[554:554 + 1380].reshape(5, 276).T
    b1 = net[1934:1939]
    W2 = net[1939:2389].reshape(90, 5).T
    b2, W3, b3 = net[2389:2479], net[2479:2569], net[2569]
    f = np.tanh if ifunc == 1 else (lambda z: 1 / (1 + np.exp(-z))) if ifunc == 2 else (lambda z: z)
    h1 = f(b1 + ((b - pavg[:276]) / pdel[:276]) @ W1)
    h2 = f(b2 + h1 @ W2)
    return (b3 + h2 @ W3) * pdel[276] + pavg[276]


def _numpy_pair(rang):
    a = [2.7475450369759, 0.218868498415108, 0.248885765371433, -0.229295466336412, -0.653389048592838,
         1.03611964035396, 1.71287482791961]
    re, de = 1.098, 225.213
    y = (rang ** 4 - re ** 4) / (rang ** 4 + re ** 4)
    u = np.exp(-sum(c * y ** i for i, c in enumerate(a)) * (rang - re))
    rb = rang / 0.52917721092
    c6, c8 = 19.7, 3 * 19.7 * 2.71175247 ** 2
    s = 0.5299 * np.sqrt(c8 / c6) + 2.20
    return de * (1 - u) ** 2 - de + (-c6 / (rb ** 6 + s ** 6) - 2 * c8 / (rb ** 8 + s ** 8)) / 0.159360144e-2


@pytest.mark.parametrize("model", ["UMN_PIPNN", "UMN_PIPNN_B"])
def test_energy_against_a_numpy_restatement(oracle_lib, model):
    cfg, o = _oracle(model)
    L = oracle_lib.lib()
    c = cfg.surfaces[0].coef
    R, _ = _points(o, 4, 40, 3)
    cs = o.condition_scale(R)
    use = [k for k in range(3) if c[k] == 1]
    for r, s in zip(R, cs):
        rang = r * 0.52917721092
        b = np.zeros(276)
        L.orc_pip_basis(1, oracle_lib.dp(np.exp(-rang)), oracle_lib.dp(b), None)
        nn = np.mean([_numpy_net(c[8 + 2570 * k: 8 + 2570 * (k + 1)], 1, b) for k in use])
        v = (nn * 23.0605 + _numpy_pair(rang).sum() - np.mean([VINF[k] for k in use])) * 0.159360144e-2
        assert abs(v - o.potential(r[None])[0]) <= 4096 * U * s[0]


def test_networks_vanish_when_the_atoms_separate(oracle_lib):
    """Far apart only the pair terms' dispersion tails remain: the networks' part minus VInf is zero."""
    cfg, o = _oracle()
    L = oracle_lib.lib()
    for r in (40.0, 80.0):
        R = np.full((1, 6), r)
        pairs = 6 * L.orc_diat_V(systems.DIAT_N2_UMN_PIPNN_FORN4, r)
        assert abs(pairs) > 1e-11 and abs(o.potential(R)[0] - pairs) < 1e-14


def test_compute_is_the_central_difference_and_no_force(oracle_lib):
    """Compute: V, dVdR from n4pipNN's central differences over 1e-5 Ang, one bond at a time, dVdQ zero."""
    cfg, o = _oracle()
    L = oracle_lib.lib()
    c = np.ascontiguousarray(cfg.surfaces[0].coef)
    R, Qall = _points(o, 4, 12, 5)
    V, g, m = o.compute(R, Qall)
    assert np.all(m == 0.0)
    kcal = lambda rb: L.orc_pipnn_kcal(oracle_lib.dp(c), oracle_lib.dp(np.ascontiguousarray(rb)))
    for r, v, gk in zip(R, V, g):
        rb = r * 0.52917721092
        assert v == kcal(rb) * 0.159360144e-2
        p = rb.copy()                      # the bonds carry each restoration's rounding to the next
        for i in range(6):
            p[i] = p[i] + 1e-5
            vp = kcal(p)
            p[i] = p[i] - 2 * 1e-5
            vm = kcal(p)
            assert gk[i] == ((vp - vm) / (2 * 1e-5)) * 0.843297564e-3
            p[i] = p[i] + 1e-5
        # and the difference is the derivative: a step three times larger agrees to its O(h^2) term
        for i in range(6):
            p, q = rb.copy(), rb.copy()
            p[i] += 3e-5
            q[i] -= 3e-5
            coarse = (kcal(p) - kcal(q)) / 6e-5 * 0.843297564e-3
            assert abs(coarse - gk[i]) < 2e-5 * max(abs(gk[i]), 1e-2)


def test_variants_are_single_networks_and_their_mean(oracle_lib):
    R = _points(_oracle()[1], 4, 10, 9)[0]
    v = {m: _oracle(m)[1].potential(R) for m in systems.PIPNN_VARIANTS}
    mean = (v["UMN_PIPNN_A"] + v["UMN_PIPNN_B"] + v["UMN_PIPNN_C"]) / 3
    scale = _oracle()[1].condition_scale(R)[:, 0]
    assert np.all(np.abs(v["UMN_PIPNN"] - mean) <= 64 * U * scale)
    assert not np.allclose(v["UMN_PIPNN_A"], v["UMN_PIPNN_B"])


def test_pipnn_diatomic(oracle_lib):
    """N2 UMN_PIPNN_ForN4: the surface's own pair term in hartree; a well of De = 225.213 kcal/mol deepened by
    the dispersion (to 228.7, the UMN_ForN4 diatomic's De) near re = 1.098 Ang; dV/dR its derivative."""
    L = oracle_lib.lib()
    D = systems.DIAT_N2_UMN_PIPNN_FORN4
    r = np.linspace(1.6, 12.0, 60)
    v = np.array([L.orc_diat_V(D, x) for x in r])
    ref = _numpy_pair(r * 0.52917721092) * 0.159360144e-2
    assert np.allclose(v, ref, rtol=1e-12, atol=1e-15)
    vmin = min(L.orc_diat_V(D, x) for x in np.linspace(2.0, 2.15, 301))
    assert -228.8 * 0.159360144e-2 < vmin < -228.6 * 0.159360144e-2
    for x in (1.8, 2.1, 3.0, 5.0):
        vv, dv = C.c_double(), C.c_double()
        L.orc_diat_VdV(D, x, C.byref(vv), C.byref(dv))
        fd = (L.orc_diat_V(D, x + 1e-6) - L.orc_diat_V(D, x - 1e-6)) / 2e-6
        assert vv.value == L.orc_diat_V(D, x) and abs(dv.value - fd) < 1e-7


def test_device_surface_code_on_the_host(gpu_lib, oracle_lib):
    cfg, o = _oracle()
    L = _harness()
    setup = _setup(gpu_lib, cfg, o.tpq)
    R, Qall = _points(o, 4, 160, 11)
    ip = np.zeros(len(R), np.int32)
    V, g, m = _host_eval(L, setup, R, Qall, ip)
    Vo, go, mo = o.compute(R, Qall)
    cs = o.condition_scale(R)
    print("PIPNN host: V %.1f, dV/dR %.1f units of the scale" %
          (np.max(np.abs(V - Vo) / (U * cs[:, 0])), np.max(np.abs(g - go) / (U * cs[:, 1:]))))
    assert np.all(np.abs(V - Vo) <= HOST_UNITS * U * cs[:, 0])
    assert np.all(np.abs(g - go) <= HOST_UNITS * U * cs[:, 1:])
    assert np.all(m == 0.0)
    Ve, _, _ = _host_eval(L, setup, R, Qall, ip, grad=False)
    assert np.array_equal(Ve, V)


def test_device_diatomic_on_the_host(gpu_lib, oracle_lib):
    cfg, o = _oracle(diat=systems.DIAT_N2_UMN_PIPNN_FORN4)
    L = _harness()
    L.diat_host_eval.restype = None
    L.diat_host_eval.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]
    devsys = _setup(gpu_lib, cfg, o.tpq)[0]
    r = np.linspace(1.5, 20.0, 200)
    v, dv = np.zeros_like(r), np.zeros_like(r)
    L.diat_host_eval(devsys, r.size, r.ctypes.data, v.ctypes.data, dv.ctypes.data)
    ol = o.L
    for x, a, b in zip(r, v, dv):
        vv, dd, sv, sd = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        ol.orc_diat_VdV(3, x, C.byref(vv), C.byref(dd))
        ol.orc_diat_scale(3, C.c_double(x), C.byref(sv), C.byref(sd))
        assert abs(a - vv.value) <= 64 * U * sv.value and abs(b - dd.value) <= 64 * U * sd.value


def test_device_attempts_on_the_host_feel_no_force(gpu_lib, oracle_lib):
    """Fixed Bulirsch-Stoer attempts of the device code: the momenta do not change, the coordinates move
    as the oracle's.  In free flight every accepted attempt grows the step by a third; 40 attempts stay well
    short of the ~80 after which the coordinates' rounding exceeds the error scale and drives the step
    control."""
    cfg, o = _oracle()
    L = _harness()
    devsys, packed, offsets, _ = _setup(gpu_lib, cfg, o.tpq)
    lv = _levels_for_oracle(systems.load_levels("N2")[[0, 30]])
    ic = o.sample_ics4(6, lv[0], lv[1], ttra=20000.0, bmax=8.0, dinit=23.0, seed=4)
    y = np.ascontiguousarray(ic["paq"]).copy()
    e = np.ascontiguousarray(ic["erra"])
    n = len(y)
    t, dt, ip = np.zeros(n), np.full(n, cfg.dt0), np.zeros(n, np.int32)
    assert L.pes_host_bs_steps(devsys, packed.ctypes.data, offsets.ctypes.data, n, ip.ctypes.data, y.ctypes.data,
                               t.ctypes.data, dt.ctypes.data, e.ctypes.data, 40) == 0
    a, ta, dta = o.bs_attempts(ic["paq"], np.zeros(n), np.full(n, cfg.dt0), ic["erra"], 40)
    assert np.array_equal(y[:, :9], ic["paq"][:, :9])
    assert np.allclose(y, a, rtol=1e-12, atol=1e-12 * np.abs(a).max()) and np.allclose(t, ta, rtol=1e-12)


def test_queue_pipeline_on_the_host(gpu_lib, oracle_lib):
    """N2 + N2 on the PIPNN surface through the host pipeline: initial states and energies as the
    oracle's, and, the motion being force-free, every final state equal to the oracle's."""
    from test_gpu_o4 import _fs_tuple
    cfg, o = _oracle()
    L = _harness()
    setup = _setup(gpu_lib, cfg, o.tpq)
    rows = systems.load_levels("N2")[[0, 30]]
    entries = [(0, 0, 10, api.process_seed(7, 1), 20000.0, 8.0, 23.0, 1)]
    items = api.work_items(entries)
    res = _queue_host(L, setup, cfg, api.level_table(rows), items, cfg.max_attempts)
    assert np.all(res["status"] == 0)
    lv = _levels_for_oracle(rows)
    ref = o.sample_ics4(10, lv[0], lv[1], ttra=20000.0, bmax=8.0, dinit=23.0, seed=entries[0][3])
    a = o.integrate(ref["paq"], ref["erra"])
    fa = [_fs_tuple(f) for f in o.analyze(o.apply_transformation(a["paq"]))]
    qn = lambda x: (np.sign(x) * np.floor(np.abs(x) + 0.5)).astype(int)
    fg = [tuple(int(x) for x in t) for t in zip(qn(res["j_f"] - 0.5), qn(res["v_f"] - 0.5), qn(res["j2_f"] - 0.5),
                                                 qn(res["v2_f"] - 0.5), qn(res["arr_f"] - 0.5))]
    gi = [tuple(int(x) for x in t) for t in zip(qn(res["j_i"] - 0.5), qn(res["v_i"] - 0.5), qn(res["j2_i"] - 0.5),
                                                 qn(res["v2_i"] - 0.5), qn(res["arr_i"] - 0.5))]
    fi = [_fs_tuple(f) for f in o.analyze(ref["paq0"])]
    print("PIPNN queue on the host: initial states", sorted(set(gi)), "final states", sorted(set(fg)))
    assert fg == fa and gi == fi


def test_setup_refuses_what_is_not_built(gpu_lib):
    """cair_create's checks (the part that needs no GPU): the UseSurface flags, iFunc, the network shape,
    the coefficient count, and the PIPNN diatomic with another surface."""
    import dataclasses
    lib = C.CDLL(gpu_lib)
    lib.cair_internal_devsys_size.restype = C.c_int64
    lib.cair_internal_setup_system.restype = C.c_int
    lib.cair_internal_setup_system.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p,
                                               C.c_char_p, C.c_int]
    size = lib.cair_internal_devsys_size()

    def setup(cfg):
        d, keep = api.system_desc(cfg)
        devsys, packed, offsets = (C.c_char * size)(), np.zeros(64 * 512), np.zeros(65, np.int64)
        err = C.create_string_buffer(256)
        rc = lib.cair_internal_setup_system(C.addressof(d), devsys, size, packed.ctypes.data, packed.size,
                                            offsets.ctypes.data, err, 256)
        return rc, err.value.decode()

    cfg = systems.n4pipnn_config()
    assert setup(cfg) == (0, "")
    assert setup(systems.n4pipnn_config(diat=systems.DIAT_N2_UMN_PIPNN_FORN4))[0] == 0

    def edited(fn):
        s = systems.load_n4_pipnn()
        return dataclasses.replace(cfg, surfaces=[dataclasses.replace(s, coef=fn(s.coef.copy()))])

    def put(i, v):
        def f(c):
            c[i] = v
            return c
        return f

    assert setup(edited(lambda c: np.concatenate([[0.0, 0.0, 0.0], c[3:]])))[0] == 1
    assert setup(edited(put(1, 0.5)))[0] == 1
    assert setup(edited(put(3, 4.0)))[0] == 1
    assert setup(edited(put(5, 6.0)))[0] == 5
    assert setup(edited(lambda c: c[:-1]))[0] == 1
    assert setup(edited(put(100, np.nan)))[0] == 4
    assert setup(dataclasses.replace(systems.n4_config(), diat_model=systems.DIAT_N2_UMN_PIPNN_FORN4))[0] == 5
    assert setup(dataclasses.replace(cfg, diat_model=4))[0] == 1
