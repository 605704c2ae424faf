"""The library's device surface and integrator code on the CPU: coarseair_gb300/csrc/cair_device.cuh compiled unchanged
by the host compiler (tests/host_pes/pes_host.cpp, CUDA qualifiers defined away), with the DevSys and
the packed coefficients from the library's own setup (cair_internal_setup_system, the part of
cair_create that needs no GPU).  Every surface model -- O3, N3, O4, N4 UMN, the nine-surface O3 mix,
O3 NN and the O3 BNN samples -- against the oracle at the same points, energies and gradients to
1e-12 relative or the rounding-level bound of the GPU parity tests, and the energy-only path against
the oracle's Potential; the device Bulirsch-Stoer attempt (Rhs, bs_attempt) over 1000 fixed attempts
against the oracle on the trajectories the oracle shows to be non-chaotic, to 1e-9 as on the GPU; and
the initial-condition kernels (the stream code of k_ic_draws, the bodies of k_sample_ic3/4 run over a
1 x 1 grid) for impact-parameter rings of every strata type against the oracle's stream; and the whole
queue pipeline (k_integrate as one lane, k_results) for stratified rings and for the 50 BNN samples.
This checks the surface and integrator arithmetic and the coefficient packing; the GPU tests check
the same code as nvcc builds it."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from coarseair_gb300 import _lib, api, systems

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HARNESS = os.path.join(ROOT, "tests", "host_pes", "pes_host.so")
U = 1.1102230246251565e-16


def _harness():
    src = [os.path.join(ROOT, "tests", "host_pes", "pes_host.cpp"), os.path.join(ROOT, "include", "cair_gpu.h")]
    csrc = os.path.join(ROOT, "coarseair_gb300", "csrc")
    src += [os.path.join(csrc, f) for f in ("cair_stats_host.cpp", "cair_device.cuh", "cair_kernels.cuh",
                                            "cair_ic.cuh", "cair_stats.cuh", "cair_stats_host.h", "cair_warp.cuh")]
    src += [os.path.join(csrc, "generated", f) for f in os.listdir(os.path.join(csrc, "generated"))]
    if not os.path.exists(HARNESS) or os.path.getmtime(HARNESS) < max(os.path.getmtime(f) for f in src):
        subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-I", os.path.join(ROOT, "include"),
                        "-o", HARNESS, src[0], src[2]], check=True)
    L = C.CDLL(HARNESS)
    L.pes_host_devsys_size.restype = C.c_int64
    L.pes_host_eval.restype = C.c_int
    L.pes_host_eval.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
    L.ic_host_sample.restype = C.c_int
    L.ic_host_sample.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int64] + \
        [C.c_void_p] * 6
    L.stats_host_run.restype = C.c_int
    L.stats_host_run.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                 C.c_int64, C.c_void_p]
    L.queue_host_run.restype = C.c_int
    L.queue_host_run.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_int64,
                                 C.c_int64, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_double, C.c_void_p]
    L.handoff_host_run.restype = C.c_int
    L.handoff_host_run.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_int64,
                                   C.c_longlong] + [C.c_void_p] * 9
    L.host_fexp.restype = None
    L.host_fexp.argtypes = [C.c_int64, C.c_void_p, C.c_void_p]
    L.warp_host_eval.restype = C.c_int
    L.warp_host_eval.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.c_void_p]
    L.pes_host_bs_steps.restype = C.c_int
    L.pes_host_bs_steps.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_int]
    return L


def _setup(gpu_lib, cfg, tpq):
    lib = C.CDLL(gpu_lib)
    lib.cair_internal_devsys_size.restype = C.c_int64
    lib.cair_internal_setup_system.restype = C.c_int
    lib.cair_internal_setup_system.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p,
                                               C.c_char_p, C.c_int]
    size = lib.cair_internal_devsys_size()
    d, keep = api.system_desc(cfg, tpq)
    devsys = (C.c_char * size)()
    packed = np.zeros(64 * 512)
    offsets = np.zeros(65, np.int64)
    err = C.create_string_buffer(256)
    rc = lib.cair_internal_setup_system(C.addressof(d), devsys, size, packed.ctypes.data, packed.size,
                                        offsets.ctypes.data, err, 256)
    assert rc == 0, err.value
    return devsys, packed, offsets, keep


def _host_eval(L, setup, R, Qall, ipes, grad=True):
    devsys, packed, offsets, _ = setup
    n, npairs = R.shape
    nv = 6 if npairs == 3 else 9
    V, dVdR, dVdQ = np.zeros(n), np.zeros((n, npairs)), np.zeros((n, nv))
    R = np.ascontiguousarray(R, np.float64)
    Q = np.ascontiguousarray(Qall, np.float64)
    ip = np.ascontiguousarray(ipes, np.int32)
    assert L.pes_host_eval(devsys, packed.ctypes.data, offsets.ctypes.data, n, ip.ctypes.data, R.ctypes.data,
                           Q.ctypes.data, V.ctypes.data, dVdR.ctypes.data, dVdQ.ctypes.data, int(grad)) == 0
    return V, dVdR, dVdQ


CASES = {
    "O3": (lambda: systems.o3_config(), 110),
    "N3": (lambda: systems.n3_config(), 110),
    "O3NN": (lambda: systems.o3nn_config(), 110),
    "O3_9": (lambda: systems.o3_mix_config(), 110),
    "O3BNN": (lambda: systems.o3bnn_config(samples=[1, 17, 33, 50]), 110),
    "O4": (lambda: systems.o4_config(), 630),
    "N4": (lambda: systems.n4_config(), 488),
}


def _points(o, natoms, n, seed):
    rng = np.random.default_rng(seed)
    out = []
    while sum(len(x) for x in out) < n:
        Q = rng.uniform(-3.0 if natoms == 3 else -3.5, 3.0 if natoms == 3 else 3.5, size=(4 * n, 3 * (natoms - 1)))
        R, Qall = o.rp(Q)
        keep = np.all((R > 1.5) & (R < 9.0), axis=1)
        out.append(Qall[keep])
    Qall = np.concatenate(out)[:n]
    return o.rp(Qall[:, :3 * (natoms - 1)])


@pytest.mark.parametrize("name", list(CASES))
def test_device_surface_code_on_the_host_matches_the_oracle(gpu_lib, oracle_lib, name):
    from oracle import Oracle
    make, depth = CASES[name]
    cfg = make()
    o = Oracle(cfg)
    L = _harness()
    setup = _setup(gpu_lib, cfg, o.tpq)
    R, Qall = _points(o, cfg.natoms, 96 if cfg.natoms == 3 else 48, 7)
    ipes = np.arange(len(R), dtype=np.int32) % len(cfg.surfaces)
    V, g, m = _host_eval(L, setup, R, Qall, ipes)
    Vo, go, mo = o.compute(R, Qall, ipes=ipes)
    cs = o.condition_scale(R, ipes=ipes)
    vs = np.maximum(np.abs(Vo), 0.1)
    gs = np.maximum(np.abs(go).max(axis=1, keepdims=True), 1e-2)
    bound_u = 2 * depth * U
    assert np.all(np.abs(V - Vo) <= np.maximum(1e-12 * vs, bound_u * cs[:, 0])), name
    assert np.all(np.abs(g - go) <= np.maximum(1e-12 * gs, bound_u * cs[:, 1:])), name
    ms = np.maximum(np.abs(mo).max(axis=1, keepdims=True), 1e-2)
    assert np.all(np.abs(m - mo) <= np.maximum(1e-12 * ms, bound_u * cs[:, 1:].max(axis=1, keepdims=True))), name
    Ve, _, _ = _host_eval(L, setup, R, Qall, ipes, grad=False)
    Vp = o.potential(R, ipes=ipes)
    assert np.all(np.abs(Ve - Vp) <= np.maximum(1e-12 * np.maximum(np.abs(Vp), 0.1), bound_u * cs[:, 0])), name


def test_layouts_agree(gpu_lib):
    lib = C.CDLL(gpu_lib)
    lib.cair_internal_devsys_size.restype = C.c_int64
    assert _harness().pes_host_devsys_size() == lib.cair_internal_devsys_size()


@pytest.mark.parametrize("name", ["O3", "N3", "O3NN", "O3BNN"])
def test_device_bs_attempts_on_the_host_match_the_oracle(gpu_lib, oracle_lib, name):
    from oracle import Oracle
    from test_gpu_parity import CFGS, LEVELS, _non_chaotic
    cfg = CFGS[name]()
    o = Oracle(cfg)
    L = _harness()
    devsys, packed, offsets, _ = _setup(gpu_lib, cfg, o.tpq)
    mol, v0, j0 = LEVELS[name]
    lv = systems.load_levels(mol)
    ic = o.sample_ics(24, lv[(lv["vqn"] == v0) & (lv["jqn"] == j0)])
    ok, a_o = _non_chaotic(o, ic, 1000)
    assert ok.sum() >= 4
    paq = np.ascontiguousarray(ic["paq"], np.float64).copy()
    n = len(paq)
    t, dt = np.zeros(n), np.full(n, cfg.dt0)
    erra = np.ascontiguousarray(ic["erra"], np.float64)
    ip = np.zeros(n, np.int32)
    assert L.pes_host_bs_steps(devsys, packed.ctypes.data, offsets.ctypes.data, n, ip.ctypes.data, paq.ctypes.data,
                               t.ctypes.data, dt.ctypes.data, erra.ctypes.data, 1000) == 0
    rel = np.abs(paq - a_o).max(axis=1) / np.abs(a_o).max(axis=1)
    assert np.all(rel[ok] < 1e-9), rel[ok]


def _ic_host(L, setup, table, items):
    devsys, packed, offsets, _ = setup
    ntot = int(items["ntraj"].sum())
    natoms = 3 if np.frombuffer(bytes(devsys)[:4], np.int32)[0] == 3 else 4
    ne = 12 if natoms == 3 else 18
    out = {k: np.zeros((ntot, ne)) for k in ("paq", "paq0", "erra")}
    out["H0"], out["b"], out["ipes"] = np.zeros(ntot), np.zeros(ntot), np.zeros(ntot, np.int32)
    tb = np.ascontiguousarray(table, dtype=_lib.LEVEL_DTYPE)
    it = np.ascontiguousarray(items, dtype=_lib.ITEM_DTYPE)
    assert L.ic_host_sample(devsys, packed.ctypes.data, offsets.ctypes.data, tb.ctypes.data, len(it), it.ctypes.data,
                            ntot, out["paq"].ctypes.data, out["paq0"].ctypes.data, out["erra"].ctypes.data,
                            out["H0"].ctypes.data, out["b"].ctypes.data, out["ipes"].ctypes.data) == 0
    return out


def _levels_for_oracle(rows):
    out = np.zeros(len(rows), dtype=[(c, "f8") for c in ("vqn", "jqn", "eint", "egam", "rmin", "rmax", "vmin", "vmax",
                                                          "tau", "ri", "ro", "rlim")])
    for c in out.dtype.names:
        out[c] = rows[c] if c in rows.dtype.names else 0.0
    return out


def _close(a, b, rtol):
    sc = np.abs(b).max(axis=1, keepdims=True)
    return np.all(np.abs(a - b) <= rtol * sc)


@pytest.mark.parametrize("strata", ["Circles", "Rings", "Segments"])
def test_ic_kernels_on_the_host_for_rings(gpu_lib, oracle_lib, strata):
    from oracle import Oracle
    cfg = systems.n3_config(rmax=30.0)
    o = Oracle(cfg)
    L = _harness()
    setup = _setup(gpu_lib, cfg, o.tpq)
    rows = systems.load_levels("N2")[[17]]
    bring, ntring, n, seed = [-2.0, -4.5, 3.0, -7.0], [1, 2, 1, 3], 71, api.process_seed(4, 1)
    items = api.work_items(api.ring_entries(0, 0, n, seed, 10000.0, 15.0, bring, ntring, strata))
    ic = _ic_host(L, setup, api.level_table(rows), items)
    ref = o.sample_ics(n, _levels_for_oracle(rows), seed=seed, ttra=10000.0, dinit=15.0,
                       rings=(bring, ntring, api.STRATA[strata]))
    for key in ("paq", "paq0", "erra"):
        assert _close(ic[key], ref[key], 1e-10), key
    assert np.all(np.abs(ic["H0"] - ref["H0"]) <= 1e-11 * np.maximum(np.abs(ref["H0"]), 0.1))
    assert np.allclose(ic["b"], ref["b"], rtol=1e-14, atol=0) and np.all(ic["b"][31:41] == 3.0)


def test_ic_kernels_on_the_host_for_diatom_diatom_rings(gpu_lib, oracle_lib):
    from oracle import Oracle
    cfg = systems.o4_config()
    o = Oracle(cfg)
    L = _harness()
    setup = _setup(gpu_lib, cfg, o.tpq)
    rows = systems.load_levels("O2")[[0, 40]]
    n, seed = 30, api.process_seed(2, 1)
    items = api.work_items(api.ring_entries(0, 1, n, seed, 1e4, 18.0, [-3.0, -8.0], [1, 2], strata="Rings",
                                            ilevel2=1))
    ic = _ic_host(L, setup, api.level_table(rows), items)
    lv = _levels_for_oracle(rows)
    ref = o.sample_ics4(n, lv[0], lv[1], ttra=1e4, dinit=18.0, seed=seed, rings=([-3.0, -8.0], [1, 2], 1))
    for key in ("paq", "paq0", "erra"):
        assert _close(ic[key], ref[key], 1e-10), key
    assert np.allclose(ic["b"], ref["b"], rtol=1e-14, atol=0)


def _queue_host(L, setup, cfg, table, items, max_attempts):
    devsys, packed, offsets, _ = setup
    tb = np.ascontiguousarray(table, dtype=_lib.LEVEL_DTYPE)
    it = np.ascontiguousarray(items, dtype=_lib.ITEM_DTYPE)
    ntot = int(it["ntraj"].sum())
    out = np.zeros(ntot, dtype=_lib.RESULT_DTYPE)
    assert L.queue_host_run(devsys, packed.ctypes.data, offsets.ctypes.data, tb.ctypes.data, len(it), it.ctypes.data,
                            ntot, int(max_attempts), cfg.nquad, cfg.rsmal, cfg.rcent, cfg.rfact, cfg.tthresau,
                            out.ctypes.data) == 0
    return out


def test_queue_pipeline_on_the_host_for_rings(gpu_lib, oracle_lib):
    """The GPU rings test's queue half through the host pipeline: rows numbered along the stream, each
    ring's |b| as bmax, the impact parameters of the oracle's stream, the fixed ring's b."""
    from oracle import Oracle
    cfg = systems.n3_config(rmax=30.0)
    o = Oracle(cfg)
    L = _harness()
    setup = _setup(gpu_lib, cfg, o.tpq)
    rows = systems.load_levels("N2")[[17]]
    bring, ntring, n, seed = [-2.0, -4.5, 3.0, -7.0], [1, 2, 1, 3], 71, api.process_seed(4, 1)
    for strata in ("Circles", "Rings", "Segments"):
        items = api.work_items(api.ring_entries(0, 0, n, seed, 10000.0, 15.0, bring, ntring, strata))
        res = _queue_host(L, setup, cfg, api.level_table(rows), items, 2000)
        ref = o.sample_ics(n, _levels_for_oracle(rows), seed=seed, ttra=10000.0, dinit=15.0,
                           rings=(bring, ntring, api.STRATA[strata]))
        assert list(res["idx"]) == list(range(1, n + 1))
        assert np.array_equal(res["bmax"], np.repeat([2.0, 4.5, 3.0, 7.0], [11, 20, 10, 30]))
        # the row's b is the analysed impact parameter of the initial point (TrajIni%b), a magnitude;
        # Segments strata after a sampled ring draw negative b
        assert np.allclose(res["b"], np.abs(ref["b"]), rtol=1e-13, atol=0), strata
        assert np.allclose(res["b"][31:41], 3.0, rtol=1e-13, atol=0)
        if strata == "Segments":
            assert np.any(ref["b"] < 0)
        assert set(np.unique(res["status"])) <= {0, 1}


def test_queue_pipeline_on_the_host_for_the_bnn_samples(gpu_lib, oracle_lib):
    """The GPU BNN queue test through the host pipeline: 100 trajectories in 50 per-sample blocks, capped
    at 20,000 attempts; final states against the oracle where both finished and the oracle is stable,
    then the finished rows of all 50 samples pooled into one run by the statistics kernels."""
    import oracle
    from oracle import Oracle
    from test_stats_host import _kernels_on_host
    cfg = systems.o3bnn_config()
    o = Oracle(cfg)
    L = _harness()
    setup = _setup(gpu_lib, cfg, o.tpq)
    lv = systems.load_levels("O2")
    row = lv[(lv["vqn"] == 0) & (lv["jqn"] == 1)]
    counts = api.degeneracy_blocks(100, cfg.degeneracy)
    seed, cap = api.process_seed(3, 1), 20000
    items = api.work_items([(0, k, nn, seed, 20000.0, 6.0, 15.0) for k, nn in enumerate(counts)])
    res = _queue_host(L, setup, cfg, api.level_table(row), items, cap)
    ic = o.sample_ics(2, _levels_for_oracle(row), seed=seed, ttra=20000.0, bmax=6.0, dinit=15.0)
    paq, erra = np.tile(ic["paq"], (50, 1)), np.tile(ic["erra"], (50, 1))
    ipv = np.repeat(np.arange(50, dtype=np.int32), 2)
    a = o.integrate(paq, erra, ipes=ipv, max_attempts=cap, procs=4)
    b = o.integrate(paq * (1 + 1e-14), erra, ipes=ipv, max_attempts=cap, procs=4)

    def qn(paqs):
        fs = o.analyze(o.apply_transformation(paqs))
        return api.histogram_assign(np.array([f["angmom"] for f in fs]), np.array([f["viba"] for f in fs]),
                                    np.array([16 * f["ipair"] + f["itype"] + 0.5 for f in fs]))

    fa, fb = qn(a["paq"]), qn(b["paq"])
    fg = api.histogram_assign(res["j_f"], res["v_f"], res["arr_f"])
    done = (res["status"] == 0) & (a["status"] == 0) & (b["status"] == 0)
    same = (fa[0] == fg[0]) & (fa[1] == fg[1]) & (fa[2] == fg[2])
    stable = done & (fa[0] == fb[0]) & (fa[1] == fb[1]) & (fa[2] == fb[2])
    assert stable.sum() >= 20 and same[stable].mean() >= 0.995
    st = api.Statistics.__new__(api.Statistics)
    P = _lib.StatsParams()
    P.qn_max, P.ncond = 300, 3
    for i in range(5):
        P.iskip[i], P.pres_even_odd[i] = (1 if i < 3 else 0), 0
    m = cfg.masses
    P.ham_abs_tol, P.xmu = 1.0e6, (m[0] + m[1]) * m[2] / sum(m)
    got = _kernels_on_host(P, items, res, [0] * 50)
    ok = res["status"] == 0
    ref, _ = oracle.statistics(res["bmax"][ok], res["b"][ok], np.stack([res["j_i"], res["v_i"], res["arr_i"]], 1)[ok],
                               np.stack([res["j_f"], res["v_f"], res["arr_f"]], 1)[ok], cap=200)
    gd = {tuple(int(x) for x in r["fin"][:3]): r for r in got}
    assert len(got) == len(ref)
    for fs, nn, cross, sd in ref:
        assert gd[fs]["count"] == nn and gd[fs]["cross"] == pytest.approx(cross, rel=1e-14)


def test_queue_pipeline_on_the_host_for_n2_n(gpu_lib, oracle_lib):
    """N2 + N on N3 UMN through the host pipeline against the oracle path, with the GPU queue test's
    criterion: final (J, v, arrangement) equal on >= 99.5 % of the trajectories whose oracle outcome is
    stable under a 1e-14 perturbation, initial states equal everywhere."""
    from oracle import Oracle
    cfg = systems.n3_config()
    o = Oracle(cfg)
    L = _harness()
    setup = _setup(gpu_lib, cfg, o.tpq)
    lv = systems.load_levels("N2")
    rows = lv[[3, 60]]
    entries = [(0, 0, 40, api.process_seed(2, 1), 10000.0, 7.0, 15.0), (1, 0, 40, api.process_seed(2, 2), 20000.0, 7.0,
                                                                           15.0)]
    items = api.work_items(entries)
    res = _queue_host(L, setup, cfg, api.level_table(rows), items, cfg.max_attempts)
    assert np.all(res["status"] == 0) and np.max(np.abs(res["dH"])) < cfg.ham_abs_tol
    same, stable = [], []
    for i, (il, _, nt, seed, T, bmax, dinit) in enumerate(entries):
        ic = o.sample_ics(nt, _levels_for_oracle(rows[il:il + 1]), seed=seed, ttra=T, bmax=bmax, dinit=dinit)
        a = o.integrate(ic["paq"], ic["erra"], procs=4)
        b = o.integrate(ic["paq"] * (1 + 1e-14), ic["erra"], procs=4)

        def qn(points):   # points: velocities and coordinates
            fs = o.analyze(points)
            return api.histogram_assign(np.array([f["angmom"] for f in fs]), np.array([f["viba"] for f in fs]),
                                        np.array([16 * f["ipair"] + f["itype"] + 0.5 for f in fs]))

        fa, fb = qn(o.apply_transformation(a["paq"])), qn(o.apply_transformation(b["paq"]))
        r = res[res["item"] == i]
        fg = api.histogram_assign(r["j_f"], r["v_f"], r["arr_f"])
        gi = api.histogram_assign(r["j_i"], r["v_i"], r["arr_i"])
        oi = qn(ic["paq0"])
        assert all(np.array_equal(x, y) for x, y in zip(gi, oi))
        same.append((fa[0] == fg[0]) & (fa[1] == fg[1]) & (fa[2] == fg[2]))
        stable.append((fa[0] == fb[0]) & (fa[1] == fb[1]) & (fa[2] == fb[2]))
    same, stable = np.concatenate(same), np.concatenate(stable)
    assert stable.mean() >= 0.9 and same[stable].mean() >= 0.995


def test_table_driven_exponential_within_one_ulp():
    """fexp (Tang's table-driven method, degree-5 polynomial) against the C library's exp: at most one
    ulp apart over the surfaces' arguments and the whole range it serves, [-707, 707)."""
    L = _harness()
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-60.0, 5.0, 400000), rng.uniform(-707.0, 707.0, 200000),
                        np.linspace(-1e-3, 1e-3, 20001), rng.uniform(-0.01, 0.01, 50000)])
    y = np.zeros_like(x)
    L.host_fexp(len(x), x.ctypes.data, y.ctypes.data)
    ref = np.exp(x)
    ulp = np.spacing(ref)
    err = np.abs(y - ref) / ulp
    print("fexp vs libm exp: max %.3f ulp, mean %.4f ulp, %.5f exact" % (err.max(), err.mean(), np.mean(err == 0)))
    assert err.max() <= 1.0


@pytest.mark.parametrize("below", [0, 1])
def test_thread_integrator_hands_its_tail_off(gpu_lib, oracle_lib, below):
    """The thread integrator's tail hand-off, run on the host (one lane, four N2 + N trajectories).  With the
    hand-off off every trajectory ends normally.  With it on at one trajectory in flight, the last trajectory
    (the one in flight once the queue is empty) is written back at its first end check: listed once, its
    attempts recorded (ncall), its status left to the warp integrator, and its state, time, step and counts
    exactly those of ncall attempts of the same Bulirsch-Stoer code from its initial conditions."""
    from oracle import Oracle
    cfg = systems.n3_config()
    o = Oracle(cfg)
    L = _harness()
    devsys, packed, offsets, _ = _setup(gpu_lib, cfg, o.tpq)
    lv = systems.load_levels("N2")
    ic = o.sample_ics(4, lv[(lv["vqn"] == 0) & (lv["jqn"] == 10)], seed=17)
    n = 4
    paq = np.ascontiguousarray(ic["paq"], np.float64).copy()
    erra = np.ascontiguousarray(ic["erra"], np.float64)
    t, dt, H = np.zeros(n), np.zeros(n), np.zeros(n)
    irej, iste, status = np.zeros(n, np.int32), np.zeros(n, np.int32), np.full(n, -7, np.int32)
    hand, hand_att, hctl = np.full(n, -1, np.int32), np.zeros(n, np.int64), np.zeros(3, np.uint64)
    assert L.handoff_host_run(devsys, packed.ctypes.data, offsets.ctypes.data, n, paq.ctypes.data, erra.ctypes.data,
                              10 ** 6, below, t.ctypes.data, dt.ctypes.data, H.ctypes.data, irej.ctypes.data,
                              iste.ctypes.data, status.ctypes.data, hand.ctypes.data, hand_att.ctypes.data,
                              hctl.ctypes.data) == 0
    if below == 0:
        assert int(hctl[1]) == 0 and np.all(status == 0)
        return
    assert int(hctl[1]) == 1 and hand[0] == n - 1
    assert np.all(status[:n - 1] == 0) and status[n - 1] == -7
    assert hand_att[n - 1] == cfg.ncall and iste[n - 1] + irej[n - 1] == cfg.ncall
    assert int(hctl[0]) == 1                      # taken four, finished three
    # the same ncall attempts through the fixed-attempt host code
    y = np.ascontiguousarray(ic["paq"][n - 1:n], np.float64).copy()
    e = np.ascontiguousarray(ic["erra"][n - 1:n], np.float64)
    t1, dt1 = np.zeros(1), np.full(1, cfg.dt0)
    ip = np.zeros(1, np.int32)
    assert L.pes_host_bs_steps(devsys, packed.ctypes.data, offsets.ctypes.data, 1, ip.ctypes.data, y.ctypes.data,
                               t1.ctypes.data, dt1.ctypes.data, e.ctypes.data, cfg.ncall) == 0
    assert np.array_equal(paq[n - 1], y[0]) and t[n - 1] == t1[0] and dt[n - 1] == dt1[0]
    h_o, _ = o.hamiltonian(paq[n - 1:n])
    assert abs(H[n - 1] - h_o[0]) < 1e-12 * max(abs(h_o[0]), 0.1)
