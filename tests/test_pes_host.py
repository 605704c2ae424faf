"""The library's device surface and integrator code on the CPU: coarseair_gb300/csrc/cair_device.cuh compiled unchanged
by the host compiler (tests/host_pes/pes_host.cpp, CUDA qualifiers defined away), with the DevSys and
the packed coefficients from the library's own setup (cair_internal_setup_system, the part of
cair_create that needs no GPU).  Every surface model -- O3, N3, O4, N4 UMN, the nine-surface O3 mix,
O3 NN and the O3 BNN samples -- against the oracle at the same points, energies and gradients to
1e-12 relative or the rounding-level bound of the GPU parity tests, and the energy-only path against
the oracle's Potential; and the device Bulirsch-Stoer attempt (Rhs, bs_attempt) over 1000 fixed attempts
against the oracle on the trajectories the oracle shows to be non-chaotic, to 1e-9 as on the GPU.
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
    src += [os.path.join(csrc, "cair_device.cuh")]
    src += [os.path.join(csrc, "generated", f) for f in os.listdir(os.path.join(csrc, "generated"))]
    if not os.path.exists(HARNESS) or os.path.getmtime(HARNESS) < max(os.path.getmtime(f) for f in src):
        subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", "-shared", "-I", os.path.join(ROOT, "include"),
                        "-o", HARNESS, src[0]], check=True)
    L = C.CDLL(HARNESS)
    L.pes_host_devsys_size.restype = C.c_int64
    L.pes_host_eval.restype = C.c_int
    L.pes_host_eval.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
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
