"""The warp integrator's lane-parallel programs (generated/warp_prog.h) against the oracle, without a GPU.

The host harness (tests/host_pes/pes_host.cpp) runs the same interpreter the kernel runs
(cair_warp.cuh: constant loading, the const program, the grad and energy programs), one instruction
after the other.  An instruction's result does not depend on the lane that executes it, so this is
the device arithmetic, contractions included (the programs' fused multiply-adds are explicit).  The
criterion is the GPU right-hand-side parity criterion: 1e-12 of the row's largest component, or the
rounding-level bound of the surface evaluated on absolute values where that is larger."""
import ctypes as C

import numpy as np
import pytest

from coarseair_gb300 import systems
from test_pes_host import _harness, _setup

U = 1.1102230246251565e-16
CFGS = {"O3": systems.o3_config, "N3": systems.n3_config, "O3_9": systems.o3_mix_config,
        "O4": systems.o4_config, "N4": systems.n4_config, "O3NN": systems.o3nn_config,
        "O3BNN": lambda: systems.o3bnn_config(samples=[1, 17, 33, 50])}
LEVELS = {"O3": ("O2", 0, 1), "N3": ("N2", 0, 0), "O3_9": ("O2", 0, 1), "O3NN": ("O2", 0, 1), "O3BNN": ("O2", 0, 1)}
# depth of the surface graph in the rounding bound (as the surface parity tests take it)
DEPTH = {"O3": 110, "N3": 110, "O3_9": 110, "O4": 630, "N4": 488, "O3NN": 110, "O3BNN": 110}


def _warp_eval(L, setup, y, ipes):
    devsys, packed, offsets, _ = setup
    n = y.shape[0]
    y = np.ascontiguousarray(y, np.float64)
    npairs = 3 if y.shape[1] == 12 else 6
    yp, H, Ri = np.zeros_like(y), np.zeros(n), np.zeros((n, npairs))
    ip = np.ascontiguousarray(ipes, np.int32)
    assert L.warp_host_eval(devsys, packed.ctypes.data, offsets.ctypes.data, n, ip.ctypes.data, y.ctypes.data,
                            yp.ctypes.data, H.ctypes.data, Ri.ctypes.data) == 0
    return yp, H, Ri


def _phase_points(o, name, n, seed):
    """Diatom + atom: initial conditions of the level the tests integrate, and random geometries with
    random momenta.  Diatom + diatom: random geometries with random momenta."""
    rng = np.random.default_rng(seed)
    nv = o.nv
    if nv == 6:
        mol, v0, j0 = LEVELS[name]
        lv = systems.load_levels(mol)
        sel = lv[(lv["vqn"] == v0) & (lv["jqn"] == j0)]
        ic = o.sample_ics(n // 2, sel, seed=seed)["paq"]
        lo, hi, span = 1.5, 9.0, 3.0
    else:
        ic = np.zeros((0, 2 * nv))
        lo, hi, span = 1.6, 10.0, 3.5
    out = []
    while sum(len(x) for x in out) < n - len(ic):
        Q = rng.uniform(-span, span, size=(4 * n, nv))
        R, _ = o.rp(Q)
        out.append(Q[np.all((R > lo) & (R < hi), axis=1)])
    Q = np.concatenate(out)[:n - len(ic)]
    P = rng.normal(0.0, 10.0, size=Q.shape)
    return np.concatenate([ic, np.concatenate([P, Q], axis=1)])


@pytest.mark.parametrize("name", list(CFGS))
def test_warp_programs_match_the_oracle(gpu_lib, oracle_lib, name):
    from oracle import Oracle
    cfg = CFGS[name]()
    o = Oracle(cfg)
    L = _harness()
    setup = _setup(gpu_lib, cfg, o.tpq)
    y = _phase_points(o, name, 160, 11)
    ipes = np.arange(len(y), dtype=np.int32) % len(cfg.surfaces)
    yp, H, Ri = _warp_eval(L, setup, y, ipes)
    yp_o = o.rhs(y, ipes=ipes)
    R, _ = o.rp(y[:, o.nv:])
    ROUND_U = 2 * DEPTH[name] * U
    cs = o.condition_scale(R, ipes=ipes)
    sc = np.maximum(1e-12 * np.abs(yp_o).max(axis=1, keepdims=True), ROUND_U * cs[:, 1:].max(axis=1, keepdims=True))
    worst = (np.abs(yp - yp_o) / sc).max()
    within = np.mean(np.all(np.abs(yp - yp_o) <= 1e-12 * np.abs(yp_o).max(axis=1, keepdims=True), axis=1))
    print("%s warp RHS: worst/bound %.2e, %.4f of the points within 1e-12" % (name, worst, within))
    assert np.all(np.abs(yp - yp_o) <= sc)
    h_o, r_o = o.hamiltonian(y, ipes=ipes)
    hs = np.maximum(1e-12 * np.maximum(np.abs(h_o), 0.1), ROUND_U * cs[:, 0])
    assert np.all(np.abs(H - h_o) <= hs)
    assert np.allclose(Ri, r_o, rtol=4e-16, atol=0)


def test_warp_programs_are_generated_from_the_committed_tables():
    """The committed header is what gen_warp.py writes from the committed PIP tables."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    gen = os.path.join(root, "coarseair_gb300", "csrc", "gen", "gen_warp.py")
    hdr = os.path.join(root, "coarseair_gb300", "csrc", "generated", "warp_prog.h")
    before = open(hdr).read()
    try:
        subprocess.run([sys.executable, gen], check=True, capture_output=True)
        assert open(hdr).read() == before
    finally:
        with open(hdr, "w") as f:
            f.write(before)
