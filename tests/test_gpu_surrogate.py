"""GPU tests of the learned surrogate's tensor-core kernels against the CPU oracle
(oracle/oracle_mlp.py): the operand conventions of one tcgen05.mma, the batched evaluation
(both members' values, the input gradient, V3 and dV3/dR), and the training step's loss and
parameter gradient, and one Adam step."""
import ctypes as C

import numpy as np
import pytest

import oracle_mlp as om
from coarseair_gb300 import _lib, surrogate

pytestmark = pytest.mark.gpu


def _probe(lib, A, B, N, b_mn, a_lbo, a_sbo, b_lbo, b_sbo):
    fn = lib.cair_internal_tc_probe
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                   C.POINTER(C.c_float)]
    D = np.zeros((128, N), dtype=np.float32)
    rc = fn(A.ctypes.data, B.ctypes.data, N, b_mn, a_lbo, a_sbo, b_lbo, b_sbo, D.ctypes.data_as(C.POINTER(C.c_float)))
    return rc, D


def _bf16_bits(a):
    b = np.asarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    return (((b + 0x7FFF + ((b >> 16) & 1)) >> 16) & 0xFFFF).astype(np.uint16)


def test_tcgen05_operand_layouts(gpu_lib):
    """D = A B^T through one 128 x N x 16 tcgen05.mma: K-major A and B (N = 128, 16) and MN-major B,
    with the descriptor offsets the kernels use; the swapped offsets must not match (so the test
    sees which field is which)."""
    lib = _lib.load()
    rng = np.random.default_rng(1)
    A = rng.uniform(-1, 1, (128, 16))
    Ab = _bf16_bits(A)
    Af = om.bf16(A)
    found = {}
    for N in (128, 16):
        B = rng.uniform(-1, 1, (N, 16))
        Bb, Bf = _bf16_bits(B), om.bf16(B)
        ref = Af @ Bf.T
        for b_mn, kstride_b, nstride_b in ((0, N * 16, 128), (1, 128, 256)):
            for a_swap in (0, 1):
                for b_swap in (0, 1):
                    a_lbo, a_sbo = (2048, 128) if not a_swap else (128, 2048)
                    b_lbo, b_sbo = (kstride_b, nstride_b) if not b_swap else (nstride_b, kstride_b)
                    rc, D = _probe(lib, Ab, Bb, N, b_mn, a_lbo, a_sbo, b_lbo, b_sbo)
                    assert rc == 0
                    ok = np.allclose(D, ref, rtol=1e-6, atol=1e-6)
                    found[(N, b_mn, a_swap, b_swap)] = ok
    print("layout probe:", {k: v for k, v in found.items() if v})
    # K-major: leading-dimension offset = the K step, stride-dimension offset = the M/N step
    assert found[(128, 0, 0, 0)] and found[(16, 0, 0, 0)]
    assert not found[(128, 0, 1, 0)] and not found[(128, 0, 0, 1)]
    # MN-major B: the kernels' convention (cair_sur.cuh MN_LBO / MN_SBO: leading-dimension offset =
    # the K step, as for K-major) holds for N = 128 and 16, and the swapped one does not
    mn_ok = [s for s in (0, 1) if found[(128, 1, 0, s)] and found[(16, 1, 0, s)]]
    print("MN-major offsets (lbo, sbo) =", "(K step, N step)" if mn_ok == [0] else "(N step, K step)"
          if mn_ok == [1] else "neither")
    assert mn_ok == [0], "MN-major convention differs from cair_sur.cuh"


CONSTS = dict(mu=np.array([1.0, 0.7, 0.25, 0.6, 0.3, 0.02, 0.5, 0.2, 0.05, 0.03]),
              isd=np.array([1.2, 1.5, 3.0, 1.5, 2.5, 20.0, 1.5, 3.0, 8.0, 15.0]),
              fmin=-np.full(10, 1e3), fmax=np.full(10, 1e3), sigma_d=2e-3)


def _geoms(n, seed=3):
    rng = np.random.default_rng(seed)
    r1 = rng.uniform(1.7, 3.0, n)
    r2 = rng.uniform(2.0, 7.0, n)
    r3 = np.abs(r1 - r2) + rng.uniform(0.3, 1.0, n) * (r1 + r2 - np.abs(r1 - r2))
    return np.stack([r1, r2, r3], 1)


def _params(seed):
    rng = np.random.default_rng(seed)
    p = om.init_params(seed)
    p[om.P_B2:om.P_B4] += rng.normal(0, 0.2, om.P_B4 - om.P_B2)
    p[om.P_B4] = 0.4
    return p


def _surrogate():
    s = surrogate.Surrogate()
    s.set_consts(CONSTS["mu"], CONSTS["isd"], CONSTS["fmin"], CONSTS["fmax"], sigma_d=CONSTS["sigma_d"])
    return s


def test_surrogate_evaluation_matches_oracle(gpu_lib):
    """Both members' values, member A's input gradient and V3, dV3/dR at 1000 geometries (not a
    multiple of the 128-row tile) against the float64 oracle with the same BF16 weights: the
    three-part operands make the tensor-core products FP32-accurate, so the agreement is at FP32
    accumulation level (relative 2e-5 of each quantity's scale)."""
    s = _surrogate()
    pa, pb = _params(1), _params(2)
    s.set_params(0, pa)
    s.set_params(1, pb)
    R = _geoms(1000)
    ya, yb, g, v3, dv3 = s.eval(R)
    f, J, D, dD, _ = om.features(R, CONSTS)
    # the device computes features in FP32: compare through the oracle at its own features
    ya_o, g_o = om.forward(pa.astype(np.float64), f)
    yb_o, _ = om.forward(pb.astype(np.float64), f)
    v3_o, dv3_o = om.v3(pa.astype(np.float64), R, CONSTS)
    sc = lambda a: np.abs(a).max()
    err = dict(ya=sc(ya - ya_o) / sc(ya_o), yb=sc(yb - yb_o) / sc(yb_o), g=sc(g - g_o) / sc(g_o),
               v3=sc(v3 - v3_o) / sc(v3_o), dv3=sc(dv3 - dv3_o) / sc(dv3_o))
    print("evaluation vs oracle (max error / scale):", {k: "%.2e" % v for k, v in err.items()})
    assert all(v < 2e-5 for v in err.values()), err
    s.close()


def test_surrogate_training_gradient_matches_oracle(gpu_lib):
    """One training gradient over 300 samples (three tiles, the last partial): the loss parts and
    every parameter block's gradient against the oracle with the device's BF16 rounding points
    (relative error of each block's norm below 2e-3), and one Adam step against numpy."""
    torch = pytest.importorskip("torch")
    s = _surrogate()
    p = _params(3)
    s.set_params(0, p)
    rng = np.random.default_rng(9)
    n = 300
    R = _geoms(n, seed=4)
    smp = np.zeros(n, dtype=_lib.SUR_SAMPLE_DTYPE)
    smp["R"] = R
    smp["e"] = rng.normal(0, 1, n)
    smp["g"] = rng.normal(0, 1, (n, 3))
    dev = torch.device("cuda", 0)
    d_smp = torch.from_numpy(smp.view(np.uint8).copy()).to(dev)
    idx = torch.arange(n, dtype=torch.int64, device=dev)
    w_e, w_f = 1.0, 0.5
    s.grad_step(0, d_smp, idx, w_e, w_f)
    loss = s.take_loss()
    grad = s.grad(0).astype(np.float64)
    le, lf, g_o = om.loss_and_grad(p.astype(np.float64), R, smp["e"].astype(np.float64),
                                   smp["g"].astype(np.float64), CONSTS, w_e, w_f, rounding="device")
    assert loss[0] == pytest.approx(le, rel=1e-4)
    assert loss[1] == pytest.approx(lf, rel=1e-4)
    blocks = dict(W1=(om.P_W1, om.P_W2), W2=(om.P_W2, om.P_W3), W3=(om.P_W3, om.P_B2), b2=(om.P_B2, om.P_B3),
                  b3=(om.P_B3, om.P_W4), w4=(om.P_W4, om.P_B4), b4=(om.P_B4, om.P_B4 + 1))
    rel = {k: np.linalg.norm(grad[a:b] - g_o[a:b]) / np.linalg.norm(g_o[a:b]) for k, (a, b) in blocks.items()}
    _, _, g_x = om.loss_and_grad(p.astype(np.float64), R, smp["e"].astype(np.float64), smp["g"].astype(np.float64),
                                 CONSTS, w_e, w_f, rounding="exact")
    rel_x = {k: np.linalg.norm(grad[a:b] - g_x[a:b]) / np.linalg.norm(g_x[a:b]) for k, (a, b) in blocks.items()}
    print("gradient vs oracle (device rounding):", {k: "%.1e" % v for k, v in rel.items()})
    print("gradient vs exact float64:", {k: "%.1e" % v for k, v in rel_x.items()})
    assert all(v < 2e-3 for v in rel.values()), rel
    # one Adam step from zero moments
    lr = 1e-3
    s.adam(0, lr)
    p1 = s.params(0).astype(np.float64)
    m = 0.1 * grad
    v = 0.001 * grad * grad
    ref = p.astype(np.float32).astype(np.float64) - lr * (m / 0.1) / (np.sqrt(v / 0.001) + 1e-8)
    assert np.allclose(p1, ref, rtol=1e-5, atol=1e-7)
    assert np.all(s.grad(0) == 0.0)
    s.close()


def test_tcgen05_mma_rate(gpu_lib):
    """Back-to-back 128 x 128 x 16 BF16 MMAs into one TMEM accumulator (the operand layouts of the
    surrogate's kernels) on one SM: the steady-state cycles per MMA, against the dense BF16 rate of
    about 73 cycles per MMA (2.25 PFLOP/s over 152 SMs at 2.07 GHz)."""
    lib = _lib.load()
    fn = lib.cair_internal_tc_rate
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
    out = {}
    for n in (12, 1200, 12000):
        a, b = C.c_longlong(), C.c_longlong()
        assert fn(n, 3, C.byref(a), C.byref(b)) == 0
        out[n] = b.value / n
    print("tcgen05 128x128x16 BF16: %.1f cycles/MMA in a 12-MMA phase, %.1f (1200), %.1f (12000)" %
          (out[12], out[1200], out[12000]))
    assert out[12000] < 150
