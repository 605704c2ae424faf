"""CPU pins of the surrogate's oracle (oracle/oracle_mlp.py): its feature Jacobian and damping
derivative against finite differences, its value/input-gradient/loss-gradient algebra against
torch autograd (float64, double backpropagation through the input gradient), and the host copy
of the feature map in the package against the oracle's."""
import numpy as np
import pytest

import oracle_mlp as om

CONSTS = dict(mu=np.linspace(0.1, 0.5, 10), isd=np.linspace(2.0, 0.7, 10), fmin=-np.ones(10) * 50,
              fmax=np.ones(10) * 50, sigma_d=2e-3)


def _geoms(n, seed=3):
    rng = np.random.default_rng(seed)
    r1 = rng.uniform(1.7, 3.0, n)
    r2 = rng.uniform(2.0, 6.0, n)
    r3 = np.abs(r1 - r2) + rng.uniform(0.3, 1.0, n) * (r1 + r2 - np.abs(r1 - r2))
    return np.stack([r1, r2, r3], 1)


def test_feature_jacobian_and_damping_against_finite_differences():
    R = _geoms(40)
    f, J, D, dD, _ = om.features(R, CONSTS)
    h = 1e-6
    for k in range(3):
        Rp, Rm = R.copy(), R.copy()
        Rp[:, k] += h
        Rm[:, k] -= h
        fp, _, Dp, _, _ = om.features(Rp, CONSTS)
        fm, _, Dm, _, _ = om.features(Rm, CONSTS)
        fd = (fp - fm)[:, :10] / (2 * h)
        assert np.allclose(J[:, :, k], fd, rtol=1e-6, atol=1e-8 * np.abs(fd).max())
        assert np.allclose(dD[:, k], (Dp - Dm) / (2 * h), rtol=1e-6, atol=1e-10)
    assert np.all(f[:, 15] == 1.0) and np.all(f[:, 10:15] == 0.0)


def test_features_are_permutation_invariant_and_damping_vanishes_asymptotically():
    R = _geoms(20)
    f0 = om.features(R, CONSTS)[0]
    for perm in ([1, 0, 2], [2, 1, 0], [0, 2, 1], [1, 2, 0]):
        assert np.allclose(om.features(R[:, perm], CONSTS)[0], f0, rtol=1e-13, atol=1e-13)
    far = np.array([[2.07, 16.0, 18.07], [2.07, 30.0, 32.07]])
    _, _, D, dD, _ = om.features(far, CONSTS)
    assert np.all(D < 1e-12) and np.all(np.abs(dD) < 1e-10)


def test_oracle_gradients_against_autograd():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    p = om.init_params(7)
    p[om.P_B2:om.P_B4] += rng.normal(0, 0.1, om.P_B4 - om.P_B2)
    p[om.P_B4] = 0.3
    R = _geoms(37)
    e = rng.normal(0, 1, 37)
    gt = rng.normal(0, 1, (37, 3))
    le, lf, grad = om.loss_and_grad(p, R, e, gt, CONSTS, 1.0, 0.5, rounding="exact")
    q = om.unpack(p)
    T = lambda a: torch.tensor(np.asarray(a, dtype=np.float64), requires_grad=True)
    W1, W2, W3 = T(om.bf16(q["W1"])), T(om.bf16(q["W2"])), T(om.bf16(q["W3"]))
    b2, b3, w4, b4 = T(q["b2"]), T(q["b3"]), T(q["w4"]), T(np.array(q["b4"]))
    f, J, D, dD, _ = om.features(R, CONSTS)
    ft = torch.tensor(f, requires_grad=True)
    h1 = torch.tanh(ft @ W1.T)
    h2 = torch.tanh(h1 @ W2.T + b2)
    h3 = torch.tanh(h2 @ W3.T + b3)
    y = h3 @ w4 + b4
    (g,) = torch.autograd.grad(y.sum(), ft, create_graph=True)
    Dt, dDt, Jt = torch.tensor(D), torch.tensor(dD), torch.tensor(J)
    gpred = y[:, None] * dDt + Dt[:, None] * torch.einsum("ni,nik->nk", g[:, :10], Jt)
    n = len(e)
    L_e = (1.0 / n) * ((Dt * y - torch.tensor(e)) ** 2).sum()
    L_f = (0.5 / n) * ((gpred - torch.tensor(gt)) ** 2).sum()
    (L_e + L_f).backward()
    assert le == pytest.approx(L_e.item(), rel=1e-12)
    assert lf == pytest.approx(L_f.item(), rel=1e-12)
    ref = om.pack(dict(W1=W1.grad.numpy(), W2=W2.grad.numpy(), W3=W3.grad.numpy(), b2=b2.grad.numpy(),
                       b3=b3.grad.numpy(), w4=w4.grad.numpy(), b4=b4.grad.item()))
    assert np.allclose(grad, ref, rtol=1e-10, atol=1e-12 * np.abs(ref).max())
    # value and input gradient of forward()
    yv, gv = om.forward(p, f)
    assert np.allclose(yv, y.detach().numpy(), rtol=1e-13, atol=1e-13)
    assert np.allclose(gv, g.detach().numpy(), rtol=1e-12, atol=1e-13)


def test_package_feature_map_matches_the_oracle():
    from coarseair_gb300 import surrogate
    R = _geoms(50)
    assert np.allclose(surrogate.raw_features_np(R), om.raw_features(R)[0], rtol=1e-15, atol=0)
    assert surrogate.init_params(3).size == om.NPARAM


def test_bf16_rounding_is_round_to_nearest_even():
    assert om.bf16(1.0) == 1.0
    assert om.bf16(1.0 + 2.0 ** -8) == 1.0               # tie to even
    assert om.bf16(1.0 + 3 * 2.0 ** -8) == 1.0 + 2.0 ** -6  # tie to even, upward
    assert om.bf16(1.0 + 2.0 ** -8 + 2.0 ** -12) == 1.0 + 2.0 ** -7
