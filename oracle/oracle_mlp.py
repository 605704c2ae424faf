"""CPU oracle -- TEST INFRASTRUCTURE ONLY: the learned N3 surrogate (its features, network, value,
input gradient, energy + force loss and the loss's parameter gradient), restated in numpy float64.

The surrogate has no counterpart in the reference; its dense-layer algebra is the one of
O3_NN_PES_Class.F90:357-477 (tanh layers, analytic backward from the output to the inputs) with a
third hidden layer and an FP32 output layer.  Definitions (all in float64 here):

    x_i   = exp(-d_i - d_i^2 / 1.5),  d_i = R_i * 0.52917721092 - 1.098    (MEG variable, angstrom)
    raw   = ten S3-orbit sums of x of degree 1..4
    f     = ((raw - mu) * isd, 0 x 5, 1)
    y     = w4 . h3 + b4,  h1 = tanh(W1 f), h2 = tanh(W2 h1 + b2), h3 = tanh(W3 h2 + b3)   [eV]
    D     = 1 - exp(-(x1 x2 + x1 x3 + x2 x3) / sigma_d)
    V3_s  = D y,  grad_R V3_s = y grad_R D + D (dy/df) (df/dR)
    loss  = w_e (V3_s - e)^2 + w_f |grad_R V3_s - g|^2          (mean over the batch)

W1, W2, W3 enter as their BF16 roundings (the weights the tensor cores hold).  The parameter
gradient follows from differentiating y and the directional derivative c . dy/df, with
r = dL/dy and c = dL/d(dy/df): a forward pass, the input-gradient pass, a tangent pass along c and
one reverse pass through both.  `rounding="device"` rounds to BF16 the operands that the device
stages as one BF16 part (c, the tangent activations, the reverse adjoints and the operands of the
weight-gradient products); `"exact"` keeps them in float64.
"""
import numpy as np

NF, NINV, NH = 16, 10, 128
P_W1 = 0
P_W2 = P_W1 + NH * NF
P_W3 = P_W2 + NH * NH
P_B2 = P_W3 + NH * NH
P_B3 = P_B2 + NH
P_W4 = P_B3 + NH
P_B4 = P_W4 + NH
NPARAM = P_B4 + 1
EV_PER_EH = 27.211386245988
B_TO_ANG = 0.52917721092


def bf16(a):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    a32 = np.asarray(a, dtype=np.float32)
    b = a32.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return dict(W1=p[P_W1:P_W2].reshape(NH, NF), W2=p[P_W2:P_W3].reshape(NH, NH), W3=p[P_W3:P_B2].reshape(NH, NH),
                b2=p[P_B2:P_B3], b3=p[P_B3:P_W4], w4=p[P_W4:P_B4], b4=p[P_B4])


def pack(d):
    out = np.zeros(NPARAM)
    out[P_W1:P_W2] = d["W1"].ravel()
    out[P_W2:P_W3] = d["W2"].ravel()
    out[P_W3:P_B2] = d["W3"].ravel()
    out[P_B2:P_B3] = d["b2"]
    out[P_B3:P_W4] = d["b3"]
    out[P_W4:P_B4] = d["w4"]
    out[P_B4] = d["b4"]
    return out


def raw_features(R):
    """raw[n][10] and d raw / d R [n][10][3] at pair distances R[n][3] (bohr)."""
    R = np.asarray(R, dtype=np.float64).reshape(-1, 3)
    d = R * B_TO_ANG - 1.098
    x = np.exp(-d - d * d / 1.5)
    dx = (-1.0 - d * (2.0 / 1.5)) * x * B_TO_ANG
    s1 = x.sum(1)
    x2, x3 = x * x, x * x * x
    s2, s3 = x2.sum(1), x3.sum(1)
    p11 = x[:, 0] * x[:, 1] + x[:, 0] * x[:, 2] + x[:, 1] * x[:, 2]
    p111 = x[:, 0] * x[:, 1] * x[:, 2]
    s4 = (x2 * x2).sum(1)
    raw = np.stack([s1, s2, p11, s3, s2 * s1 - s3, p111, s4, s3 * s1 - s4,
                    x2[:, 0] * x2[:, 1] + x2[:, 0] * x2[:, 2] + x2[:, 1] * x2[:, 2], p111 * s1], 1)
    dr = np.zeros((R.shape[0], NINV, 3))
    for k in range(3):
        o = s1 - x[:, k]
        po = x[:, (k + 1) % 3] * x[:, (k + 2) % 3]
        dr[:, 0, k] = 1.0
        dr[:, 1, k] = 2 * x[:, k]
        dr[:, 2, k] = o
        dr[:, 3, k] = 3 * x2[:, k]
        dr[:, 4, k] = 2 * x[:, k] * o + (s2 - x2[:, k])
        dr[:, 5, k] = po
        dr[:, 6, k] = 4 * x3[:, k]
        dr[:, 7, k] = 3 * x2[:, k] * o + (s3 - x3[:, k])
        dr[:, 8, k] = 2 * x[:, k] * (s2 - x2[:, k])
        dr[:, 9, k] = po * s1 + p111
    dR = dr * dx[:, None, :]
    return raw, dR, x, dx, p11


def features(R, consts):
    """f[n][16], J = df/dR [n][10][3], D[n], dD/dR [n][3], in_range[n]."""
    raw, dR, x, dx, p11 = raw_features(R)
    mu, isd = np.asarray(consts["mu"], float), np.asarray(consts["isd"], float)
    f = np.zeros((raw.shape[0], NF))
    f[:, :NINV] = (raw - mu) * isd
    f[:, NF - 1] = 1.0
    J = dR * isd[None, :, None]
    sd = float(consts["sigma_d"])
    e = np.exp(-p11 / sd)
    D = 1.0 - e
    dp11 = np.stack([x[:, 1] + x[:, 2], x[:, 0] + x[:, 2], x[:, 0] + x[:, 1]], 1) * dx
    dD = (e / sd)[:, None] * dp11
    fn = f[:, :NINV]
    in_range = np.all((fn >= np.asarray(consts["fmin"])) & (fn <= np.asarray(consts["fmax"])), axis=1)
    return f, J, D, dD, in_range


def forward(p, f):
    """y[n], dy/df [n][16] (BF16 hidden weights, float64 activations)."""
    q = unpack(p)
    W1, W2, W3 = bf16(q["W1"]), bf16(q["W2"]), bf16(q["W3"])
    h1 = np.tanh(f @ W1.T)
    h2 = np.tanh(h1 @ W2.T + q["b2"])
    h3 = np.tanh(h2 @ W3.T + q["b3"])
    y = h3 @ q["w4"] + q["b4"]
    d3 = q["w4"] * (1 - h3 * h3)
    d2 = (d3 @ W3) * (1 - h2 * h2)
    d1 = (d2 @ W2) * (1 - h1 * h1)
    g = d1 @ W1
    return y, g


def v3(p, R, consts):
    """The surrogate's V3 [Eh] and dV3/dR [Eh/bohr] at R[n][3]."""
    f, J, D, dD, _ = features(R, consts)
    y, g = forward(p, f)
    grad = y[:, None] * dD + D[:, None] * np.einsum("ni,nik->nk", g[:, :NINV], J)
    return D * y / EV_PER_EH, grad / EV_PER_EH


def loss_and_grad(p, R, e, gt, consts, w_e, w_f, rounding="exact"):
    """Mean loss parts (energy, force) over the batch and the gradient d loss / d params [NPARAM]."""
    rnd = bf16 if rounding == "device" else (lambda a: np.asarray(a, dtype=np.float64))
    q = unpack(p)
    W1, W2, W3 = bf16(q["W1"]), bf16(q["W2"]), bf16(q["W3"])
    b2, b3, w4, b4 = q["b2"], q["b3"], q["w4"], q["b4"]
    f, J, D, dD, _ = features(R, consts)
    n = f.shape[0]
    we, wf = w_e / n, w_f / n
    # forward and input gradient
    h1 = np.tanh(f @ W1.T)
    h2 = np.tanh(h1 @ W2.T + b2)
    h3 = np.tanh(h2 @ W3.T + b3)
    s1, s2, s3 = 1 - h1 * h1, 1 - h2 * h2, 1 - h3 * h3
    y = h3 @ w4 + b4
    d3 = w4 * s3
    u2 = d3 @ W3
    d2 = u2 * s2
    u1 = d2 @ W2
    d1 = u1 * s1
    g = d1 @ W1
    # loss and its partials r = dL/dy, c = dL/dg
    err_e = D * y - np.asarray(e, float)
    gpred = y[:, None] * dD + D[:, None] * np.einsum("ni,nik->nk", g[:, :NINV], J)
    rg = gpred - np.asarray(gt, float)
    loss_e = float(np.sum(we * err_e ** 2))
    loss_f = float(np.sum(wf * np.sum(rg ** 2, 1)))
    r = 2 * we * err_e * D + np.sum(2 * wf * rg * dD, 1)
    c = np.zeros((n, NF))
    c[:, :NINV] = np.einsum("nk,nik->ni", 2 * wf * rg * D[:, None], J)
    # tangent pass along c
    z1d = rnd(c) @ W1.T
    hd1 = s1 * z1d
    z2d = rnd(hd1) @ W2.T
    hd2 = s2 * z2d
    z3d = rnd(hd2) @ W3.T
    # reverse through the value and the tangent
    hb3 = w4 * (r[:, None] - 2 * h3 * z3d)
    zb3 = s3 * hb3
    gW3 = rnd(d3).T @ rnd(hd2) + rnd(zb3).T @ rnd(h2)
    gb3 = zb3.sum(0)
    gw4 = (r[:, None] * h3 + s3 * z3d).sum(0)
    gb4 = r.sum()
    hb2 = rnd(zb3) @ W3 - 2 * h2 * z2d * u2
    zb2 = s2 * hb2
    gW2 = rnd(d2).T @ rnd(hd1) + rnd(zb2).T @ rnd(h1)
    gb2 = zb2.sum(0)
    hb1 = rnd(zb2) @ W2 - 2 * h1 * z1d * u1
    zb1 = s1 * hb1
    gW1 = rnd(d1).T @ rnd(c) + rnd(zb1).T @ rnd(f)
    grad = pack(dict(W1=gW1, W2=gW2, W3=gW3, b2=gb2, b3=gb3, w4=gw4, b4=gb4))
    return loss_e, loss_f, grad


def init_params(seed):
    """Random initial parameters: Glorot-uniform hidden weights, zero biases, a small output layer."""
    rng = np.random.default_rng(seed)
    d = {}
    a = np.sqrt(6.0 / (NINV + 1 + NH))
    d["W1"] = np.zeros((NH, NF))
    d["W1"][:, :NINV] = rng.uniform(-a, a, (NH, NINV))
    d["W1"][:, NF - 1] = rng.uniform(-0.1, 0.1, NH)
    a = np.sqrt(6.0 / (2 * NH))
    d["W2"] = rng.uniform(-a, a, (NH, NH))
    d["W3"] = rng.uniform(-a, a, (NH, NH))
    d["b2"], d["b3"] = np.zeros(NH), np.zeros(NH)
    d["w4"] = rng.uniform(-a, a, NH)
    d["b4"] = 0.0
    return pack(d)
