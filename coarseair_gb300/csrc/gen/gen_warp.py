#!/usr/bin/env python3
"""Generator of the lane-parallel right-hand-side programs of the warp integrator.

The warp integrator (csrc/cair_warp.cu) gives one trajectory a whole warp: its two half-warps
run different modified-midpoint sequences of a Bulirsch-Stoer attempt at the same time, and the
16 lanes of a half-warp evaluate one right-hand side together.  A right-hand side is a program
of levels; a level holds up to 16 independent instructions of one kind, lane l executes the
l-th, and the half-warp meets (__syncwarp) between levels.  Instructions read and write slots
of a per-half-warp array of doubles in shared memory:

  SOP    r = sum_j (+-) s[a_j] * s[b_j]        first term a multiply, the rest fused multiply-adds
  EXP    r = exp(s[a])                           the library's table-driven exponential (fexp)
  RSQRT  r = 1 / sqrt(s[a])
  RECIP  r = 1 / s[a]
  TANH   r = tanh(s[a])                          the library's ftanh (derivative taken as 1 - r^2)

This script restates the device surfaces as expression graphs (the same formulas and constants
as csrc/cair_device.cuh, which cites the reference routine of each), differentiates the energy
by reverse mode (adjoints accumulated left to right as they are produced), folds every product
used once into the sum that consumes it, hoists what depends only on a surface's constants into
a program run once per surface load, splits long sums, schedules the instructions into levels
by longest remaining path and assigns slots by liveness.  Per surface model it writes three
programs: `grad` (y -> dy/dt, Hamilton's equations with dV/dQ), `energy` (y -> H and the
reciprocal pair distances, the end-of-collision check) and `const` (constants -> hoisted values).

Input: csrc/generated/pip_tables.json (written by gen_pip.py from the reference's PIP routines)
and the O2 UMN coefficients of csrc/cair_device.cuh.  Output: csrc/generated/warp_prog.h.

Usage:  python gen_warp.py
"""
import json
import math
import os
import re
import struct

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.abspath(os.path.join(HERE, ".."))
SPLIT = 3           # sums with more terms are split into partial sums (a record holds 3 terms)
COST = {"sop": None, "exp": 12, "rsqrt": 8, "recip": 10, "tanh": 22}
KIND = {"sop": 0, "exp": 1, "rsqrt": 2, "recip": 3, "tanh": 4}

B_TO_ANG = 0.52917721092
KCM_TO_HARTREE = 0.159360144e-2
KCMANG_TO_HARTB = 0.843297564e-3

# runtime constant sources (the kernel reads them from DevSys / DevPes)
SRC = {"lit": 0, "tpq": 1, "mmimn": 2, "o2ab": 3, "coef": 4, "pes": 5}
PES_FIELD = {"a": 0, "ab": 1, "ra": 2, "rb": 3, "inv_a": 4, "inv_ab": 5}


# ----------------------------------------------------------------------------------------------
# Expression graph with constant folding, identities and common-subexpression merging
# ----------------------------------------------------------------------------------------------
def _bits(v):
    return struct.pack("<d", float(v))


class Graph:
    def __init__(self):
        self.ops = []       # (op, args tuple, payload)
        self.memo = {}

    def _mk(self, op, args=(), payload=None):
        key = (op, args, payload)
        n = self.memo.get(key)
        if n is None:
            n = len(self.ops)
            self.ops.append(key)
            self.memo[key] = n
        return E(self, n)

    def lit(self, v):
        return self._mk("lit", (), _bits(v))

    def const(self, src, idx=0):
        return self._mk("const", (), (src, idx))

    def inp(self, i):
        return self._mk("in", (), i)

    def litval(self, n):
        op, _, p = self.ops[n]
        return struct.unpack("<d", p)[0] if op == "lit" else None

    # constructors with simplification
    def add(self, a, b):
        va, vb = self.litval(a.n), self.litval(b.n)
        if va is not None and vb is not None:
            return self.lit(va + vb)
        if va == 0.0:
            return b
        if vb == 0.0:
            return a
        x, y = sorted((a.n, b.n))
        return self._mk("add", (x, y))

    def sub(self, a, b):
        va, vb = self.litval(a.n), self.litval(b.n)
        if va is not None and vb is not None:
            return self.lit(va - vb)
        if vb == 0.0:
            return a
        if va == 0.0:
            return self.neg(b)
        return self._mk("sub", (a.n, b.n))

    def mul(self, a, b):
        va, vb = self.litval(a.n), self.litval(b.n)
        if va is not None and vb is not None:
            return self.lit(va * vb)
        if va == 0.0 or vb == 0.0:
            return self.lit(0.0)
        if va == 1.0:
            return b
        if vb == 1.0:
            return a
        if va == -1.0:
            return self.neg(b)
        if vb == -1.0:
            return self.neg(a)
        x, y = sorted((a.n, b.n))
        return self._mk("mul", (x, y))

    def neg(self, a):
        va = self.litval(a.n)
        if va is not None:
            return self.lit(-va)
        op, args, _ = self.ops[a.n]
        if op == "neg":
            return E(self, args[0])
        return self._mk("neg", (a.n,))

    def fn(self, op, a):
        return self._mk(op, (a.n,))

    # reverse mode: d out / d wrt[i], contributions summed in the order they are produced
    def grad(self, out, wrt):
        wset = {w.n for w in wrt}
        dep = {}
        for n in range(out.n + 1):
            op, args, _ = self.ops[n]
            dep[n] = n in wset or any(dep.get(a, False) for a in args)
        adj = {out.n: [self.lit(1.0)]}
        for n in range(out.n, -1, -1):
            if n not in adj or n in wset or not dep[n]:
                continue
            terms = adj.pop(n)
            a = terms[0]
            for t in terms[1:]:
                a = a + t
            op, args, _ = self.ops[n]

            def push(k, v):
                if dep[k]:
                    adj.setdefault(k, []).append(v)
            if op == "add":
                push(args[0], a)
                push(args[1], a)
            elif op == "sub":
                push(args[0], a)
                push(args[1], -a)
            elif op == "neg":
                push(args[0], -a)
            elif op == "mul":
                x, y = E(self, args[0]), E(self, args[1])
                push(args[0], a * y)
                push(args[1], a * x)
            elif op == "exp":
                push(args[0], a * E(self, n))
            elif op == "recip":
                r = E(self, n)
                push(args[0], -(a * (r * r)))
            elif op == "tanh":
                t = E(self, n)
                push(args[0], a * (1.0 - t * t))
            else:
                raise ValueError("no derivative for " + op)
        res = []
        for w in wrt:
            terms = adj.get(w.n, [])
            if not terms:
                res.append(self.lit(0.0))
                continue
            a = terms[0]
            for t in terms[1:]:
                a = a + t
            res.append(a)
        return res


class E:
    __slots__ = ("g", "n")

    def __init__(self, g, n):
        self.g, self.n = g, n

    def _w(self, o):
        return o if isinstance(o, E) else self.g.lit(o)

    def __add__(self, o):
        return self.g.add(self, self._w(o))

    def __radd__(self, o):
        return self.g.add(self._w(o), self)

    def __sub__(self, o):
        return self.g.sub(self, self._w(o))

    def __rsub__(self, o):
        return self.g.sub(self._w(o), self)

    def __mul__(self, o):
        return self.g.mul(self, self._w(o))

    def __rmul__(self, o):
        return self.g.mul(self._w(o), self)

    def __neg__(self):
        return self.g.neg(self)


def fexp(x):
    return x.g.fn("exp", x)


def rsqrt(x):
    return x.g.fn("rsqrt", x)


def recip(x):
    return x.g.fn("recip", x)


def tanh(x):
    return x.g.fn("tanh", x)


# ----------------------------------------------------------------------------------------------
# The device formulas (csrc/cair_device.cuh) as graphs
# ----------------------------------------------------------------------------------------------
def o2_coefficients():
    text = open(os.path.join(CSRC, "cair_device.cuh")).read()
    body = re.search(r"kO2A\[8\]\s*=\s*\{(.*?)\};", text, re.S).group(1)
    vals = [float(x) for x in re.findall(r"[-+]?\d+\.\d+e[-+]?\d+", body)]
    assert len(vals) == 8
    return vals


def o2_umn(g, r, A):
    """o2_umn: eight Gaussians in r^2 plus the dispersion edisp (O2_UMN_DiatomicPotential_Class.F90)."""
    rang = r * B_TO_ANG
    r2 = rang * rang
    vv = g.lit(0.0)
    for k in range(8):
        e = fexp(-(g.const("o2ab", k) * r2))
        vv = vv + A[k] * e
    vv = vv * 1.e-3
    r2r4, rs6, rs8, c6 = 2.59361680, 0.5299, 2.20, 12.8
    c8step = 3.0 * c6 * (r2r4 * r2r4)
    tmp = math.sqrt(c8step / c6)
    ss = rs6 * tmp + rs8
    s2 = ss * ss
    s3 = s2 * ss
    s6 = s3 * s3
    s4 = s2 * s2
    s8 = s4 * s4
    rr2 = r * r
    r3 = rr2 * r
    r4 = rr2 * rr2
    r6 = r3 * r3
    r8 = r4 * r4
    d6 = r6 + s6
    d8 = r8 + s8
    q = recip(d6 * d8)
    i6 = d8 * q
    i8 = d6 * q
    e6 = c6 * i6
    e8 = c8step * i8
    vd = -e6 - 2.0 * e8
    return vv + vd


def n2_umn(g, r):
    """n2_umn: the UMN_ForN4 N2 curve (N2_UMN_ForN4 Ev2gm2)."""
    cs = [2.70963254293, 1.32620177271e-1, 2.96757048793e-1, 1.97112432229e-1, -5.02002309588e-1,
          3.80734244606e-1, 1.21001628750]
    de, red, red4 = 228.7, 1.098, 1.4534810048
    rang = r * B_TO_ANG
    r3 = (rang * rang) * rang
    r4 = r3 * rang
    ts = r4 + red4
    its = recip(ts)
    y = (r4 - red4) * its
    y2 = y * y
    y3 = y2 * y
    y4 = y2 * y2
    y5 = y3 * y2
    y6 = y3 * y3
    fy = cs[0] + cs[1] * y + cs[2] * y2 + cs[3] * y3 + cs[4] * y4 + cs[5] * y5 + cs[6] * y6
    u = fexp(-(fy * (rang - red)))
    minu = 1.0 - u
    return (de * (minu * minu) - de) * KCM_TO_HARTREE


def pip_value(g, tab, x, coef, v0):
    """V0 + sum_k C_k B_k over the PIP tables (monomials, polynomials, basis)."""
    mv = []
    for t in tab["mono"]:
        if t[0] == "one":
            mv.append(g.lit(1.0))
        elif t[0] == "var":
            mv.append(x[t[1]])
        else:
            mv.append(mv[t[1]] * mv[t[2]])
    pv = []
    for t in tab["poly"]:
        if t[0] == "sum":
            e = mv[t[1][0]]
            for k in t[1][1:]:
                e = e + mv[k]
            pv.append(e)
        else:
            e = pv[t[1]] * pv[t[2]]
            for c in t[3]:
                e = e - pv[c]
            pv.append(e)
    v = g.lit(v0)
    for i, j in enumerate(tab["basis"]):
        v = v + coef(i) * pv[j]
    return v


def pes_o3(g, R, tabs):
    """pes_o3 (O3 UMN): MEG variables, O2 UMN diatomics, the O3 PIP.  Returns V and dV/dR: the PIP's
    gradient is taken in angstrom and converted with the surface's own factor KCMANG, the diatomics'
    in bohr, as the surface evaluates them."""
    A = o2_coefficients()
    x, vd, rang = [], [], []
    for i in range(3):
        ra = R[i] * B_TO_ANG
        rang.append(ra)
        d1 = ra - g.const("pes", PES_FIELD["ra"])
        d2 = ra - g.const("pes", PES_FIELD["rb"])
        x.append(fexp(-(d1 * g.const("pes", PES_FIELD["inv_a"])) - (d2 * d2) * g.const("pes", PES_FIELD["inv_ab"])))
        vd.append(o2_umn(g, R[i], A))
    vdiat = (vd[0] + vd[1]) + vd[2]
    vp = pip_value(g, tabs["O3"], x, lambda i: g.const("coef", i), 0.0)
    V = vp * KCM_TO_HARTREE + vdiat
    gp = g.grad(vp, rang)
    dVdR = [gp[i] * KCMANG_TO_HARTB + g.grad(vd[i], [R[i]])[0] for i in range(3)]
    return V, dVdR


def pes_n3(g, R, tabs):
    """pes_n3 (N3 UMN on the N4 PIP, the pinned pairs' MEG variables exactly zero); V and dV/dR."""
    x = [g.lit(0.0)] * 6
    vd, rang = [], []
    for i in range(3):
        ra = R[i] * B_TO_ANG
        rang.append(ra)
        d = ra - 1.098
        e = fexp(-d - (d * d) * (1.0 / 1.5))
        x[3 if i == 2 else i] = e  # RTemp(1), RTemp(2), RTemp(4)
        vd.append(n2_umn(g, R[i]))
    vdiat = ((0.0 + vd[0]) + vd[1]) + vd[2]
    vp = pip_value(g, tabs["N4"], x, lambda i: g.const("coef", i), 457.4)
    V = vdiat + vp * KCM_TO_HARTREE
    gp = g.grad(vp, rang)
    dVdR = [g.grad(vd[i], [R[i]])[0] + (gp[i] * KCM_TO_HARTREE) * B_TO_ANG for i in range(3)]
    return V, dVdR


def pes_o4(g, R, tabs):
    """pes_o4 (O4 UMN): MEG variables of the six pairs, the O4 PIP, six O2 UMN diatomics."""
    A = o2_coefficients()
    x, vd, rang = [], [], []
    for i in range(6):
        ra = R[i] * B_TO_ANG
        rang.append(ra)
        d1 = ra - g.const("pes", PES_FIELD["ra"])
        d2 = ra - g.const("pes", PES_FIELD["rb"])
        x.append(fexp(-(d1 * g.const("pes", PES_FIELD["inv_a"])) - (d2 * d2) * g.const("pes", PES_FIELD["inv_ab"])))
        vd.append(o2_umn(g, R[i], A))
    vdiat = g.lit(0.0)
    for v in vd:
        vdiat = vdiat + v
    vp = pip_value(g, tabs["O4"], x, lambda i: g.const("coef", i), 0.0)
    V = vp * KCM_TO_HARTREE + vdiat
    gp = g.grad(vp, rang)
    dVdR = [(gp[i] * KCM_TO_HARTREE) * B_TO_ANG + g.grad(vd[i], [R[i]])[0] for i in range(6)]
    return V, dVdR


def pes_n4(g, R, tabs):
    """pes_n4 (N4 UMN): the N4 PIP on all six MEG variables, six N2 UMN_ForN4 diatomics."""
    x, vd, rang = [], [], []
    for i in range(6):
        ra = R[i] * B_TO_ANG
        rang.append(ra)
        d = ra - 1.098
        x.append(fexp(-d - (d * d) * (1.0 / 1.5)))
        vd.append(n2_umn(g, R[i]))
    vdiat = g.lit(0.0)
    for v in vd:
        vdiat = vdiat + v
    vp = pip_value(g, tabs["N4"], x, lambda i: g.const("coef", i), 457.4)
    V = (vp * KCM_TO_HARTREE + 0.0) + vdiat
    gp = g.grad(vp, rang)
    dVdR = [(gp[i] * KCM_TO_HARTREE) * B_TO_ANG + g.grad(vd[i], [R[i]])[0] for i in range(6)]
    return V, dVdR


def nn_layout():
    """The packed device layout of the O3 NN / BNN coefficients (the CAIR_NN_* offsets of cair_device.cuh)."""
    text = open(os.path.join(CSRC, "cair_device.cuh")).read()
    return {k: int(v) for k, v in re.findall(r"#define CAIR_(?:NN|BNN)_(\w+) (\d+)", text)}


EV_TO_HARTREE = 1.0 / 27.2113839712790


def pes_o3nn(g, R, tabs, bnn=False, grad=True):
    """pes_o3nn: Compute (grad, six features, 6 -> 20 -> 10 -> 1 tanh network) or Potential (three scaled
    features through W1's storage read as 3 x NHL1); the BNN takes the output through exp(v + Noise)."""
    L = nn_layout()
    c = lambda i: g.const("coef", i)
    A = o2_coefficients()
    lam, re_ = c(L["LAM"]), c(L["RE"])
    p = [fexp(-(lam * (R[i] - re_))) for i in range(3)]
    vd = [o2_umn(g, R[i], A) for i in range(3)]
    vdiat = (vd[0] + vd[1]) + vd[2]
    gvp = [p[0] * p[1], p[1] * p[2], p[2] * p[0]]
    H1, H2 = L["H1"], L["H2"]
    if grad:
        gprod = gvp[0] * p[2]
        gc = [gvp[0] * p[0], gvp[0] * p[1], gvp[1] * p[1], gvp[1] * p[2], gvp[2] * p[0], gvp[2] * p[2]]
        G = [(gvp[0] + gvp[1]) + gvp[2], gprod,
             ((((gc[0] + gc[1]) + gc[2]) + gc[3]) + gc[4]) + gc[5],
             ((((gc[0] * p[0] + gc[1] * p[1]) + gc[2] * p[1]) + gc[3] * p[2]) + gc[4] * p[0]) + gc[5] * p[2],
             (gc[0] * p[2] + gc[2] * p[0]) + gc[5] * p[1],
             (gc[0] * p[1] + gc[2] * p[2]) + gc[4] * p[2]]
        y1 = []
        for j in range(H1):
            z = g.lit(0.0)
            for i in range(6):
                z = z + G[i] * c(L["W1"] + i + 6 * j)
            y1.append(tanh(z + c(L["B1"] + j)))
        v = g.lit(0.0)
        for k in range(H2):
            z = g.lit(0.0)
            for j in range(H1):
                z = z + y1[j] * c(L["W2"] + j + H1 * k)
            v = v + tanh(z + c(L["B2"] + k)) * c(L["W3"] + k)
    else:
        gvs = [p[0] + p[1], p[1] + p[2], p[2] + p[0]]
        G = [(gvp[0] + gvp[1]) + gvp[2], gvp[0] * p[2], (gvp[0] * gvs[0] + gvp[1] * gvs[1]) + gvp[2] * gvs[2]]
        G = [(G[i] - c(L["MEAN"] + i)) * recip(c(L["SD"] + i)) for i in range(3)]
        y1 = []
        for j in range(H1):
            z = c(L["B1"] + j)
            for l in range(3):
                z = z + c(L["W1P"] + l + 3 * j) * G[l]
            y1.append(tanh(z))
        v = g.lit(0.0)
        for k in range(H2):
            z = c(L["B2"] + k)
            for j in range(H1):
                z = z + c(L["W2"] + j + H1 * k) * y1[j]
            v = v + tanh(z) * c(L["W3"] + k)
    v = v + c(L["B3"])
    vout = fexp(v + c(L["NOISE"])) if bnn else v
    V = (vout - c(L["YSC"])) * EV_TO_HARTREE + vdiat
    dVdR = g.grad(V, R) if grad else None
    return V, dVdR


def pes_o3nn_pair(bnn):
    """Compute for the right-hand side, Potential for the Hamiltonian: the two networks the surface has."""
    def fn(g, R, tabs, grad=True):
        return pes_o3nn(g, R, tabs, bnn=bnn, grad=grad)
    fn.two_networks = True
    return fn


# surface -> (formula, atoms, lanes of the group that evaluates one right-hand side)
MODELS = {"o3_umn": (pes_o3, 3, 16), "n3_umn": (pes_n3, 3, 16), "o4_umn": (pes_o4, 4, 32), "n4_umn": (pes_n4, 4, 32),
          "o3_nn": (pes_o3nn_pair(False), 3, 16), "o3_bnn": (pes_o3nn_pair(True), 3, 16)}


def system(g, natoms):
    """Inputs y = [p(NV), q(NV)]; the last atom's position and the pair distances (rp3 / rp4)."""
    nv = 3 * (natoms - 1)
    y = [g.inp(i) for i in range(2 * nv)]
    p, q = y[:nv], y[nv:]
    Q = list(q) + [None] * 3
    m = [g.const("mmimn", i) for i in range(natoms - 1)]
    for c in range(3):
        acc = m[0] * Q[c]
        for i in range(1, natoms - 1):
            acc = acc + m[i] * Q[3 * i + c]
        Q[nv + c] = acc
    pairs = [(a, b) for a in range(natoms) for b in range(a + 1, natoms)]
    R, Ri = [], []
    for a, b in pairs:
        d = [Q[3 * a + c] - Q[3 * b + c] for c in range(3)]
        s2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2]
        ri = rsqrt(s2)
        R.append(s2 * ri)
        Ri.append(ri)
    return y, p, q, Q, R, Ri


def trans_to_cart(g, natoms, Ri, Q, dVdR):
    """trans_to_cart_3 / trans_to_cart_4: dV/dQ of the NV relative coordinates."""
    if natoms == 3:
        d0, d1, d2 = dVdR[0] * Ri[0], dVdR[1] * Ri[1], dVdR[2] * Ri[2]
        m1, m2 = g.const("mmimn", 0), g.const("mmimn", 1)
        a1, b1, a2, b2 = (1.0 - m1) * d1, m1 * d2, m2 * d1, (1.0 - m2) * d2
        m = [None] * 6
        for c in range(3):
            X0, X1, X2 = Q[c] - Q[3 + c], Q[c] - Q[6 + c], Q[3 + c] - Q[6 + c]
            m[c] = d0 * X0 + a1 * X1 - b1 * X2
            m[3 + c] = -(d0 * X0) - a2 * X1 + b2 * X2
        return m
    d = [dVdR[i] * Ri[i] for i in range(6)]
    m1, m2, m3 = g.const("mmimn", 0), g.const("mmimn", 1), g.const("mmimn", 2)
    m = [None] * 9
    for c in range(3):
        X0, X1, X2 = Q[c] - Q[3 + c], Q[c] - Q[6 + c], Q[c] - Q[9 + c]
        X3, X4, X5 = Q[3 + c] - Q[6 + c], Q[3 + c] - Q[9 + c], Q[6 + c] - Q[9 + c]
        m[c] = d[0] * X0 + d[1] * X1 + (1.0 - m1) * d[2] * X2 - m1 * d[4] * X4 - m1 * d[5] * X5
        m[3 + c] = -(d[0] * X0) - m2 * d[2] * X2 + d[3] * X3 + (1.0 - m2) * d[4] * X4 - m2 * d[5] * X5
        m[6 + c] = -(d[1] * X1) - m3 * d[2] * X2 - d[3] * X3 - m3 * d[4] * X4 + (1.0 - m3) * d[5] * X5
    return m


def rhs(g, surface, tabs):
    """Rhs (Hamilton's equations): [-dV/dQ (NV), Tpq p (NV)]."""
    fn, natoms, _ = MODELS[surface]
    y, p, q, Q, R, Ri = system(g, natoms)
    nv = len(p)
    dq = []
    for j in range(nv):
        i0 = j % 3
        acc = g.const("tpq", j + 9 * i0) * p[i0]
        for i in range(i0 + 3, nv, 3):
            acc = acc + g.const("tpq", j + 9 * i) * p[i]
        dq.append(acc)
    V, dVdR = fn(g, R, tabs)
    m = trans_to_cart(g, natoms, Ri, Q, dVdR)
    return [-m[i] for i in range(nv)] + dq


def energy(g, surface, tabs):
    """hamiltonian: [H, 1/R_p for every pair]."""
    fn, natoms, _ = MODELS[surface]
    y, p, q, Q, R, Ri = system(g, natoms)
    nv = len(p)
    h = g.lit(0.0)
    for i in range(nv):
        j0 = i % 3
        eki = g.const("tpq", j0 + 9 * i) * p[j0]
        for j in range(j0 + 3, nv, 3):
            eki = eki + g.const("tpq", j + 9 * i) * p[j]
        h = h + p[i] * eki
    V, _ = fn(g, R, tabs, grad=False) if getattr(fn, "two_networks", False) else fn(g, R, tabs)
    return [h * 0.5 + V] + Ri


# ----------------------------------------------------------------------------------------------
# Lowering: instructions, hoisting, splitting, levels, slots
# ----------------------------------------------------------------------------------------------
class Program:
    pass


def lower(g, outputs, ninputs):
    ops = g.ops
    outs = [o.n for o in outputs]
    # live nodes and use counts
    live, stack = set(), list(outs)
    while stack:
        n = stack.pop()
        if n in live:
            continue
        live.add(n)
        stack.extend(ops[n][1])
    uses = {n: 0 for n in live}
    for n in live:
        for a in ops[n][1]:
            uses[a] += 1
    atom = lambda n: ops[n][0] in ("lit", "const", "in")
    special = lambda n: ops[n][0] in ("exp", "rsqrt", "recip", "tanh")
    one = g.lit(1.0).n
    mat = set()
    for n in live:
        if atom(n):
            continue
        if special(n) or uses[n] > 1 or n in outs:
            mat.add(n)

    def strip(f):
        s = 1
        while ops[f][0] == "neg" and not (f in mat):
            s, f = -s, ops[f][1][0]
        return s, f
    changed = True
    while changed:
        changed = False
        for n in sorted(live):
            op, args, _ = ops[n]
            if op == "mul":
                for f in args:
                    s, h = strip(f)
                    if not atom(h) and h not in mat:
                        mat.add(h)
                        changed = True
            elif special(n):
                f = args[0]
                if not atom(f) and f not in mat:
                    mat.add(f)
                    changed = True
    for o in outs:
        if atom(o):
            mat.add(o)

    def expand(n, sign, root):
        op, args, _ = ops[n]
        if atom(n) or (n in mat and n != root):
            return [(sign, n, one)]
        if op == "add":
            return expand(args[0], sign, root) + expand(args[1], sign, root)
        if op == "sub":
            return expand(args[0], sign, root) + expand(args[1], -sign, root)
        if op == "neg":
            return expand(args[0], -sign, root)
        if op == "mul":
            sa, fa = strip(args[0])
            sb, fb = strip(args[1])
            return [(sign * sa * sb, fa, fb)]
        raise ValueError(op)

    # instructions: node -> (kind, operands)
    ins = {}
    for n in sorted(mat):
        op, args, _ = ops[n]
        if special(n):
            ins[n] = (op, [args[0]])
        else:
            ins[n] = ("sop", expand(n, 1, n))
    # hoisting: instructions over constants only
    const_node = {}

    def is_const(n):
        if n in const_node:
            return const_node[n]
        op = ops[n][0]
        if op in ("lit", "const"):
            r = True
        elif op == "in":
            r = False
        else:
            kind, opd = ins[n]
            srcs = [x for t in opd for x in t[1:]] if kind == "sop" else opd
            r = all(is_const(x) for x in srcs)
        const_node[n] = r
        return r
    for n in sorted(ins):
        is_const(n)
    # signs onto constant factors: a negative term takes -1 (for a sum's term x * 1), or the negated
    # constant (a literal, or a hoisted negation of a surface / system constant), so that the only
    # signed terms left multiply two variables
    nxt = [-1]
    minus_one = g.lit(-1.0).n
    negs = {}

    def const_operand(x):
        return (x >= 0 and ops[x][0] in ("lit", "const")) or const_node.get(x, False)

    def negated(x):
        if x >= 0 and ops[x][0] == "lit":
            return g.lit(-struct.unpack("<d", ops[x][2])[0]).n
        if x not in negs:
            m = nxt[0]
            nxt[0] -= 1
            ins[m] = ("sop", [(1, x, minus_one)])
            const_node[m] = True
            negs[x] = m
        return negs[x]
    for n in sorted(list(ins)):
        kind, opd = ins[n]
        if kind != "sop":
            continue
        terms = []
        for sg, a, b in opd:
            if sg < 0:
                if b == one:
                    b, sg = minus_one, 1
                elif const_operand(b):
                    b, sg = negated(b), 1
                elif const_operand(a):
                    a, sg = negated(a), 1
            terms.append((sg, a, b))
        ins[n] = ("sop", terms)
    # splitting of long sums (new nodes get negative ids)
    for n in sorted(list(ins)):
        kind, opd = ins[n]
        if kind != "sop" or len(opd) <= SPLIT:
            continue
        terms = opd
        while len(terms) > SPLIT:
            parts = []
            for k in range(0, len(terms), SPLIT):
                chunk = terms[k:k + SPLIT]
                if len(chunk) == 1:
                    parts.append(chunk[0])
                    continue
                m = nxt[0]
                nxt[0] -= 1
                ins[m] = ("sop", chunk)
                const_node[m] = all(const_node.get(x, True) if ops_kind(ops, x) != "in" else False
                                    for t in chunk for x in t[1:])
                parts.append((1, m, one))
            terms = parts
        ins[n] = ("sop", terms)
    return ins, const_node, one


def ops_kind(ops, x):
    return "node" if x < 0 else ops[x][0]


def operands(ins, n):
    kind, opd = ins[n]
    return [x for t in opd for x in t[1:]] if kind == "sop" else list(opd)


def schedule(ins, nodes, width):
    """Levels of at most `width` instructions of one kind, by longest remaining path, none costlier than the
    level's most critical instruction."""
    nodes = set(nodes)
    deps = {n: [x for x in operands(ins, n) if x in nodes] for n in nodes}
    users = {n: [] for n in nodes}
    for n in nodes:
        for d in set(deps[n]):
            users[d].append(n)
    cost = {n: (len(ins[n][1]) if ins[n][0] == "sop" else COST[ins[n][0]]) for n in nodes}
    prio = {}
    order = topo_order(nodes, deps)
    for n in reversed(order):
        prio[n] = cost[n] + max((prio[u] for u in users[n]), default=0)
    done, levels = set(), []
    pending = {n: len(set(deps[n])) for n in nodes}
    ready = [n for n in nodes if pending[n] == 0]
    while ready:
        # the most critical ready instruction sets the level's kind and its cost: a costlier instruction
        # would hold the level's lanes longer than the critical path needs, so it waits for a later level
        best = max(ready, key=lambda n: (prio[n], -abs(n)))
        kind, budget = ins[best][0], cost[best]
        cand = sorted([n for n in ready if ins[n][0] == kind and cost[n] <= budget],
                      key=lambda n: (-prio[n], abs(n)))[:width]
        levels.append((kind, cand))
        cs = set(cand)
        ready = [n for n in ready if n not in cs]
        for n in cand:
            done.add(n)
            for u in users[n]:
                pending[u] -= 1
                if pending[u] == 0:
                    ready.append(u)
    assert len(done) == len(nodes), "cycle in program"
    return levels


def topo_order(nodes, deps):
    seen, order = set(), []
    for n0 in sorted(nodes, key=abs):
        stack = [(n0, False)]
        while stack:
            n, post = stack.pop()
            if post:
                order.append(n)
                continue
            if n in seen:
                continue
            seen.add(n)
            stack.append((n, True))
            for d in deps[n]:
                if d not in seen:
                    stack.append((d, False))
    return order


def compile_model(surface, tabs):
    """Lower both programs; merge their constants and hoisted nodes into one const program."""
    _, natoms, lanes = MODELS[surface]
    ne = 6 * (natoms - 1)
    res = {}
    const_atoms = {}   # key (src, idx) or ('lit', bits) -> slot
    const_list = []    # (src, idx, value)

    def cslot(key, src, idx, val=0.0):
        if key not in const_atoms:
            const_atoms[key] = len(const_list)
            const_list.append((src, idx, val))
        return const_atoms[key]
    # the constant 1.0 first: SOP terms of sums use it as their second factor; 0.0 pads records
    cslot(("lit", _bits(1.0)), SRC["lit"], 0, 1.0)
    zero = cslot(("lit", _bits(0.0)), SRC["lit"], 0, 0.0)
    hoisted_all = []   # (program name, node) for the const program, program-local ids mapped later
    lowered = {}
    for name in ("grad", "energy"):
        g = Graph()
        outs = (rhs if name == "grad" else energy)(g, surface, tabs)
        ins, cnode, one = lower(g, outs, ne)
        lowered[name] = (g, outs, ins, cnode, one)
    # slot map per program: atoms (lits / consts) shared, hoisted nodes in the const region
    out = {}
    hoist_progs = []
    for name in ("grad", "energy"):
        g, outs, ins, cnode, one = lowered[name]
        ops = g.ops
        slot = {}
        for n in list(ins):
            for x in operands(ins, n):
                if x >= 0 and ops[x][0] == "lit":
                    v = struct.unpack("<d", ops[x][2])[0]
                    slot[x] = cslot(("lit", ops[x][2]), SRC["lit"], 0, v)
                elif x >= 0 and ops[x][0] == "const":
                    src, idx = ops[x][2]
                    slot[x] = cslot((src, idx), SRC[src], idx)
        hoisted = [n for n in ins if cnode.get(n, False)]
        hoist_progs.append((name, g, ins, hoisted, slot))
        out[name] = (g, outs, ins, cnode, one, slot)
    # hoisted nodes: const slots after the atoms, computed by the const program
    for name, g, ins, hoisted, slot in hoist_progs:
        for n in hoisted:
            slot[n] = cslot(("hoist", name, n), -1, 0)
    nconst = len(const_list)
    # inputs follow the constants
    ninp = ne
    base_in = nconst
    progs = {}
    cprog_levels = []
    for name, g, ins, hoisted, slot in hoist_progs:
        if hoisted:
            lv = schedule(ins, hoisted, 64)
            cprog_levels.append((name, lv, ins, slot, g))
    for name in ("grad", "energy"):
        g, outs, ins, cnode, one, slot = out[name]
        ops = g.ops
        for n in range(len(ops)):
            if ops[n][0] == "in":
                slot[n] = base_in + ops[n][2]
        body = [n for n in ins if not cnode.get(n, False)]
        levels = schedule(ins, body, lanes)
        # liveness: last level reading each value; outputs live to the end
        lvl_of = {}
        for L, (k, nodes) in enumerate(levels):
            for n in nodes:
                lvl_of[n] = L
        last = {}
        for L, (k, nodes) in enumerate(levels):
            for n in nodes:
                for x in operands(ins, n):
                    if x in lvl_of:
                        last[x] = L
        outset = [o.n for o in outs]
        for o in outset:
            last[o] = len(levels)
        free, nslot = [], base_in + ninp
        release = {}
        for L, (k, nodes) in enumerate(levels):
            for s_ in release.pop(L - 1, []):
                free.append(s_)
            free.sort(reverse=True)
            for n in nodes:
                if free:
                    s_ = free.pop()
                else:
                    s_ = nslot
                    nslot += 1
                slot[n] = s_
                release.setdefault(last.get(n, L), []).append(s_)
        progs[name] = dict(levels=levels, ins=ins, slot=slot, outs=[slot[o] for o in outset], out_nodes=outset,
                           ins_slots=[base_in + i for i in range(ninp)], nslot=nslot)
    nslot = max(p["nslot"] for p in progs.values())
    return dict(progs=progs, const_list=const_list, nconst=nconst, cprog=cprog_levels, nslot=nslot, lanes=lanes,
                zero=zero)


# ----------------------------------------------------------------------------------------------
# Emission: one 16-byte record per lane and level
# ----------------------------------------------------------------------------------------------
def records(levels, ins, slot, width, zero):
    """Levels of more than `width` instructions are cut into several; lane l of level L executes
    record L * width + l, 8 words:  w0 = active << 31 | kind << 28 (3 bits) | nt << 24 | signed << 23 |
    sign of term j << (20 + j), nt and `signed` the same for every record of the level (the most
    terms of its sums, whether any term still carries a sign); w1 = byte offset of the result;
    w2..w7 = byte offsets of the factors a_j, b_j of the terms (+-) s[a_j] * s[b_j], missing terms
    0 * 0 (a special instruction's operand is w2)."""
    out = []
    for kind, nl in levels:
        for c in range(0, len(nl), width):
            chunk = nl[c:c + width]
            ntm = max((len(ins[n][1]) if ins[n][0] == "sop" else 1) for n in chunk)
            sgn = any(t[0] < 0 for n in chunk if ins[n][0] == "sop" for t in ins[n][1])
            for lane in range(width):
                if lane >= len(chunk):
                    out += [0] * 8
                    continue
                n = chunk[lane]
                k, opd = ins[n]
                w = [0, 8 * slot[n]] + [8 * zero] * 6
                meta = (1 << 31) | (KIND[k] << 28) | (ntm << 24) | ((1 << 23) if sgn else 0)
                if k == "sop":
                    assert 1 <= len(opd) <= 3
                    for j, (sg, x, y) in enumerate(opd):
                        w[2 + 2 * j], w[3 + 2 * j] = 8 * slot[x], 8 * slot[y]
                        if sg < 0:
                            meta |= 1 << (20 + j)
                else:
                    w[2] = 8 * slot[opd[0]]
                assert max(w[1:]) < (1 << 20)
                w[0] = meta
                out += w
    return out


def stats(levels, ins):
    nins = sum(len(nl) for _, nl in levels)
    flops = sum((len(ins[n][1]) if k == "sop" else COST[k]) for k, nl in levels for n in nl)
    crit = sum(max((len(ins[n][1]) if k == "sop" else COST[k]) for n in nl) for k, nl in levels)
    return nins, flops, crit


def arr(ctype, name, vals, align=None):
    body = ",".join(str(v) for v in vals) if vals else "0"
    att = " __attribute__((aligned(%d)))" % align if align else ""
    return "__device__ static const %s %s[%d]%s = {%s};" % (ctype, name, max(1, len(vals)), att, body)


def emit(models, path):
    L = ["/* Lane-parallel right-hand-side programs of the warp integrator (cair_warp.cu).",
         " * Generated by csrc/gen/gen_warp.py, do not edit.",
         " * A program is NLEV levels of W records of 8 words (W the model's LANES), lane l of level L executing",
         " * record W L + l: w0 = active << 31 | kind << 28 | nterm << 24 | signed << 23 | term signs << 20 (kind",
         " * 0 sum of products, 1 exp, 2 rsqrt, 3 reciprocal, 4 tanh; nterm and signed uniform over the level),",
         " * w1 = result byte offset, w2..w7 = byte offsets of a0, b0, a1, b1, a2, b2: sum_j (+-) s[a_j] * s[b_j]",
         " * (a special's operand is w2). */",
         "#pragma once", ""]
    for key, m in models.items():
        P = m["progs"]
        L.append("/* %s: %d slots, %d constants (%d from the surface / system, %d hoisted)" %
                 (key, m["nslot"], m["nconst"], sum(1 for c in m["const_list"] if c[0] >= 0),
                  sum(1 for c in m["const_list"] if c[0] < 0)))
        for name in ("grad", "energy"):
            nins, flops, crit = stats(P[name]["levels"], P[name]["ins"])
            L.append(" * %-6s: %d levels, %d instructions, %d FP64 operations, critical path %d" %
                     (name, len(P[name]["levels"]), nins, flops, crit))
        L.append(" */")
        L.append("#define WP_%s_LANES %d" % (key.upper(), m["lanes"]))
        L.append("#define WP_%s_NSLOT %d" % (key.upper(), m["nslot"]))
        L.append("#define WP_%s_NCONST %d" % (key.upper(), m["nconst"]))
        cs = [c[0] if c[0] >= 0 else 255 for c in m["const_list"]]
        ci = [c[1] for c in m["const_list"]]
        lits = [repr(c[2]) if c[0] == SRC["lit"] else "0.0" for c in m["const_list"]]
        L.append(arr("unsigned char", "wp_%s_csrc" % key, cs))
        L.append(arr("unsigned short", "wp_%s_cidx" % key, ci))
        L.append(arr("double", "wp_%s_clit" % key, lits))
        # const program: the hoisted nodes of both programs
        rec = []
        for pname, lv, ins, slot, g in m["cprog"]:
            rec += records(lv, ins, slot, m["lanes"], m["zero"])
        L.append("#define WP_%s_CPROG_NLEV %d" % (key.upper(), len(rec) // (8 * m["lanes"])))
        L.append(arr("unsigned int", "wp_%s_cprog_rec" % key, rec, 16))
        for name in ("grad", "energy"):
            p = P[name]
            rec = records(p["levels"], p["ins"], p["slot"], m["lanes"], m["zero"])
            L.append("#define WP_%s_%s_NLEV %d" % (key.upper(), name.upper(), len(rec) // (8 * m["lanes"])))
            L.append(arr("unsigned int", "wp_%s_%s_rec" % (key, name), rec, 16))
            L.append(arr("unsigned short", "wp_%s_%s_in" % (key, name), p["ins_slots"]))
            L.append(arr("unsigned short", "wp_%s_%s_out" % (key, name), p["outs"]))
        L.append("")
    with open(path, "w") as f:
        f.write("\n".join(L) + "\n")


def main():
    tabs = json.load(open(os.path.join(CSRC, "generated", "pip_tables.json")))
    models = {}
    for key in MODELS:
        models[key] = compile_model(key, tabs)
        for name in ("grad", "energy"):
            p = models[key]["progs"][name]
            print(key, name, "levels", len(p["levels"]), "stats", stats(p["levels"], p["ins"]), "slots", p["nslot"])
    emit(models, os.path.join(CSRC, "generated", "warp_prog.h"))


if __name__ == "__main__":
    main()
