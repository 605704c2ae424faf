"""Golden values of the O4 UMN surfaces from the original UMN Fortran that the reference ships beside
its fit files (dtb/Systems/O4/PESs/UMN/ReCheck/PES_O4_{singlet_umn_v1,triplet_umn_v2,quintet_umn_v1}.f90):
the module's inline C(430), a, ab, ra, rb, Eref, totdiss and unit constants, and sum_i C(i) B(i)
[kcal/mol] at seeded geometries, evaluated by interpreting the module's own EvMorse/EvMono/EvPoly/evbas
statements (parsed with the parsers of coarseair_gb300/csrc/gen/gen_pip.py) in double precision, in
statement order, together with the same sum on absolute values (the rounding scale).

This is an independent second source for the O4 surfaces: the oracle and the library follow
O4_UMN_PES_Class.F90 and the dtb/ .dat files instead.

Usage: python tests/golden/make_o4_original_umn.py <reference checkout>  (writes o4_original_umn.json here)
"""
import json
import math
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "coarseair_gb300", "csrc", "gen"))
import gen_pip  # noqa: E402

FILES = {"Singlet": "PES_O4_singlet_umn_v1.f90", "Triplet": "PES_O4_triplet_umn_v2.f90",
         "Quintet": "PES_O4_quintet_umn_v1.f90"}


def fnum(s):
    return float(s.lower().replace("d", "e"))


def parameter(text, name):
    g = re.search(r"double precision\s*,\s*parameter\s*::\s*%s\s*=\s*([-+0-9.dDeE]+)" % name, text, re.I)
    return fnum(g.group(1))


def coefficients(text):
    g = re.search(r"double precision\s*,\s*parameter\s*::\s*C\(430\)\s*=\s*\(/(.*?)/\)", text, re.I | re.S)
    body = re.sub(r"!.*", "", g.group(1)).replace("&", " ")
    vals = [fnum(x) for x in body.replace(",", " ").split()]
    assert len(vals) == 430
    return vals


def structures(text):
    norm = lambda stmts: [re.sub(r"=\s*1\.0d0$", "= One", s, flags=re.I) for s in stmts]
    mono = gen_pip.parse_monomials(norm(gen_pip.subroutine_body(text, "EvMono")), "rm", "rms")
    poly = gen_pip.parse_polynomials(gen_pip.subroutine_body(text, "EvPoly"), "p", "rm")
    basis = gen_pip.parse_basis(gen_pip.subroutine_body(text, "evbas"), "b", "b1", len(poly))
    return mono, poly, basis


def evaluate(mono, poly, basis, C, x, absolute=False):
    """sum C(i) b(i) with the module's statements in order (absolute: every operand taken absolute)."""
    op = abs if absolute else (lambda v: v)
    m = []
    for t in mono:
        m.append(1.0 if t[0] == "one" else op(x[t[1]]) if t[0] == "var" else m[t[1]] * m[t[2]])
    p = []
    for t in poly:
        if t[0] == "sum":
            acc = m[t[1][0]]
            for k in t[1][1:]:
                acc = acc + m[k]
        else:
            acc = p[t[1]] * p[t[2]]
            for k in t[3]:
                acc = acc + p[k] if absolute else acc - p[k]
        p.append(acc)
    v = 0.0
    for i, j in enumerate(basis):
        v = v + (abs(C[i]) * abs(p[j]) if absolute else C[i] * p[j])
    return v


def geometries(n, seed):
    """Seeded O4 configurations with all six pair distances in 2..6 bohr, pairs (12,13,14,23,24,34)."""
    import random
    rnd = random.Random(seed)
    out = []
    while len(out) < n:
        X = [[rnd.uniform(-3.0, 3.0) for _ in range(3)] for _ in range(4)]
        R = [math.dist(X[i], X[j]) for i, j in ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3))]
        if all(2.0 <= r <= 6.0 for r in R):
            out.append(R)
    return out


def main(ref):
    src = os.path.join(ref, "dtb", "Systems", "O4", "PESs", "UMN", "ReCheck")
    out = {}
    for name, fn in FILES.items():
        text = open(os.path.join(src, fn)).read()
        C = coefficients(text)
        a, ab, ra, rb = (parameter(text, k) for k in ("a", "ab", "ra", "rb"))
        cconv = parameter(text, "Cconv")
        mono, poly, basis = structures(text)
        R = geometries(16, {"Singlet": 1, "Triplet": 2, "Quintet": 3}[name])
        vals, scales = [], []
        for Rb in R:
            x = [math.exp(-(r * cconv - ra) / a - ((r * cconv - rb) ** 2.0) / ab) for r in Rb]
            vals.append(evaluate(mono, poly, basis, C, x))
            scales.append(evaluate(mono, poly, basis, C, x, absolute=True))
        out[name] = {"file": fn, "C": C, "a": a, "ab": ab, "ra": ra, "rb": rb, "Eref": parameter(text, "Eref"),
                     "totdiss": parameter(text, "totdiss"), "Cconv": cconv, "Econv": parameter(text, "Econv"),
                     "n_monomials": len(mono), "n_polynomials": len(poly), "n_basis": len(basis),
                     "R_bohr": R, "sum_cb_kcal": vals, "abs_sum_cb_kcal": scales}
    with open(os.path.join(HERE, "o4_original_umn.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1])
