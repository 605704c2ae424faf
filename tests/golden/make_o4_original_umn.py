"""Golden values of the O4 UMN surfaces from the original UMN Fortran that the reference ships beside
its fit files (dtb/Systems/O4/PESs/UMN/ReCheck/PES_O4_{singlet_umn_v1,triplet_umn_v2,quintet_umn_v1}.f90):
the module's inline C(430), a, ab, ra, rb, Eref, totdiss and unit constants, and sum_i C(i) B(i)
[kcal/mol] at seeded geometries, evaluated by interpreting the module's own EvMorse/EvMono/EvPoly/evbas
statements (parsed with the parsers of coarseair_gb300/csrc/gen/gen_pip.py) in double precision, in
statement order, together with the same sum on absolute values (the rounding scale); and the module's
O2 diatomic (ev2gm2 with its D3 dispersion, constants read from the module) on a grid of distances,
in the module's units (kcal/mol, its own autoang and autokcal) and in the units the reference's
O2_UMN_DiatomicPotential_Class keeps (hartree, B_To_Ang).

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


def diatomic(text):
    """ev2gm2's Gaussian sum and d3disp/edisp's two-body D3 term of the module, for O2 (imol = 4):
    v(r) = 0.627509523475149 sum_k as(k) exp(-alpha beta^k r^2) + (-s6 e6 - s8 e8) autokcal [kcal/mol],
    r in Angstrom, e6 = c6 / (d^6 + (rs6 sqrt(c8/c6) + rs8)^6), e8 likewise, d = r / autoang,
    c8 = 3 c6 r2r4(O)^2."""
    ev = "\n".join(gen_pip.subroutine_body(text, "ev2gm2"))
    alpha = fnum(re.search(r"alpha\s*=\s*([-+0-9.dDeE]+)", ev).group(1))
    beta = fnum(re.search(r"beta\s*=\s*([-+0-9.dDeE]+)", ev).group(1))
    as_ = [fnum(re.search(r"as\(%d\)\s*=\s*([-+0-9.dDeE]+)" % k, ev).group(1)) for k in range(8)]
    fac = fnum(re.search(r"v\s*=\s*v\s*\*\s*([-+0-9.dDeE]+)", ev).group(1))
    d3 = "\n".join(gen_pip.subroutine_body(text, "d3disp"))
    get = lambda name, body: fnum(re.search(r"%s\s*=\s*([-+0-9.dDeE]+)" % name, body).group(1))
    autoang, autokcal = get("autoang", d3), get("autokcal", d3)
    s6, s8, rs6, rs8 = get("s6", d3), get("s8", d3), get("rs6", d3), get("rs8", d3)
    c6 = get(r"c6\(1\)", d3)
    ed = re.search(r"subroutine edisp.*?r2r4\(1:94\)\s*=\s*\(/(.*?)/\)", text, re.I | re.S).group(1)
    r2r4 = [fnum(x) for x in re.sub(r"!.*", "", ed).replace("&", " ").replace(",", " ").split()]
    assert len(r2r4) == 94
    c8 = 3.0 * c6 * r2r4[7] * r2r4[7]
    tmp = math.sqrt(c8 / c6)

    def v(r_ang):
        g = 0.0
        for k in range(8):
            g = g + as_[k] * math.exp(-alpha * beta ** k * r_ang ** 2)
        g = g * fac
        d = r_ang / autoang
        e6 = c6 / (d ** 6 + (rs6 * tmp + rs8) ** 6)
        e8 = c8 / (d ** 8 + (rs6 * tmp + rs8) ** 8)
        return g + (-s6 * e6 - s8 * e8) * autokcal

    def v_hartree(r_bohr, b_to_ang):
        """The same terms in the units O2_UMN_DiatomicPotential_Class.F90:134-381 keeps: the Gaussian
        sum x 1e-3 [Eh], the dispersion [Eh] at d = (r B_To_Ang) / B_To_Ang."""
        r_ang = r_bohr * b_to_ang
        g = 0.0
        for k in range(8):
            g = g + as_[k] * math.exp(-alpha * beta ** k * r_ang ** 2)
        g = g * 1.0e-3
        d = r_ang / b_to_ang
        e6 = c6 / (d ** 6 + (rs6 * tmp + rs8) ** 6)
        e8 = c8 / (d ** 8 + (rs6 * tmp + rs8) ** 8)
        return g + (-s6 * e6 - s8 * e8)

    v.hartree = v_hartree
    consts = {"alpha": alpha, "beta": beta, "as": as_, "factor": fac, "autoang": autoang, "autokcal": autokcal,
              "s6": s6, "s8": s8, "rs6": rs6, "rs8": rs8, "c6": c6, "r2r4_O": r2r4[7]}
    return v, consts


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
    text = open(os.path.join(src, FILES["Quintet"])).read()
    v, consts = diatomic(text)
    cconv = parameter(text, "Cconv")
    r_bohr = [1.6 + 0.2 * i for i in range(60)]
    out["O2"] = {"file": FILES["Quintet"], "constants": consts, "r_bohr": r_bohr,
                 "v_kcal": [v(r * cconv) for r in r_bohr],
                 "v_hartree_reference_units": [v.hartree(r, cconv) for r in r_bohr]}
    with open(os.path.join(HERE, "o4_original_umn.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1])
