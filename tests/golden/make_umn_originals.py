"""Golden values of the UMN surfaces from the original UMN Fortran modules the reference ships beside its
fits -- an independent second source (the oracle and the library follow the reference's
src/PESs/*_UMN_PES_Class.F90 and its dtb/ coefficient files instead):

* O4: dtb/Systems/O4/PESs/UMN/ReCheck/PES_O4_{singlet_umn_v1,triplet_umn_v2,quintet_umn_v1}.f90;
* N4 (whose PIP and 276 coefficients N3 UMN evaluates with three distances at 10^3 bohr):
  module PES_N4_singlet_umn_v3 in dtb/Systems/N4/PESs/UMN/ReCheck/ReCheckOriginalPESsAndDiatomic.F90;
* O3 2 5A': module PES_O3_2_5Ap_umn_v1 in dtb/Systems/O3/PESs/AbInitioData/ReCheckOriginalPESsAndDiatomic.F90;
* the O2 diatomic (ev2gm2 with its D3 dispersion, in the O4 quintet module) and the N2 diatomic
  (ev2gm2, imol = 1, in the N4 module).

For each surface: the module's inline C(:), MEG parameters, Eref, totdiss and unit constants, and
sum_i C(i) B(i) [kcal/mol] at seeded geometries, evaluated by interpreting the module's own
EvMorse/EvMono/EvPoly/evbas statements (parsed with the parsers of
coarseair_gb300/csrc/gen/gen_pip.py) in double precision, in statement order, together with the same sum
on absolute values (the rounding scale).  For the diatomics: the module's values on a grid of
distances, and for O2 also in the units the reference's O2_UMN_DiatomicPotential_Class keeps.

Usage: python tests/golden/make_umn_originals.py <reference checkout>  (writes umn_originals.json here)
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
    g = re.search(r"double precision\s*,\s*parameter\s*::\s*%s\s*=\s*&?\s*([-+0-9.dDeE]+)" % name, text, re.I)
    return fnum(g.group(1))


def coefficients(text):
    g = re.search(r"double precision\s*,\s*parameter\s*::\s*C\((\d+)\)\s*=\s*\(/(.*?)/\)", text, re.I | re.S)
    body = re.sub(r"!.*", "", g.group(2)).replace("&", " ")
    vals = [fnum(x) for x in body.replace(",", " ").split()]
    assert len(vals) == int(g.group(1))
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


def geometries(n, seed, natoms):
    """Seeded configurations with every pair distance in 2..6 bohr; pairs (12,13,14,23,24,34) or (12,13,23)."""
    import random
    rnd = random.Random(seed)
    pairs = ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)) if natoms == 4 else ((0, 1), (0, 2), (1, 2))
    out = []
    while len(out) < n:
        X = [[rnd.uniform(-3.0, 3.0) for _ in range(3)] for _ in range(natoms)]
        R = [math.dist(X[i], X[j]) for i, j in pairs]
        if all(2.0 <= r <= 6.0 for r in R):
            out.append(R)
    return out


def surface(text, R_list):
    """The module's coefficients and parameters, and sum C B (and its absolute-value scale) at each
    distance set of R_list [bohr]."""
    C = coefficients(text)
    a, ab = parameter(text, "a"), parameter(text, "ab")
    if re.search(r"parameter\s*::\s*re\s*=", text, re.I):
        ra = rb = parameter(text, "re")
    else:
        ra, rb = parameter(text, "ra"), parameter(text, "rb")
    cconv = parameter(text, "Cconv")
    mono, poly, basis = structures(text)
    vals, scales = [], []
    for Rb in R_list:
        x = [math.exp(-(r * cconv - ra) / a - ((r * cconv - rb) ** 2.0) / ab) for r in Rb]
        vals.append(evaluate(mono, poly, basis, C, x))
        scales.append(evaluate(mono, poly, basis, C, x, absolute=True))
    return {"C": C, "a": a, "ab": ab, "ra": ra, "rb": rb, "Eref": parameter(text, "Eref"),
            "totdiss": parameter(text, "totdiss"), "Cconv": cconv, "Econv": parameter(text, "Econv"),
            "n_monomials": len(mono), "n_polynomials": len(poly), "n_basis": len(basis),
            "R_bohr": R_list, "sum_cb_kcal": vals, "abs_sum_cb_kcal": scales}


def n2_diatomic(text):
    """ev2gm2 of the N4 module for N2 (imol = 1): y = (r^4 - re^4)/(r^4 + re^4), f(y) a sextic,
    u = exp(-f (r - re)), v = de (1 - u)^2 - de [kcal/mol], r in Angstrom."""
    ev = "\n".join(gen_pip.subroutine_body(text, "ev2gm2"))
    blk = re.search(r"if\s*\(imol\s*\.eq\.\s*1\)\s*then(.*?)else", ev, re.I | re.S).group(1)
    red = fnum(re.search(r"red\s*=\s*([-+0-9.dDeE]+)", blk).group(1))
    de = fnum(re.search(r"de\s*=\s*([-+0-9.dDeE]+)", blk).group(1))
    cs = [fnum(re.search(r"cs\(%d\)\s*=\s*([-+0-9.dDeE]+)" % k, blk).group(1)) for k in range(7)]

    def v(r):
        y = (r * r * r * r - red * red * red * red) / (r * r * r * r + red * red * red * red)
        fy = (cs[0] + cs[1] * y + cs[2] * y * y + cs[3] * y * y * y + cs[4] * y * y * y * y
              + cs[5] * y * y * y * y * y + cs[6] * y * y * y * y * y * y)
        u = math.exp(-fy * (r - red))
        return de * (1.0 - u) * (1.0 - u) - de

    return v, {"red": red, "de": de, "cs": cs}


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
    dtb = os.path.join(ref, "dtb", "Systems")
    out = {}
    for name, fn in FILES.items():
        text = open(os.path.join(dtb, "O4", "PESs", "UMN", "ReCheck", fn)).read()
        out["O4_" + name] = dict(surface(text, geometries(16, {"Singlet": 1, "Triplet": 2, "Quintet": 3}[name], 4)),
                                 file=fn)
    text = open(os.path.join(dtb, "O4", "PESs", "UMN", "ReCheck", FILES["Quintet"])).read()
    v, consts = diatomic(text)
    cconv = parameter(text, "Cconv")
    r_bohr = [1.6 + 0.2 * i for i in range(60)]
    out["O2"] = {"file": FILES["Quintet"], "constants": consts, "r_bohr": r_bohr,
                 "v_kcal": [v(r * cconv) for r in r_bohr],
                 "v_hartree_reference_units": [v.hartree(r, cconv) for r in r_bohr]}
    n4 = open(os.path.join(dtb, "N4", "PESs", "UMN", "ReCheck", "ReCheckOriginalPESsAndDiatomic.F90")).read()
    out["N4"] = dict(surface(n4, geometries(16, 4, 4)), file="ReCheckOriginalPESsAndDiatomic.F90 (N4)")
    # N3 UMN: the N4 surface with the pairs 1-4, 2-4, 3-4 at 10^3 bohr
    tri = geometries(16, 5, 3)
    out["N3"] = dict(surface(n4, [[R[0], R[1], 1.0e3, R[2], 1.0e3, 1.0e3] for R in tri]), R3_bohr=tri,
                     file="ReCheckOriginalPESsAndDiatomic.F90 (N4)")
    v2, c2 = n2_diatomic(n4)
    cconv = parameter(n4, "Cconv")
    out["N2"] = {"constants": c2, "r_bohr": r_bohr, "v_kcal": [v2(r * cconv) for r in r_bohr]}
    o3 = open(os.path.join(dtb, "O3", "PESs", "AbInitioData", "ReCheckOriginalPESsAndDiatomic.F90")).read()
    out["O3_25A1"] = dict(surface(o3, geometries(16, 6, 3)), file="ReCheckOriginalPESsAndDiatomic.F90 (O3 2 5A')")
    with open(os.path.join(HERE, "umn_originals.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1])
