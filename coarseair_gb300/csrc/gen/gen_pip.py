#!/usr/bin/env python3
"""Generator for the permutation-invariant-polynomial (PIP) tables of the UMN surfaces.

The UMN surfaces of CoarseAIR define their PIP bases as long lists of Fortran
assignments (monomials from products of the Morse/MEG variables, polynomials
from products of earlier polynomials minus correction terms, and a selection of
the polynomials that form the fitted basis).  Those lists are data that both the
CPU oracle and the CUDA kernels must reproduce exactly, so this script reads them
once from the reference sources and writes:

* ``oracle/pip_tables.h``                         -- the tables as plain C arrays,
  interpreted by the oracle's generic evaluator;
* ``coarseair_gb300/csrc/generated/pip_*.cuh``    -- straight-line FP64 device code
  for the GPU kernels (energy plus forward-mode gradient, keeping the reference's
  left-to-right evaluation order; for the N3 surface the three MEG variables of
  the pinned 10^3-bohr pairs are exactly zero, so every term that contains them is
  dropped, which leaves every remaining rounding step unchanged);
* ``coarseair_gb300/data/N3_UMN.dat``             -- the 276 linear coefficients that
  the N3 surface keeps inline in its source.

Sources (paths inside the CoarseAIR tree):

* O3:  src/PESs/O3_UMN_PES_Class.F90   ``Unified`` (336-478) / ``UnifiedBis`` (483-638)
* N3:  src/PESs/N3_UMN_PES_Class.F90   ``EvMono`` 677-799, ``EvdMdR`` 804-930,
       ``EvPoly`` 935-1249, ``evbas`` 1254-1325, ``EvdPdr`` 1330-1976, C(276) 108-201
* O4:  src/PESs/O4_UMN_PES_Class.F90   ``EvMono`` 571-693, ``EvdMdR`` 698-824,
       ``EvPoly`` 829-1303, ``evbas`` 1308-1388, ``EvdPdr`` 1393-1875
* N4 PIPNN: src/PESs/N4_UMN_PIPNN_PES_Class.F90 ``evmono49`` 1023-1145, ``evpoly49`` 1150-1466,
       ``bmx2b109`` 1753-1830: checked equal to the N4 tables; its basis values feed the networks
       (``generated/pip_n4nn.cuh``)

The derivative routines (EvdMdR / EvdPdr / UnifiedBis) are parsed only to check
that each of their statements is the product rule applied to the matching value
statement; the tables themselves come from the value routines.

Usage:  python gen_pip.py <path-to-CoarseAIR-tree>
"""
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.abspath(os.path.join(HERE, "..", "..", ".."))


# ----------------------------------------------------------------------------------------------
# Fortran text helpers
# ----------------------------------------------------------------------------------------------
def read(path):
    with open(path) as f:
        return f.read()


def subroutine_body(text, name):
    """Return the statements of subroutine `name` (case-insensitive), continuations joined."""
    lines = text.split("\n")
    start = None
    pat = re.compile(r"^\s*(pure\s+)?subroutine\s+" + name + r"\b", re.I)
    for i, l in enumerate(lines):
        if pat.match(l):
            start = i
            break
    if start is None:
        raise RuntimeError("subroutine %s not found" % name)
    body = []
    for l in lines[start + 1:]:
        if re.match(r"^\s*end\s+subroutine", l, re.I):
            break
        body.append(l)
    # strip comments, join '&' continuations
    stmts, cur = [], ""
    for l in body:
        l = l.split("!")[0].rstrip()
        if not l.strip():
            continue
        s = l.strip()
        if s.startswith("&"):
            s = s[1:]
        if s.endswith("&"):
            cur += s[:-1] + " "
            continue
        cur += s
        stmts.append(cur.strip())
        cur = ""
    return stmts


def idx(s):
    return int(s.strip())


# ----------------------------------------------------------------------------------------------
# Parsers for the value routines
# ----------------------------------------------------------------------------------------------
def parse_monomials(stmts, m, var):
    """rm(k) = One | var(i) | rm(a)*rm(b)  ->  list of ('one',) / ('var', i0) / ('mul', a, b)."""
    mono = {}
    r_one = re.compile(r"^%s\((\s*\d+)\)\s*=\s*One$" % m, re.I)
    r_var = re.compile(r"^%s\((\s*\d+)\)\s*=\s*%s\((\s*\d+)\)$" % (m, var), re.I)
    r_mul = re.compile(r"^%s\((\s*\d+)\)\s*=\s*%s\((\s*\d+)\)\s*\*\s*%s\((\s*\d+)\)$" % (m, m, m), re.I)
    for s in stmts:
        if not re.match(r"^%s\(" % m, s, re.I):
            continue
        for r, kind in ((r_one, "one"), (r_var, "var"), (r_mul, "mul")):
            g = r.match(s)
            if g:
                k = idx(g.group(1))
                if kind == "one":
                    mono[k] = ("one",)
                elif kind == "var":
                    mono[k] = ("var", idx(g.group(2)) - 1)
                else:
                    mono[k] = ("mul", idx(g.group(2)), idx(g.group(3)))
                break
        else:
            raise RuntimeError("unparsed monomial statement: " + s)
    n = max(mono) + 1
    assert sorted(mono) == list(range(n)), "monomial indices not contiguous"
    return [mono[k] for k in range(n)]


def parse_polynomials(stmts, p, m):
    """p(k) = m(..)+m(..)... | p(a)*p(b) [- p(c)]...  ->  ('sum', [monos]) / ('prod', a, b, [subs])."""
    poly = {}
    head = re.compile(r"^%s\((\s*\d+)\)\s*=\s*(.*)$" % p, re.I)
    term_m = re.compile(r"^%s\((\s*\d+)\)$" % m, re.I)
    prod = re.compile(r"^%s\((\s*\d+)\)\s*\*\s*%s\((\s*\d+)\)(.*)$" % (p, p), re.I)
    sub = re.compile(r"-\s*%s\((\s*\d+)\)" % p, re.I)
    for s in stmts:
        g = head.match(s)
        if not g:
            continue
        k, rhs = idx(g.group(1)), g.group(2).strip()
        gp = prod.match(rhs)
        if gp:
            rest = gp.group(3).strip()
            subs = [idx(x) for x in sub.findall(rest)]
            check = re.sub(r"\s", "", rest)
            expect = "".join("-%s(%d)" % (p.lower(), c) for c in subs)
            assert re.sub(r"\(\s*0*(\d+)\)", r"(\1)", check.lower()) == expect.lower(), s
            poly[k] = ("prod", idx(gp.group(1)), idx(gp.group(2)), subs)
        else:
            terms = [t.strip() for t in rhs.split("+")]
            ms = []
            for t in terms:
                gm = term_m.match(t)
                if not gm:
                    raise RuntimeError("unparsed polynomial statement: " + s)
                ms.append(idx(gm.group(1)))
            poly[k] = ("sum", ms)
    n = max(poly) + 1
    assert sorted(poly) == list(range(n)), "polynomial indices not contiguous"
    return [poly[k] for k in range(n)]


def parse_basis(stmts, b, b1, npoly):
    """Simulate the copy b1(i)=p(i-1) and the b(i)=b1(..) statements / do-loops."""
    basis = {}
    loop = None
    r_do = re.compile(r"^do\s+i\s*=\s*(\d+)\s*,\s*(\d+)$", re.I)
    r_end = re.compile(r"^end\s*do$|^enddo$", re.I)
    r_fix = re.compile(r"^%s\((\s*\d+)\)\s*=\s*%s\((\s*\d+)\)$" % (b, b1), re.I)
    r_lop = re.compile(r"^%s\(i\)\s*=\s*%s\(i\s*\+\s*(\d+)\)$" % (b, b1), re.I)
    for s in stmts:
        s2 = s.strip()
        g = r_do.match(s2)
        if g:
            loop = (int(g.group(1)), int(g.group(2)))
            continue
        if r_end.match(s2):
            loop = None
            continue
        g = r_fix.match(s2)
        if g:
            basis[idx(g.group(1))] = idx(g.group(2)) - 1
            continue
        g = r_lop.match(s2)
        if g and loop is not None:
            off = int(g.group(1))
            for i in range(loop[0], loop[1] + 1):
                basis[i] = i + off - 1
            continue
    nb = max(basis)
    assert sorted(basis) == list(range(1, nb + 1)), "basis indices not contiguous"
    out = [basis[i] for i in range(1, nb + 1)]
    assert all(0 <= j < npoly for j in out)
    return out


# ----------------------------------------------------------------------------------------------
# Structural check of the derivative routines against the product rule
# ----------------------------------------------------------------------------------------------
def check_derivatives(stmts, mono, poly, dm, dp, dvar, m, p):
    nm = np = 0
    norm = lambda s: re.sub(r"\s", "", s).lower()
    for s in stmts:
        s = norm(s)
        g = re.match(r"^%s\(i,(\d+)\)=(.*)$" % dm.lower(), s)
        if g:
            k, rhs = int(g.group(1)), g.group(2)
            t = mono[k]
            if t[0] == "one":
                exp = "zero"
            elif t[0] == "var":
                exp = "%s(i,%d)" % (dvar.lower(), t[1] + 1)
            else:
                a, bb = t[1], t[2]
                exp = "%s(i,%d)*%s(%d)+%s(%d)*%s(i,%d)" % (dm.lower(), a, m.lower(), bb, m.lower(), a, dm.lower(), bb)
            assert rhs == exp, (s, exp)
            nm += 1
            continue
        g = re.match(r"^%s\(i,(\d+)\)=(.*)$" % dp.lower(), s)
        if g:
            k, rhs = int(g.group(1)), g.group(2)
            t = poly[k]
            if t[0] == "sum":
                exp = "+".join("%s(i,%d)" % (dm.lower(), x) for x in t[1])
            else:
                a, bb, subs = t[1], t[2], t[3]
                exp = "%s(i,%d)*%s(%d)+%s(%d)*%s(i,%d)" % (dp.lower(), a, p.lower(), bb, p.lower(), a, dp.lower(), bb)
                exp += "".join("-%s(i,%d)" % (dp.lower(), c) for c in subs)
            assert rhs == exp, (s, exp)
            np += 1
    assert nm == len(mono), (nm, len(mono))
    assert np == len(poly), (np, len(poly))


# ----------------------------------------------------------------------------------------------
# Surface definitions
# ----------------------------------------------------------------------------------------------
def load_surfaces(ref):
    out = {}
    # O3 UMN: Unified / UnifiedBis (rM, P, rMs; dMdR, dPdR, dMsdR)
    t = read(os.path.join(ref, "src/PESs/O3_UMN_PES_Class.F90"))
    st = subroutine_body(t, "Unified")
    mono = parse_monomials(st, "rM", "rMs")
    poly = parse_polynomials(st, "P", "rM")
    basis = parse_basis(st, "B", "b1", len(poly))
    check_derivatives(subroutine_body(t, "UnifiedBis"), mono, poly, "dMdR", "dPdR", "dMsdR", "rM", "P")
    out["O3"] = dict(mono=mono, poly=poly, basis=basis, nvar=3)
    # N3 UMN (the N4 PIP on six MEG variables) and O4 UMN
    for key, fn in (("N4", "src/PESs/N3_UMN_PES_Class.F90"), ("O4", "src/PESs/O4_UMN_PES_Class.F90")):
        t = read(os.path.join(ref, fn))
        mono = parse_monomials(subroutine_body(t, "EvMono"), "rm", "rms")
        poly = parse_polynomials(subroutine_body(t, "EvPoly"), "p", "rm")
        basis = parse_basis(subroutine_body(t, "evbas"), "b", "b1", len(poly))
        dm_st = subroutine_body(t, "EvdMdR")
        dp_st = subroutine_body(t, "EvdPdr")
        check_derivatives(dm_st + dp_st, mono, poly, "dmdr", "dpdr", "dmsdr", "rm", "p")
        out[key] = dict(mono=mono, poly=poly, basis=basis, nvar=6)
    # N3 linear coefficients (inline array C(276))
    t = read(os.path.join(ref, "src/PESs/N3_UMN_PES_Class.F90"))
    g = re.search(r"dimension\(276\)\s*,parameter\s*::\s*C\s*=\s*\(/(.*?)/\)", t, re.S | re.I)
    nums = re.findall(r"[-+]?\d+\.\d*D[-+]?\d+", g.group(1), re.I)
    assert len(nums) == 276, len(nums)
    out["N3_C"] = [float(x.replace("D", "e").replace("d", "e")) for x in nums]
    out["N3_C_text"] = nums
    # N4 UMN (N2 + N2): the same N4 PIP routines with its own inline coefficients
    t = read(os.path.join(ref, "src/PESs/N4_UMN_PES_Class.F90"))
    for sub in ("EvMono", "EvPoly", "evbas"):
        assert subroutine_body(t, sub) == subroutine_body(read(os.path.join(ref, "src/PESs/N3_UMN_PES_Class.F90")),
                                                            sub), "N4 UMN %s differs from the N3 file's" % sub
    g = re.search(r"dimension\(276\)\s*,parameter\s*::\s*C\s*=\s*\(/(.*?)/\)", t, re.S | re.I)
    nums = re.findall(r"[-+]?\d+\.\d*D[-+]?\d+", g.group(1), re.I)
    assert len(nums) == 276, len(nums)
    out["N4_C_text"] = nums
    # N4 UMN PIPNN: its bemsav49 (evmono49 + evpoly49) and bmx2b109 build the same 276 basis functions
    # from exp(-r / 1 Ang) (N4_UMN_PIPNN_PES_Class.F90:1004-1466, 1753-1830)
    t = read(os.path.join(ref, "src/PESs/N4_UMN_PIPNN_PES_Class.F90"))
    mono = parse_monomials(subroutine_body(t, "evmono49"), "m", "x")
    poly = parse_polynomials(subroutine_body(t, "evpoly49"), "p", "m")
    basis = parse_basis(subroutine_body(t, "bmx2b109"), "bm2", "bm1", len(poly))
    assert (mono, poly, basis) == (out["N4"]["mono"], out["N4"]["poly"], out["N4"]["basis"]), \
        "N4 UMN PIPNN basis differs from the N4 PIP"
    return out


# ----------------------------------------------------------------------------------------------
# Emitters
# ----------------------------------------------------------------------------------------------
def emit_oracle_header(S, path):
    L = ["/* Generated by coarseair_gb300/csrc/gen/gen_pip.py from the CoarseAIR UMN surface sources.",
         " * PIP tables: monomials (op 0 = one, 1 = MEG variable, 2 = product), polynomials",
         " * (op 0 = sum of monomials, 1 = product of two polynomials minus a list), basis map.",
         " * Do not edit by hand. */",
         "#ifndef CAIR_PIP_TABLES_H", "#define CAIR_PIP_TABLES_H", ""]
    for key in ("O3", "N4", "O4"):
        s = S[key]
        mono, poly, basis = s["mono"], s["poly"], s["basis"]
        mo, ma, mb = [], [], []
        for t in mono:
            if t[0] == "one":
                mo.append(0); ma.append(0); mb.append(0)
            elif t[0] == "var":
                mo.append(1); ma.append(t[1]); mb.append(0)
            else:
                mo.append(2); ma.append(t[1]); mb.append(t[2])
        po, pa, pb, off, ln, lst = [], [], [], [], [], []
        for t in poly:
            off.append(len(lst))
            if t[0] == "sum":
                po.append(0); pa.append(0); pb.append(0); lst.extend(t[1]); ln.append(len(t[1]))
            else:
                po.append(1); pa.append(t[1]); pb.append(t[2]); lst.extend(t[3]); ln.append(len(t[3]))
        def arr(name, vals, ty="short"):
            rows = []
            for i in range(0, len(vals), 24):
                rows.append("  " + ",".join(str(v) for v in vals[i:i + 24]))
            return "static const %s %s[%d] = {\n%s\n};" % (ty, name, len(vals), ",\n".join(rows))
        p = "pip_%s_" % key.lower()
        L.append("/* %s: %d monomials, %d polynomials, %d basis functions */" % (key, len(mono), len(poly), len(basis)))
        L.append("#define PIP_%s_NMONO %d" % (key, len(mono)))
        L.append("#define PIP_%s_NPOLY %d" % (key, len(poly)))
        L.append("#define PIP_%s_NBASIS %d" % (key, len(basis)))
        L.append("#define PIP_%s_NLIST %d" % (key, len(lst)))
        for name, vals in (("mono_op", mo), ("mono_a", ma), ("mono_b", mb), ("poly_op", po), ("poly_a", pa),
                           ("poly_b", pb), ("poly_off", off), ("poly_len", ln), ("poly_list", lst), ("basis", basis)):
            L.append(arr(p + name, vals))
        L.append("")
    L.append("#endif")
    with open(path, "w") as f:
        f.write("\n".join(L) + "\n")


class Emitter:
    """Straight-line FP64 code with exact-zero pruning.

    Values are symbolic: None means "exactly zero" (the term drops out), otherwise
    a C expression naming a temporary.  The order of every remaining operation is
    the reference's left-to-right order, so pruning changes no rounding step.
    """

    def __init__(self):
        self.lines = []
        self.nt = 0

    def tmp(self, expr):
        name = "t%d" % self.nt
        self.nt += 1
        self.lines.append("  const double %s = %s;" % (name, expr))
        return name

    @staticmethod
    def chain(terms):
        """Left-to-right chain of ('+'|'-', operand) with zeros dropped; returns expr or None."""
        expr = None
        for sign, x in terms:
            if x is None:
                continue
            if expr is None:
                expr = x if sign == "+" else "(-%s)" % x
            else:
                expr = "(%s %s %s)" % (expr, sign, x)
        return expr


def emit_device(S, key, name, zero_vars, dirs, path, coeff_symbol, value_only=False):
    """Device function computing V_poly = sum C_i B_i and dV/dvar_d for d in `dirs`.

    Signature: __device__ void name(const double x[NVAR], const double dx[NVAR],
                                   const double* C, double& V, double dV[len(dirs)])
    x = MEG variables, dx = their derivatives d x_i / d R_i (diagonal).
    """
    s = S[key]
    mono, poly, basis = s["mono"], s["poly"], s["basis"]
    if value_only:
        dirs = []
    E = Emitter()
    mv = []                       # monomial values
    md = {d: [] for d in dirs}    # monomial derivatives per direction
    for k, t in enumerate(mono):
        if t[0] == "one":
            mv.append("1.0")
            for d in dirs:
                md[d].append(None)
        elif t[0] == "var":
            v = t[1]
            mv.append(None if v in zero_vars else "x[%d]" % v)
            for d in dirs:
                md[d].append("dx[%d]" % v if (d == v and v not in zero_vars) else None)
        else:
            a, b = t[1], t[2]
            va, vb = mv[a], mv[b]
            val = None if (va is None or vb is None) else E.tmp("%s * %s" % (va, vb))
            mv.append(val)
            for d in dirs:
                da, db = md[d][a], md[d][b]
                t1 = None if (da is None or vb is None) else "%s * %s" % (da, vb)
                t2 = None if (va is None or db is None) else "%s * %s" % (va, db)
                e = E.chain([("+", t1), ("+", t2)])
                md[d].append(None if e is None else E.tmp(e))
    pv = []
    pd = {d: [] for d in dirs}
    for k, t in enumerate(poly):
        if t[0] == "sum":
            e = E.chain([("+", mv[x]) for x in t[1]])
            if e is not None and e == mv[t[1][0]] and len(t[1]) == 1:
                pv.append(e)
            else:
                pv.append(None if e is None else E.tmp(e))
            for d in dirs:
                e = E.chain([("+", md[d][x]) for x in t[1]])
                pd[d].append(None if e is None else (e if e.startswith("t") or e.startswith("dx") else E.tmp(e)))
        else:
            a, b, subs = t[1], t[2], t[3]
            va, vb = pv[a], pv[b]
            lead = None if (va is None or vb is None) else "%s * %s" % (va, vb)
            e = E.chain([("+", lead)] + [("-", pv[c]) for c in subs])
            pv.append(None if e is None else E.tmp(e))
            for d in dirs:
                da, db = pd[d][a], pd[d][b]
                t1 = None if (da is None or vb is None) else "%s * %s" % (da, vb)
                t2 = None if (va is None or db is None) else "%s * %s" % (va, db)
                e = E.chain([("+", t1), ("+", t2)] + [("-", pd[d][c]) for c in subs])
                pd[d].append(None if e is None else E.tmp(e))
    # V = sum_i C_i * B_i (left to right, the caller adds the leading constant)
    vt = [("+", None if pv[j] is None else "%s[%d] * %s" % (coeff_symbol, i, pv[j])) for i, j in enumerate(basis)]
    live_v = sum(1 for _, x in vt if x is not None)
    body = list(E.lines)
    out = []
    nflop = sum(l.count("*") + l.count(" + ") + l.count(" - ") + l.count("(-") for l in E.lines)
    nflop += 2 * live_v * (1 + len(dirs))
    out.append("/* %s: %d live basis terms of %d, %d temporaries, %d FP64 operations. Generated, do not edit. */" %
               (name, live_v, len(basis), E.nt, nflop))
    out.append("#define %s_FLOPS %d" % (name.upper(), nflop))
    if value_only:
        out.append("__device__ __forceinline__ void %s(const double* __restrict__ x," % name)
        out.append("    const double* __restrict__ %s, double V0, double& V) {" % coeff_symbol)
    else:
        out.append("__device__ __forceinline__ void %s(const double* __restrict__ x, const double* __restrict__ dx," % name)
        out.append("    const double* __restrict__ %s, double V0, double& V, double* __restrict__ dV) {" % coeff_symbol)
    out.extend(body)
    acc = "V0"
    out.append("  double v = V0;")
    for sgn, x in vt:
        if x is not None:
            out.append("  v = v + %s;" % x)
    out.append("  V = v;")
    for n, d in enumerate(dirs):
        out.append("  double g%d = 0.0;" % n)
        for i, j in enumerate(basis):
            if pd[d][j] is not None:
                out.append("  g%d = g%d + %s[%d] * %s;" % (n, n, coeff_symbol, i, pd[d][j]))
        out.append("  dV[%d] = g%d;" % (n, n))
    out.append("}")
    mode = "a" if value_only else "w"
    with open(path, mode) as f:
        f.write("\n".join(out) + "\n")
    return live_v, E.nt, nflop


def emit_device_basis(S, key, name, path):
    """Device function writing the basis functions themselves, b[i] = B_{i+1} for i < nbasis, from
    the variables x, in the value function's rounding order (EvMono/EvPoly, then the basis map).
    Signature: __device__ void name(const double x[NVAR], double b[NBASIS])."""
    s = S[key]
    mono, poly, basis = s["mono"], s["poly"], s["basis"]
    E = Emitter()
    mv = []
    for t in mono:
        if t[0] == "one":
            mv.append("1.0")
        elif t[0] == "var":
            mv.append("x[%d]" % t[1])
        else:
            mv.append(E.tmp("%s * %s" % (mv[t[1]], mv[t[2]])))
    pv = []
    for t in poly:
        if t[0] == "sum":
            e = E.chain([("+", mv[x]) for x in t[1]])
            pv.append(e if len(t[1]) == 1 else E.tmp(e))
        else:
            a, b, subs = t[1], t[2], t[3]
            pv.append(E.tmp(E.chain([("+", "%s * %s" % (pv[a], pv[b]))] + [("-", pv[c]) for c in subs])))
    nflop = sum(l.count("*") + l.count(" + ") + l.count(" - ") for l in E.lines)
    out = ["/* %s: %d basis functions, %d temporaries, %d FP64 operations. Generated, do not edit. */" %
           (name, len(basis), E.nt, nflop),
           "#define %s_FLOPS %d" % (name.upper(), nflop),
           "__device__ __forceinline__ void %s(const double* __restrict__ x, double* __restrict__ b) {" % name]
    out.extend(E.lines)
    for i, j in enumerate(basis):
        out.append("  b[%d] = %s;" % (i, pv[j]))
    out.append("}")
    with open(path, "a") as f:
        f.write("\n".join(out) + "\n")
    return len(basis), E.nt, nflop


def emit_device_reverse(S, key, name, zero_vars, dirs, path, coeff_symbol):
    """Energy and gradient with a reverse-mode (adjoint) sweep over the PIP graph.

    Forward: the pruned monomial and polynomial values (as the value-only function).
    Reverse: adjoints seeded with the linear coefficients C_i on the basis polynomials and
    propagated through p_k = p_a p_b - sum p_c (adj_a += adj_k p_b, adj_b += adj_k p_a,
    adj_c -= adj_k) and the monomial products down to the MEG variables; dV/dvar_d is the
    MEG variable's adjoint times dx_d.  Nodes that are exactly zero (pinned pairs) and terms
    whose factor is exactly zero are skipped.  Same signature as emit_device's function.
    """
    s = S[key]
    mono, poly, basis = s["mono"], s["poly"], s["basis"]
    L = []
    nt = [0]

    def tmp(expr):
        nm = "t%d" % nt[0]
        nt[0] += 1
        L.append("  const double %s = %s;" % (nm, expr))
        return nm

    flops = [0]
    # forward values
    mv = []
    for t in mono:
        if t[0] == "one":
            mv.append("1.0")
        elif t[0] == "var":
            mv.append(None if t[1] in zero_vars else "x[%d]" % t[1])
        else:
            a, b = mv[t[1]], mv[t[2]]
            if a is None or b is None:
                mv.append(None)
            else:
                mv.append(tmp("%s * %s" % (a, b)))
                flops[0] += 1
    pv = []
    for t in poly:
        if t[0] == "sum":
            terms = [mv[x] for x in t[1] if mv[x] is not None]
            if not terms:
                pv.append(None)
            elif len(terms) == 1:
                pv.append(terms[0])
            else:
                e = terms[0]
                for x in terms[1:]:
                    e = "(%s + %s)" % (e, x)
                flops[0] += len(terms) - 1
                pv.append(tmp(e))
        else:
            a, b, subs = pv[t[1]], pv[t[2]], t[3]
            lead = None if (a is None or b is None) else "%s * %s" % (a, b)
            chain = [("+", lead)] + [("-", pv[c]) for c in subs]
            e = Emitter.chain(chain)
            nterm = sum(1 for _, x in chain if x is not None)
            flops[0] += (1 if lead else 0) + max(0, nterm - 1)
            pv.append(None if e is None else tmp(e))
    # energy
    L.append("  double v = V0;")
    live = 0
    for i, j in enumerate(basis):
        if pv[j] is not None:
            L.append("  v = v + %s[%d] * %s;" % (coeff_symbol, i, pv[j]))
            live += 1
            flops[0] += 2
    L.append("  V = v;")
    # adjoint seeds: basis polynomials carry their coefficients
    adj_p = {}
    adj_m = {}
    decl = []

    def add_adj(table, k, expr, sign="+"):
        """adj[k] (+|-)= expr, declaring the variable at the first contribution."""
        nm = table.get(k)
        if nm is None:
            nm = ("ap%d" if table is adj_p else "am%d") % k
            table[k] = nm
            L.append("  double %s = %s%s;" % (nm, "" if sign == "+" else "-", expr))
        else:
            L.append("  %s = %s %s %s;" % (nm, nm, sign, expr))
            flops[0] += 1

    for i, j in enumerate(basis):
        if pv[j] is not None:
            add_adj(adj_p, j, "%s[%d]" % (coeff_symbol, i))
    for k in range(len(poly) - 1, -1, -1):
        if pv[k] is None or k not in adj_p:
            continue
        t = poly[k]
        ak = adj_p[k]
        if t[0] == "sum":
            for x in t[1]:
                if mv[x] is not None and mono[x][0] != "one":
                    add_adj(adj_m, x, ak)
        else:
            a, b, subs = t[1], t[2], t[3]
            if pv[a] is not None and pv[b] is not None:
                if a == b:
                    add_adj(adj_p, a, "(2.0 * %s) * %s" % (ak, pv[b]))
                    flops[0] += 2
                else:
                    add_adj(adj_p, a, "%s * %s" % (ak, pv[b]))
                    add_adj(adj_p, b, "%s * %s" % (ak, pv[a]))
                    flops[0] += 2
            for c in subs:
                if pv[c] is not None:
                    add_adj(adj_p, c, ak, sign="-")
    gsum = {d: None for d in dirs}
    for k in range(len(mono) - 1, -1, -1):
        if mv[k] is None or k not in adj_m:
            continue
        t = mono[k]
        ak = adj_m[k]
        if t[0] == "mul":
            a, b = t[1], t[2]
            if a == b:
                add_adj(adj_m, a, "(2.0 * %s) * %s" % (ak, mv[b]))
                flops[0] += 2
            else:
                add_adj(adj_m, a, "%s * %s" % (ak, mv[b]))
                add_adj(adj_m, b, "%s * %s" % (ak, mv[a]))
                flops[0] += 2
        elif t[0] == "var" and t[1] in dirs:
            d = t[1]
            if gsum[d] is None:
                gsum[d] = ak
            else:
                gsum[d] = "(%s + %s)" % (gsum[d], ak)
                flops[0] += 1
    for n, d in enumerate(dirs):
        L.append("  dV[%d] = %s * dx[%d];" % (n, gsum[d] if gsum[d] else "0.0", d))
        flops[0] += 1
    out = ["/* %s: reverse-mode gradient, %d live basis terms of %d, %d FP64 operations. Generated, do not edit. */"
           % (name, live, len(basis), flops[0]),
           "#define %s_FLOPS %d" % (name.upper(), flops[0]),
           "__device__ __forceinline__ void %s(const double* __restrict__ x, const double* __restrict__ dx," % name,
           "    const double* __restrict__ %s, double V0, double& V, double* __restrict__ dV) {" % coeff_symbol]
    out += L
    out.append("}")
    with open(path, "a") as f:
        f.write("\n".join(out) + "\n")
    return live, nt[0], flops[0]


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("COARSEAIR_REF", "")
    if not ref or not os.path.isdir(ref):
        sys.exit("usage: gen_pip.py <CoarseAIR source tree>")
    S = load_surfaces(ref)
    emit_oracle_header(S, os.path.join(REPO, "oracle", "pip_tables.h"))
    gen = os.path.join(REPO, "coarseair_gb300", "csrc", "generated")
    os.makedirs(gen, exist_ok=True)
    # N3 on the N4 PIP: MEG variables 3, 5, 6 (0-based 2, 4, 5) belong to the pinned pairs
    info = emit_device(S, "N4", "pip_n3_eval", zero_vars={2, 4, 5}, dirs=[0, 1, 3],
                       path=os.path.join(gen, "pip_n3.cuh"), coeff_symbol="C")
    print("N3 pruned:", info)
    info = emit_device(S, "N4", "pip_n3_value", zero_vars={2, 4, 5}, dirs=[0, 1, 3],
                       path=os.path.join(gen, "pip_n3.cuh"), coeff_symbol="C", value_only=True)
    print("N3 pruned value:", info)
    info = emit_device_reverse(S, "N4", "pip_n3_eval_rev", zero_vars={2, 4, 5}, dirs=[0, 1, 3],
                               path=os.path.join(gen, "pip_n3.cuh"), coeff_symbol="C")
    print("N3 pruned reverse:", info)
    info = emit_device(S, "O3", "pip_o3_eval", zero_vars=set(), dirs=[0, 1, 2],
                       path=os.path.join(gen, "pip_o3.cuh"), coeff_symbol="C")
    print("O3:", info)
    info = emit_device(S, "O3", "pip_o3_value", zero_vars=set(), dirs=[0, 1, 2],
                       path=os.path.join(gen, "pip_o3.cuh"), coeff_symbol="C", value_only=True)
    print("O3 value:", info)
    info = emit_device_reverse(S, "O3", "pip_o3_eval_rev", zero_vars=set(), dirs=[0, 1, 2],
                               path=os.path.join(gen, "pip_o3.cuh"), coeff_symbol="C")
    print("O3 reverse:", info)
    # O4 on its own PIP (six MEG variables, all live): energy and adjoint-sweep gradient only
    o4 = os.path.join(gen, "pip_o4.cuh")
    with open(o4, "w") as f:
        f.write("/* O4 UMN PIP (O4_UMN_PES_Class.F90 EvMono/EvPoly/evbas). Generated by gen_pip.py, do not edit. */\n")
    info = emit_device(S, "O4", "pip_o4_value", zero_vars=set(), dirs=[], path=o4, coeff_symbol="C",
                       value_only=True)
    print("O4 value:", info)
    info = emit_device_reverse(S, "O4", "pip_o4_eval_rev", zero_vars=set(), dirs=[0, 1, 2, 3, 4, 5], path=o4,
                               coeff_symbol="C")
    print("O4 reverse:", info)
    # N4 UMN on the full N4 PIP (all six MEG variables live): energy and adjoint-sweep gradient
    n4 = os.path.join(gen, "pip_n4.cuh")
    with open(n4, "w") as f:
        f.write("/* N4 UMN PIP (N4_UMN_PES_Class.F90 EvMono/EvPoly/evbas). Generated by gen_pip.py, do not edit. */\n")
    info = emit_device(S, "N4", "pip_n4_value", zero_vars=set(), dirs=[], path=n4, coeff_symbol="C",
                       value_only=True)
    print("N4 value:", info)
    info = emit_device_reverse(S, "N4", "pip_n4_eval_rev", zero_vars=set(), dirs=[0, 1, 2, 3, 4, 5], path=n4,
                               coeff_symbol="C")
    print("N4 reverse:", info)
    # N4 UMN PIPNN: the basis functions themselves, the networks' input
    nn = os.path.join(gen, "pip_n4nn.cuh")
    with open(nn, "w") as f:
        f.write("/* N4 PIP basis for the N4 UMN PIPNN networks (N4_UMN_PIPNN_PES_Class.F90 bemsav49/bmx2b109, the\n"
                " * same tables as N4_UMN_PES_Class.F90 EvMono/EvPoly/evbas). Generated by gen_pip.py, do not edit. */\n")
    info = emit_device_basis(S, "N4", "pip_n4_basis", path=nn)
    print("N4 basis:", info)
    # the N3 surface is this fit with three pairs pinned: one coefficient file serves both
    assert S["N4_C_text"] == S["N3_C_text"], "N4 UMN coefficients differ from the N3 UMN ones"
    with open(os.path.join(REPO, "coarseair_gb300", "data", "N3_UMN.dat"), "w") as f:
        f.write("# N3 UMN surface (N4 PIP, MEG variables): 276 linear coefficients [kcal/mol]\n")
        f.write("# a = 1.0 Ang, ab = 1.5 Ang^2, re = 1.098 Ang, totdiss = 457.4 kcal/mol\n")
        for x in S["N3_C_text"]:
            f.write(x.replace("D", "e").replace("d", "e") + "\n")
    for key in ("O3", "N4", "O4"):
        s = S[key]
        print(key, len(s["mono"]), len(s["poly"]), len(s["basis"]))
    # the same tables as data, for the lane-parallel program generator (gen_warp.py)
    import json
    with open(os.path.join(gen, "pip_tables.json"), "w") as f:
        json.dump({key: {k: S[key][k] for k in ("mono", "poly", "basis", "nvar")} for key in ("O3", "N4", "O4")},
                  f, separators=(",", ":"))
        f.write("\n")


if __name__ == "__main__":
    main()
