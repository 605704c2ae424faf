"""System descriptions for the trajectory path: surfaces, masses, integrator and final-state
parameters, level lists.

This module reads the same data the reference reads at start-up:

* O3 UMN surfaces: ``dtb/Systems/O3/PESs/<Model>.inp`` (O3_UMN_PES_Class.F90:114-131): a title
  line, then ``a ab ra rb`` and ``C(1:56)`` in list-directed format;
* O4 UMN surfaces: ``dtb/Systems/O4/PESs/UMN/<Model>.dat`` (O4_UMN_PES_Class.F90:179-203):
  ``a, ab, ra, rb, Eref, totdiss``, 143 lines of three coefficients, then ``C(430)``;
* N3 UMN: the 276 coefficients the reference keeps inline (N3_UMN_PES_Class.F90:108-201),
  stored here as ``data/N3_UMN.dat``;
* O3 NN surfaces: ``dtb/Systems/O3/PESs/NN/<Model>/<NHL1>_<NHL2>/`` (O3_NN_PES_Class.F90:74-232):
  ``ScalingValues.csv`` and ``CalibratedParams/{Lambda,re,W1,b1,W2,b2,W3,b3}.csv``;
* N4 UMN PIPNN: ``dtb/Systems/N4/PESs/UMN_PIPNN/{Weights,Biases}.dat``
  (N4_UMN_PIPNN_PES_Class.F90:176-330), three networks read in list-directed format;
* O3 BNN posterior samples: ``dtb/Systems/O3/PESs/BNN/<Folder>/`` (BNN_PES_Class.F90:95-200,
  686-770): ``ScalingValues.csv`` and ``CalibratedParams/<name>.csv.<sample>``, packed one line per
  sample into ``data/O3_BNN/<Folder>/samples.csv.gz`` by ``data/O3_BNN/pack_samples.py``;
* level lists ``vqn jqn eint egam rmin rmax vmin vmax tau ri ro`` (LevelsContainer_Class.F90).

and fills the input-file keys of the hot path with the values of the reference's own input
templates (input/O3/UMN/input/CoarseAIR.inp, input/N3/UMN/input/CoarseAIR.inp).
"""
import gzip
import os
import re
from dataclasses import dataclass

import numpy as np

DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")

AMU_TO_AU = 1822.888486209          # [amu] -> electron masses (kgm_To_au / 1000)
PES_O3_UMN, PES_N3_UMN, PES_O4_UMN, PES_O3_NN, PES_N4_UMN, PES_O3_BNN, PES_N4_PIPNN = 1, 2, 3, 4, 5, 6, 7
DIAT_O2_UMN, DIAT_N2_UMN_FORN4, DIAT_N2_UMN_PIPNN_FORN4 = 1, 2, 3

_FNUM = re.compile(r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[dDeE][-+]?\d+)?")


def _fortran_floats(text):
    return [float(x.replace("d", "e").replace("D", "e")) for x in _FNUM.findall(text)]


@dataclass
class Surface:
    model: int
    coef: np.ndarray
    a: float = 0.0
    ab: float = 0.0
    ra: float = 0.0
    rb: float = 0.0
    eref: float = 0.0
    totdiss: float = 0.0
    name: str = ""


def load_o3_umn(model="UMN_11A1"):
    """O3_UMN_PES_Class.F90:114-131."""
    with open(os.path.join(DATA, "O3_UMN", model + ".inp")) as f:
        lines = f.read().split("\n")
    vals = _fortran_floats("\n".join(lines[1:]))
    a, ab, ra, rb = vals[:4]
    coef = np.array(vals[4:60], dtype=np.float64)
    assert coef.size == 56
    return Surface(PES_O3_UMN, coef, a, ab, ra, rb, name="O3 " + model)


def load_o4_umn(model="UMN_Singlet"):
    """O4_UMN_PES_Class.F90:179-203."""
    with open(os.path.join(DATA, "O4_UMN", model + ".dat")) as f:
        vals = _fortran_floats(f.read())
    a, ab, ra, rb, eref, totdiss = vals[:6]
    coef = np.array(vals[6:436], dtype=np.float64)
    assert coef.size == 430
    return Surface(PES_O4_UMN, coef, a, ab, ra, rb, eref, totdiss, name="O4 " + model)


def load_n3_umn():
    """N3_UMN_PES_Class.F90:96-201 (a = 1 Ang, ab = 1.5 Ang^2, re = 1.098 Ang, totdiss = 457.4)."""
    with open(os.path.join(DATA, "N3_UMN.dat")) as f:
        vals = [float(l) for l in f if l.strip() and not l.startswith("#")]
    coef = np.array(vals, dtype=np.float64)
    assert coef.size == 276
    return Surface(PES_N3_UMN, coef, 1.0, 1.5, 1.098, 1.098, 0.0, 457.4, name="N3 UMN")


LEVEL_COLS = ("vqn", "jqn", "eint", "egam", "rmin", "rmax", "vmin", "vmax", "tau", "ri", "ro")


def load_o3_nn(model="NN_11A1_MPE", hidden=(20, 10)):
    """O3 NN surface as the reference reads it (O3_NN_PES_Class.F90:139-230), packed into one
    coefficient array: NHL1, NHL2, Lambda, re, Scaling_MEAN(3), Scaling_SD(3), y_Scaling,
    W1(6, NHL1), b1, W2(NHL1, NHL2), b2, W3, b3, matrices column-major."""
    h1, h2 = hidden
    d = os.path.join(DATA, "O3_NN", model, "%d_%d" % (h1, h2))
    cp = os.path.join(d, "CalibratedParams")

    def rows(name):
        with open(os.path.join(cp, name)) as f:
            return [[float(x) for x in ln.replace(",", " ").split()] for ln in f if ln.strip()]

    with open(os.path.join(d, "ScalingValues.csv")) as f:
        lines = [ln for ln in f.read().splitlines() if ln.strip()]
    mean = [float(x) for x in lines[1].split(",")]
    sd = [float(x) for x in lines[2].split(",")]
    ysc = float(lines[3].split(",")[0])
    lam, re_ = rows("Lambda.csv")[0][0], rows("re.csv")[0][0]
    W1 = np.array(rows("W1.csv"))                  # row i = W1(i, 1:NHL1)
    W2 = np.array(rows("W2.csv"))                  # row i = W2(i, 1:NHL2)
    b1 = np.array(rows("b1.csv")).ravel()
    b2 = np.array(rows("b2.csv")).ravel()
    W3 = np.array(rows("W3.csv")).ravel()
    b3 = rows("b3.csv")[0][0]
    assert W1.shape == (6, h1) and W2.shape == (h1, h2) and b1.size == h1 and b2.size == h2 and W3.size == h2
    coef = np.concatenate([[h1, h2, lam, re_], mean, sd, [ysc], W1.ravel(order="F"), b1, W2.ravel(order="F"),
                           b2, W3, [b3]]).astype(np.float64)
    assert coef.size == 12 + 7 * h1 + h1 * h2 + 2 * h2
    return Surface(PES_O3_NN, coef, name="O3 " + model)


def _bnn_samples(folder):
    with gzip.open(os.path.join(DATA, "O3_BNN", folder, "samples.csv.gz"), "rt") as f:
        rows = [ln.split(",") for ln in f.read().splitlines() if ln.strip() and not ln.startswith("#")]
    return {int(r[0]): [float(x) for x in r[1:]] for r in rows}


def load_o3_bnn(sample, folder="PES9_Case2_LHS50"):
    """One posterior sample of the O3 BNN surface as ReadParamPost_BNN reads it
    (BNN_PES_Class.F90:686-770) with the folder's ScalingValues.csv, packed like load_o3_nn with
    the sample's Noise appended."""
    v = _bnn_samples(folder)[int(sample)]
    h1, h2 = int(v[0]), int(v[1])
    lam, re_, noise, b3 = v[2:6]
    q = 6
    W1 = np.array(v[q:q + 6 * h1]).reshape(6, h1); q += 6 * h1
    b1 = np.array(v[q:q + h1]); q += h1
    W2 = np.array(v[q:q + h1 * h2]).reshape(h1, h2); q += h1 * h2
    b2 = np.array(v[q:q + h2]); q += h2
    W3 = np.array(v[q:q + h2]); q += h2
    assert q == len(v)
    with open(os.path.join(DATA, "O3_BNN", folder, "ScalingValues.csv")) as f:
        lines = [ln for ln in f.read().splitlines() if ln.strip()]
    mean = [float(x) for x in lines[1].split(",")]
    sd = [float(x) for x in lines[2].split(",")]
    ysc = float(lines[3].split(",")[0])
    coef = np.concatenate([[h1, h2, lam, re_], mean, sd, [ysc], W1.ravel(order="F"), b1, W2.ravel(order="F"),
                           b2, W3, [b3, noise]]).astype(np.float64)
    return Surface(PES_O3_BNN, coef, name="O3 BNN %s sample %d" % (folder, sample))


class _ListDirected:
    """Fortran list-directed reads over a file's records: every READ starts on a new record and
    drops what is left of its last record."""

    def __init__(self, path):
        with open(path) as f:
            self.lines = f.read().split("\n")
        self.pos = 0

    def skip(self):
        self.pos += 1

    def read(self, n):
        vals = []
        while len(vals) < n:
            if self.pos >= len(self.lines):
                raise ValueError("end of file")
            vals += _fortran_floats(self.lines[self.pos])
            self.pos += 1
        return vals[:n]


# PES_Factory_Class.F90:276-296: the PES model string selects the networks averaged
PIPNN_VARIANTS = {"UMN_PIPNN": (1, 1, 1), "UMN_PIPNN_A": (1, 0, 0), "UMN_PIPNN_B": (0, 1, 0),
                  "UMN_PIPNN_C": (0, 0, 1)}


def load_n4_pipnn(model="UMN_PIPNN"):
    """N4 UMN PIPNN as Initialize_N4_UMN_PIPNN_PES reads it (N4_UMN_PIPNN_PES_Class.F90:176-330): per
    network a title record in each file, NInput NHid NOutput, the hidden layer sizes, iFunc NWe,
    pdel(NScale), pavg(NScale), then for every node of every layer its weights, one per record, from
    Weights.dat and its bias from Biases.dat.  The three networks share one set of layer sizes and one
    iFunc (each read overwrites the last).  Packed as UseSurface(3), iFunc, NInput, NHid1, NHid2,
    NOutput, then per network pdel, pavg, W1(NInput, NHid1), b1, W2(NHid1, NHid2), b2, W3, b3."""
    use = PIPNN_VARIANTS[model]
    d = os.path.join(DATA, "N4_PIPNN")
    W, B = _ListDirected(os.path.join(d, "Weights.dat")), _ListDirected(os.path.join(d, "Biases.dat"))
    nets, shape = [], None
    for _ in range(3):
        B.skip()
        W.skip()
        nin, nhid, nout = (int(x) for x in W.read(3))
        nodes = [nin] + [int(x) for x in W.read(nhid)] + [nout]
        ifunc, nwe = (int(x) for x in W.read(2))
        pdel, pavg = W.read(nin + nout), W.read(nin + nout)
        layers, iwe = [], 0
        for l in range(1, len(nodes)):
            w = np.zeros((nodes[l - 1], nodes[l]))
            b = np.zeros(nodes[l])
            for j in range(nodes[l]):
                for i in range(nodes[l - 1]):
                    w[i, j] = W.read(1)[0]
                    iwe += 1
                b[j] = B.read(1)[0]
                iwe += 1
            layers.append((w, b))
        if iwe != nwe:
            raise ValueError("N4 PIPNN: %d parameters read, the file gives %d" % (iwe, nwe))
        if nhid != 2 or nout != 1:
            raise ValueError("N4 PIPNN: two hidden layers and one output are built")
        nets.append(np.concatenate([pdel, pavg] + [np.concatenate([w.ravel(order="F"), b]) for w, b in layers]))
        shape = (ifunc, nin, nodes[1], nodes[2], nout)
    coef = np.concatenate([np.array(use + shape, dtype=np.float64)] + nets)
    return Surface(PES_N4_PIPNN, coef, name="N4 " + model)


def load_levels(name):
    """Level list as a structured array (columns LEVEL_COLS)."""
    fn = {"N2": "N2_UMN_ForN4_FromRoss.inp.gz", "O2": "O2_UMN_FromUMN_Sorted.inp.gz"}[name]
    rows = []
    with gzip.open(os.path.join(DATA, "levels", fn), "rt") as f:
        for line in f:
            s = line.strip()
            if not s or s.startswith("#"):
                continue
            rows.append([float(x.replace("D", "E")) for x in s.split()])
    arr = np.array(rows, dtype=np.float64)
    out = np.zeros(arr.shape[0], dtype=[(c, "f8") for c in LEVEL_COLS] + [("rlim", "f8")])
    for i, c in enumerate(LEVEL_COLS):
        out[c] = arr[:, i]
    return out


@dataclass
class SystemConfig:
    """The hot-path subset of the reference's input file, plus the surfaces."""
    name: str
    natoms: int
    masses: tuple
    surfaces: list
    diat_model: int
    dt0: float = 5.0                # "Initial time step"
    eps: float = 1.0e-8             # "Error control parameter"
    relax: float = 0.5              # "Stepsize increase damping factor"
    nsteps: int = 3                 # "Nb of extrapolation steps"
    inc_step: int = 1               # "Try to increase stepsize?"
    ncall: int = 10                 # "Nb of integration between end checking"
    rmax: float = 16.0              # "Max distance between atom pair [bohr]"
    tmax: float = 4.0e5             # "Max trajectory time [a.u.]"
    ham_abs_tol: float = 1.0e-5     # "Tolerance on Hamiltonian" (Input_Class.F90:227 default)
    nquad: int = 50                 # "Nb of Quadrature Pts for Action Integral"
    rsmal: float = 1.0              # "Lower Bound for Position of Centrifugal Barrier Max"
    rcent: float = 30.0             # "Upper Bound for Position of Centrifugal Barrier Max"
    rfact: float = 0.0              # "Factor for q.b. Levels"
    tthresau: float = 1.0e-100      # "Time threshold for q.b. Levels [Eh]"
    max_attempts: int = 1000000     # IterMax (1e5) x ncall (Integrator_Class.F90:269)
    ttra: float = 10000.0           # "Translational Temperature [K] 1"
    bmax: float = 6.0               # impact-parameter ring bound (Circles, one ring)
    dinit: float = 15.0             # "Initial Distance between Target and Projectile"
    seed: int = 1                   # "Initial Random Nb Seed"
    degeneracy: tuple = (1.0,)

    @property
    def neqtvar(self):
        return 3 * (self.natoms - 1)

    @property
    def neqttot(self):
        return 2 * self.neqtvar

    @property
    def npairs(self):
        return self.natoms * (self.natoms - 1) // 2


def o3_config(model="UMN_11A1", mass_amu=15.9994, **kw):
    """O2 + O on one O3 UMN surface (the ground state UMN_11A1 by default)."""
    m = mass_amu * AMU_TO_AU
    return SystemConfig("O2+O " + model, 3, (m, m, m), [load_o3_umn(model)], DIAT_O2_UMN, **kw)


# input/O3/UMN/input/CoarseAIR.inp:116-134: the nine O3 UMN surfaces and their degeneracies
O3_MIX = (("UMN_11A1", 1.0), ("UMN_11A2", 1.0), ("UMN_13A1", 3.0), ("UMN_13A2", 3.0), ("UMN_15A1", 5.0),
          ("UMN_15A2", 5.0), ("UMN_21A1", 1.0), ("UMN_23A1", 3.0), ("UMN_25A1", 5.0))


def o3_mix_config(mass_amu=15.9994, **kw):
    """O2 + O on the nine O3 UMN surfaces of the reference's O3 input, degeneracies 1/1/3/3/5/5/1/3/5."""
    m = mass_amu * AMU_TO_AU
    return SystemConfig("O2+O UMN 9 surfaces", 3, (m, m, m), [load_o3_umn(name) for name, _ in O3_MIX], DIAT_O2_UMN,
                        degeneracy=tuple(d for _, d in O3_MIX), **kw)


def o3nn_config(model="NN_11A1_MPE", mass_amu=15.9994, **kw):
    """O2 + O on an O3 NN surface with the O2 UMN diatomic."""
    m = mass_amu * AMU_TO_AU
    return SystemConfig("O2+O " + model, 3, (m, m, m), [load_o3_nn(model)], DIAT_O2_UMN, **kw)


def o3bnn_config(samples=range(1, 51), folder="PES9_Case2_LHS50", mass_amu=15.9994, **kw):
    """O2 + O on the O3 BNN with the O2 UMN diatomic, one surface per posterior sample
    ("Nb of PESs Samples"; with "Initial Random Nb Seed for PES Parameters Sampling = 0" sample i
    is file .i, Collision_Class.F90:383-394), degeneracy one each (Input_Class.F90:905-923)."""
    m = mass_amu * AMU_TO_AU
    surfs = [load_o3_bnn(i, folder) for i in samples]
    return SystemConfig("O2+O BNN " + folder, 3, (m, m, m), surfs, DIAT_O2_UMN, degeneracy=(1.0,) * len(surfs), **kw)


def n3_config(mass_amu=14.0067, **kw):
    """N2 + N on the N3 UMN surface (N4 PIP) with the UMN_ForN4 N2 diatomic."""
    m = mass_amu * AMU_TO_AU
    kw.setdefault("bmax", 7.0)
    return SystemConfig("N2+N UMN", 3, (m, m, m), [load_n3_umn()], DIAT_N2_UMN_FORN4, **kw)


def load_n4_umn():
    """N4 UMN (N4_UMN_PES_Class.F90): the N4 PIP on all six pairs with the same 276 coefficients as N3 UMN."""
    n3 = load_n3_umn()
    return Surface(PES_N4_UMN, n3.coef, 1.0, 1.5, 1.098, 1.098, 0.0, 457.4, name="N4 UMN")


def n4_config(mass_amu=14.0067, **kw):
    """N2 + N2 on the N4 UMN surface with the UMN_ForN4 N2 diatomic (Dinit 23 bohr and Stratified rings
    up to 8 bohr as input/N4/UMN/input/CoarseAIR_VS_UMNDiat.inp; one ring of 8 bohr here)."""
    m = mass_amu * AMU_TO_AU
    kw.setdefault("bmax", 8.0)
    kw.setdefault("dinit", 23.0)
    kw.setdefault("rmax", 30.0)
    return SystemConfig("N2+N2 UMN", 4, (m, m, m, m), [load_n4_umn()], DIAT_N2_UMN_FORN4, **kw)


def n4pipnn_config(model="UMN_PIPNN", diat=DIAT_N2_UMN_FORN4, mass_amu=14.0067, **kw):
    """N2 + N2 on the N4 UMN PIPNN surface (input/N4/UMN_PIPNN/input/CoarseAIR_VS.inp: Dinit 23 bohr,
    rmax 30 bohr).  That input pairs it with the UMN_PIPNN_ForN4 diatomic, whose level list is not
    shipped; the level list here is the UMN_ForN4 one, so the default diatomic is UMN_ForN4."""
    m = mass_amu * AMU_TO_AU
    kw.setdefault("bmax", 8.0)
    kw.setdefault("dinit", 23.0)
    kw.setdefault("rmax", 30.0)
    return SystemConfig("N2+N2 " + model, 4, (m, m, m, m), [load_n4_pipnn(model)], diat, **kw)


def o4_config(mass_amu=15.9994, **kw):
    """O2 + O2 on the three O4 UMN surfaces (degeneracies 1/3/5, CoarseAIR_StS.inp)."""
    m = mass_amu * AMU_TO_AU
    kw.setdefault("bmax", 8.0)
    kw.setdefault("dinit", 18.0)
    kw.setdefault("rmax", 35.0)     # input/O4/UMN/input/CoarseAIR_StS.inp:228-229
    kw.setdefault("tmax", 5.0e5)
    surfs = [load_o4_umn(x) for x in ("UMN_Singlet", "UMN_Triplet", "UMN_Quintet")]
    return SystemConfig("O2+O2 UMN", 4, (m, m, m, m), surfs, DIAT_O2_UMN, degeneracy=(1.0, 3.0, 5.0), **kw)
