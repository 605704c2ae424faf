"""ctypes wrapper of the CPU oracle (liborc.so) -- TEST INFRASTRUCTURE ONLY.

The oracle is the checker for the CUDA library: the tests, the smoke check and the bench's
CPU-baseline leg use it.  The product never imports it.  See oracle.h for what it restates
and how it is pinned.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liborc.so")

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)


class OrcPes(C.Structure):
    _fields_ = [("model", C.c_int), ("ncoef", C.c_int), ("coef", _D), ("a", C.c_double), ("ab", C.c_double),
                ("ra", C.c_double), ("rb", C.c_double), ("eref", C.c_double), ("totdiss", C.c_double)]


class OrcSys(C.Structure):
    _fields_ = [("natoms", C.c_int), ("neqtvar", C.c_int), ("neqttot", C.c_int), ("npairs", C.c_int),
                ("mass", C.c_double * 4), ("mMiMn", C.c_double * 3), ("Tqp", C.c_double * 81),
                ("Tpq", C.c_double * 81), ("npes", C.c_int), ("pes", OrcPes * 64), ("diat", C.c_int),
                ("dt0", C.c_double), ("eps", C.c_double), ("relax", C.c_double), ("rmax", C.c_double),
                ("tmax", C.c_double), ("hamabstol", C.c_double), ("nsteps", C.c_int), ("incstpsz", C.c_int),
                ("ncall", C.c_int), ("nquad", C.c_int), ("rsmal", C.c_double), ("rcent", C.c_double),
                ("rfact", C.c_double), ("tthresau", C.c_double)]


class OrcRng(C.Structure):
    _fields_ = [("state", C.c_uint64), ("x", C.c_double * 100)]


class OrcLevel(C.Structure):
    _fields_ = [("vqn", C.c_int), ("jqn", C.c_int), ("eint", C.c_double), ("egam", C.c_double),
                ("rmin", C.c_double), ("rmax", C.c_double), ("vmin", C.c_double), ("vmax", C.c_double),
                ("tau", C.c_double), ("ri", C.c_double), ("ro", C.c_double), ("rlim", C.c_double)]


class OrcIcCfg(C.Structure):
    _fields_ = [("ttra", C.c_double), ("bmax", C.c_double), ("dinit", C.c_double), ("state_specific", C.c_int),
                ("b_mode", C.c_int), ("bmin", C.c_double)]


def impact_rings(ntrajtot, bring, ntring):
    """InitializeImpactParameter (src/Collision/ImpactParameter_Class.F90:55-160): iTrajMax of each
    ring for NTrajTot trajectories, NTraj = int(dfloat(Weight * NTrajTot) / SumAllWeight) with the
    remainder added to the first ring; with a negative weight every iTrajMax stays 0."""
    nr = len(bring)
    itrajmax = [0] * nr
    if any(w < 0 for w in ntring):
        return itrajmax
    sum_all = sum(ntring)
    ntraj = [int(float(w * ntrajtot) / sum_all) for w in ntring]
    if sum(ntraj) != ntrajtot:
        ntraj[0] = ntraj[0] + ntrajtot - sum(ntraj)
    acc = 0
    for r in range(nr):
        itrajmax[r] = acc + ntraj[r]
        acc = itrajmax[r]
    return itrajmax


def impact_ring_of(idx, bring, itrajmax):
    """GetImpactParamValue (ImpactParameter_Class.F90:202-221) for the 1-based trajectory idx:
    (bmin, b) of the first ring whose iTrajMax reaches idx; None when none does."""
    for r in range(len(bring)):
        if idx > itrajmax[r]:
            continue
        return (bring[r - 1] if r > 0 else 0.0), bring[r]
    return None


class OrcMol(C.Structure):
    _fields_ = [("ipair", C.c_int), ("itype", C.c_int), ("eint", C.c_double), ("angmom", C.c_double),
                ("viba", C.c_double)]


class OrcPoint(C.Structure):
    _fields_ = [("mol", OrcMol * 2), ("b", C.c_double), ("xkin", C.c_double), ("vrel", C.c_double * 3),
                ("nmol", C.c_int)]


def build(quiet=True):
    """Compile liborc.so with the committed Makefile (gcc, no FMA)."""
    r = subprocess.run(["make", "-C", HERE, "liborc.so"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        L.orc_sys_init.argtypes = [C.POINTER(OrcSys)]
        L.orc_diat_V.restype = C.c_double
        L.orc_diat_V.argtypes = [C.c_int, C.c_double]
        L.orc_diat_VdV.argtypes = [C.c_int, C.c_double, _D, _D]
        L.orc_pes_compute.argtypes = [C.POINTER(OrcSys), C.c_int, _D, _D, _D, _D, _D]
        L.orc_pes_potential.restype = C.c_double
        L.orc_pes_potential.argtypes = [C.POINTER(OrcSys), C.c_int, _D]
        L.orc_pip_eval.argtypes = [C.c_int, _D, _D, C.c_int, _D, C.c_double, _D, _D]
        L.orc_pes_scale.argtypes = [C.POINTER(OrcSys), C.c_int, _D, _D]
        L.orc_pip_basis.argtypes = [C.c_int, _D, _D, _D]
        L.orc_pipnn_net.restype = C.c_double
        L.orc_pipnn_net.argtypes = [_D, C.c_int, _D]
        L.orc_pipnn_kcal.restype = C.c_double
        L.orc_pipnn_kcal.argtypes = [_D, _D]
        L.orc_rp.argtypes = [C.POINTER(OrcSys), _D, _D, _D]
        _I64 = C.POINTER(C.c_int64)
        L.orc_sample_ic4.argtypes = [C.POINTER(OrcSys), C.POINTER(OrcRng), C.POINTER(OrcLevel), C.POINTER(OrcLevel),
                                     C.POINTER(OrcIcCfg), C.c_int, _D, _D, _D, _D, _D, _D]
        L.orc_statistics.argtypes = [C.c_int, C.c_int, _I, _I, C.c_int, _D, _D, _D, _D, C.c_int, _I64, _I, _I, _I64,
                                     _D, _D]
        L.orc_mean_velocity.argtypes = [C.c_double, C.c_double]
        L.orc_mean_velocity.restype = C.c_double
        L.orc_rhs.argtypes = [C.POINTER(OrcSys), C.c_int, _D, _D]
        L.orc_hamiltonian.argtypes = [C.POINTER(OrcSys), C.c_int, _D, _D, _D]
        L.orc_bs_attempts.argtypes = [C.POINTER(OrcSys), C.c_int, _I, _D, _D, _D, _D, C.c_int]
        L.orc_integrate.argtypes = [C.POINTER(OrcSys), C.c_int, _I, _D, _D, _D, _D, _D, _D, _D, _I, _I, _I,
                                    C.c_int64]
        L.orc_error_factor.argtypes = [C.POINTER(OrcSys), C.c_double, _D, _D]
        L.orc_apply_transformation.argtypes = [C.POINTER(OrcSys), _D, _D]
        L.orc_rng_seed.argtypes = [C.POINTER(OrcRng), C.c_int64]
        L.orc_rng_draw.restype = C.c_double
        L.orc_rng_draw.argtypes = [C.POINTER(OrcRng)]
        L.orc_sample_ic.argtypes = [C.POINTER(OrcSys), C.POINTER(OrcRng), C.POINTER(OrcLevel), C.c_int,
                                    C.POINTER(OrcIcCfg), C.c_int, _D, _D, _D, _D, _D, _I, _D]
        L.orc_boltzmann_er.restype = C.c_double
        L.orc_boltzmann_er.argtypes = [C.c_double, C.c_double]
        L.orc_bond_length.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, _D, _D]
        L.orc_analyze.argtypes = [C.POINTER(OrcSys), _D, C.POINTER(OrcPoint)]
        L.orc_turning_point.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, _D]
        L.orc_action_integral.restype = C.c_double
        L.orc_action_integral.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_double]
        L.orc_find_extremum.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, _D, _D]
        _lib = L
    return _lib


def dp(a):
    return a.ctypes.data_as(_D)


def ip(a):
    return a.ctypes.data_as(_I)


class Oracle:
    """CPU restatement bound to one system configuration (coarseair_gb300.systems.SystemConfig)."""

    def __init__(self, cfg):
        L = lib()
        self.L = L
        self.cfg = cfg
        s = OrcSys()
        s.natoms = cfg.natoms
        for i, m in enumerate(cfg.masses):
            s.mass[i] = m
        s.npes = len(cfg.surfaces)
        self._keep = []
        for i, srf in enumerate(cfg.surfaces):
            c = np.ascontiguousarray(srf.coef, dtype=np.float64)
            self._keep.append(c)
            p = s.pes[i]
            p.model, p.ncoef, p.coef = srf.model, c.size, dp(c)
            p.a, p.ab, p.ra, p.rb, p.eref, p.totdiss = srf.a, srf.ab, srf.ra, srf.rb, srf.eref, srf.totdiss
        s.diat = cfg.diat_model
        s.dt0, s.eps, s.relax, s.rmax, s.tmax, s.hamabstol = cfg.dt0, cfg.eps, cfg.relax, cfg.rmax, cfg.tmax, cfg.ham_abs_tol
        s.nsteps, s.incstpsz, s.ncall, s.nquad = cfg.nsteps, cfg.inc_step, cfg.ncall, cfg.nquad
        s.rsmal, s.rcent, s.rfact, s.tthresau = cfg.rsmal, cfg.rcent, cfg.rfact, cfg.tthresau
        if L.orc_sys_init(C.byref(s)) != 0:
            raise RuntimeError("singular mass matrix")
        self.s = s
        self.nv, self.ne, self.npairs = s.neqtvar, s.neqttot, s.npairs

    @property
    def tpq(self):
        nv = self.nv
        return np.array(self.s.Tpq[:]).reshape(9, 9, order="F")[:nv, :nv].copy()

    @property
    def tqp(self):
        nv = self.nv
        return np.array(self.s.Tqp[:]).reshape(9, 9, order="F")[:nv, :nv].copy()

    # -- surfaces --
    def compute(self, R, Qall, ipes=None):
        R = np.ascontiguousarray(R, np.float64).reshape(-1, self.npairs)
        n = R.shape[0]
        Q = np.ascontiguousarray(Qall, np.float64).reshape(n, -1)
        V, g, m = np.zeros(n), np.zeros((n, self.npairs)), np.zeros((n, self.nv))
        for k in range(n):
            self.L.orc_pes_compute(C.byref(self.s), 0 if ipes is None else int(ipes[k]), dp(R[k]), dp(Q[k]),
                                   dp(V[k:k + 1]), dp(g[k]), dp(m[k]))
        return V, g, m

    def condition_scale(self, R, ipes=None):
        """Magnitudes of the terms summed into V (column 0) and dV/dR_i (columns 1..NPairs): the scale at
        which a different evaluation order of the same surface changes the result."""
        R = np.ascontiguousarray(R, np.float64).reshape(-1, self.npairs)
        out = np.zeros((R.shape[0], 1 + self.npairs))
        for k in range(R.shape[0]):
            self.L.orc_pes_scale(C.byref(self.s), 0 if ipes is None else int(ipes[k]), dp(R[k]), dp(out[k]))
        return out

    def potential(self, R, ipes=None):
        R = np.ascontiguousarray(R, np.float64).reshape(-1, self.npairs)
        return np.array([self.L.orc_pes_potential(C.byref(self.s), 0 if ipes is None else int(ipes[k]), dp(R[k]))
                         for k in range(R.shape[0])])

    def rp(self, Q):
        Q = np.ascontiguousarray(Q, np.float64).reshape(-1, self.nv)
        n = Q.shape[0]
        R = np.zeros((n, self.npairs))
        Qall = np.zeros((n, self.nv + 3))
        for k in range(n):
            Qall[k, :self.nv] = Q[k]
            self.L.orc_rp(C.byref(self.s), dp(Qall[k]), dp(Qall[k, self.nv:]), dp(R[k]))
        return R, Qall

    def rhs(self, y, ipes=None):
        y = np.ascontiguousarray(y, np.float64).reshape(-1, self.ne)
        yp = np.zeros_like(y)
        for k in range(y.shape[0]):
            self.L.orc_rhs(C.byref(self.s), 0 if ipes is None else int(ipes[k]), dp(y[k]), dp(yp[k]))
        return yp

    def hamiltonian(self, paq, ipes=None):
        paq = np.ascontiguousarray(paq, np.float64).reshape(-1, self.ne)
        n = paq.shape[0]
        H, rpi = np.zeros(n), np.zeros((n, self.npairs))
        for k in range(n):
            self.L.orc_hamiltonian(C.byref(self.s), 0 if ipes is None else int(ipes[k]), dp(paq[k]),
                                   dp(H[k:k + 1]), dp(rpi[k]))
        return H, rpi

    def apply_transformation(self, paq):
        paq = np.ascontiguousarray(paq, np.float64).reshape(-1, self.ne)
        out = np.zeros_like(paq)
        for k in range(paq.shape[0]):
            self.L.orc_apply_transformation(C.byref(self.s), dp(paq[k]), dp(out[k]))
        return out

    # -- dynamics --
    def bs_attempts(self, paq, t, dt, erra, nattempts, ipes=None):
        paq = np.ascontiguousarray(paq, np.float64).copy()
        n = paq.shape[0]
        t, dt = np.ascontiguousarray(t, np.float64).copy(), np.ascontiguousarray(dt, np.float64).copy()
        erra = np.ascontiguousarray(erra, np.float64)
        ipe = np.zeros(n, np.int32) if ipes is None else np.ascontiguousarray(ipes, np.int32)
        self.L.orc_bs_attempts(C.byref(self.s), n, ip(ipe), dp(paq), dp(t), dp(dt), dp(erra), int(nattempts))
        return paq, t, dt

    def integrate(self, paq, erra, dt0=None, ipes=None, max_attempts=None, procs=1):
        """orc_integrate over a batch; procs > 1 splits it over that many spawned processes
        (trajectories are independent, so the result is the same)."""
        n = np.shape(paq)[0]
        if procs > 1 and n >= 2 * procs:
            import multiprocessing as mp
            parts = np.array_split(np.arange(n), procs)
            args = [(self.cfg, np.asarray(paq)[ix], np.asarray(erra)[ix], dt0,
                     None if ipes is None else np.asarray(ipes)[ix], max_attempts) for ix in parts]
            with mp.get_context("spawn").Pool(procs) as pool:
                outs = pool.starmap(_integrate_part, args)
            return {k: np.concatenate([o[k] for o in outs]) for k in outs[0]}
        paq = np.ascontiguousarray(paq, np.float64).copy()
        n = paq.shape[0]
        t = np.zeros(n)
        dt = np.full(n, self.cfg.dt0 if dt0 is None else dt0)
        H, smax, smin = np.zeros(n), np.full(n, -np.finfo(float).max), np.full(n, np.finfo(float).max)
        irej, iste, st = np.zeros(n, np.int32), np.zeros(n, np.int32), np.zeros(n, np.int32)
        ipe = np.zeros(n, np.int32) if ipes is None else np.ascontiguousarray(ipes, np.int32)
        ma = self.cfg.max_attempts if max_attempts is None else max_attempts
        self.L.orc_integrate(C.byref(self.s), n, ip(ipe), dp(paq), dp(t), dp(dt), dp(np.ascontiguousarray(erra)),
                             dp(H), dp(smax), dp(smin), ip(irej), ip(iste), ip(st), int(ma))
        return dict(paq=paq, t=t, dt=dt, H=H, smax=smax, smin=smin, irej=irej, iste=iste, status=st)

    # -- initial conditions --
    def sample_ics(self, n, levels, state_specific=True, ttra=None, bmax=None, dinit=None, seed=None, ilevels=None,
                   rings=None):
        """Sample n initial conditions from one RNG stream as the reference does for one PES.
        rings = (bring, ntring, b_mode): the n trajectories stratified as ImpactParameter_Class
        splits them (ring input values bring, weights ntring); otherwise one Circles ring bmax."""
        cfg = self.cfg
        rng = OrcRng()
        self.L.orc_rng_seed(C.byref(rng), int(cfg.seed if seed is None else seed))
        lv = (OrcLevel * len(levels))()
        for i, row in enumerate(levels):
            L = lv[i]
            L.vqn, L.jqn = int(row["vqn"]), int(row["jqn"])
            for c in ("eint", "egam", "rmin", "rmax", "vmin", "vmax", "tau", "ri", "ro", "rlim"):
                setattr(L, c, float(row[c]))
        ic = OrcIcCfg(cfg.ttra if ttra is None else ttra, cfg.bmax if bmax is None else bmax,
                      cfg.dinit if dinit is None else dinit, 1 if state_specific else 0)
        ne = self.ne
        paq, paq0, erra = np.zeros((n, ne)), np.zeros((n, ne)), np.zeros((n, ne))
        H0, b, er = np.zeros(n), np.zeros(n), np.zeros(n)
        il = np.zeros(n, np.int32)
        if rings is not None:
            itm = impact_rings(n, rings[0], rings[1])
        for k in range(n):
            if rings is not None:
                bmin_r, b_r = impact_ring_of(k + 1, rings[0], itm)
                ic.bmax, ic.bmin, ic.b_mode = -b_r, -bmin_r, int(rings[2])
            self.L.orc_sample_ic(C.byref(self.s), C.byref(rng), lv, len(levels), C.byref(ic), 0, dp(paq[k]),
                                 dp(paq0[k]), dp(H0[k:k + 1]), dp(erra[k]), dp(b[k:k + 1]), ip(il[k:k + 1]),
                                 dp(er[k:k + 1]))
        return dict(paq=paq, paq0=paq0, H0=H0, erra=erra, b=b, ilevel=il, er=er)

    def sample_ics4(self, n, level1, level2, ttra=None, bmax=None, dinit=None, seed=None, rings=None):
        """Diatom + diatom initial conditions (state-specific, one level per molecule) from one stream;
        rings as for sample_ics."""
        cfg = self.cfg
        rng = OrcRng()
        self.L.orc_rng_seed(C.byref(rng), int(cfg.seed if seed is None else seed))
        lv = (OrcLevel * 2)()
        for i, row in enumerate((level1, level2)):
            L = lv[i]
            L.vqn, L.jqn = int(row["vqn"]), int(row["jqn"])
            for c in ("eint", "egam", "rmin", "rmax", "vmin", "vmax", "tau", "ri", "ro"):
                setattr(L, c, float(row[c]))
            L.rlim = 0.0
        ic = OrcIcCfg(cfg.ttra if ttra is None else ttra, cfg.bmax if bmax is None else bmax,
                      cfg.dinit if dinit is None else dinit, 1)
        ne = self.ne
        paq, paq0, erra = np.zeros((n, ne)), np.zeros((n, ne)), np.zeros((n, ne))
        H0, b, er = np.zeros(n), np.zeros(n), np.zeros(n)
        if rings is not None:
            itm = impact_rings(n, rings[0], rings[1])
        for k in range(n):
            if rings is not None:
                bmin_r, b_r = impact_ring_of(k + 1, rings[0], itm)
                ic.bmax, ic.bmin, ic.b_mode = -b_r, -bmin_r, int(rings[2])
            self.L.orc_sample_ic4(C.byref(self.s), C.byref(rng), C.byref(lv[0]), C.byref(lv[1]), C.byref(ic), 0,
                                  dp(paq[k]), dp(paq0[k]), dp(H0[k:k + 1]), dp(erra[k]), dp(b[k:k + 1]),
                                  dp(er[k:k + 1]))
        return dict(paq=paq, paq0=paq0, H0=H0, erra=erra, b=b, er=er)

    # -- final states --
    def analyze(self, paq_vel):
        paq_vel = np.ascontiguousarray(paq_vel, np.float64).reshape(-1, self.ne)
        out = []
        for k in range(paq_vel.shape[0]):
            p = OrcPoint()
            self.L.orc_analyze(C.byref(self.s), dp(paq_vel[k]), C.byref(p))
            out.append(dict(ipair=p.mol[0].ipair, itype=p.mol[0].itype, eint=p.mol[0].eint,
                            angmom=p.mol[0].angmom, viba=p.mol[0].viba, b=p.b, xkin=p.xkin,
                            ipair1=p.mol[1].ipair, itype1=p.mol[1].itype, angmom1=p.mol[1].angmom,
                            viba1=p.mol[1].viba))
        return out


def _integrate_part(cfg, paq, erra, dt0, ipes, max_attempts):
    return Oracle(cfg).integrate(paq, erra, dt0=dt0, ipes=ipes, max_attempts=max_attempts)


def statistics(bmax, bsamp, qini, qfin, iskip=(1, 1, 1), pres=(0, 0, 0), qnmax=300, cap=4096):
    """orc_statistics for the rows of one run: list of (fincond tuple, count, cross, cross_sd) in order
    of first appearance, and IniState."""
    L = lib()
    n = len(bmax)
    qini = np.ascontiguousarray(qini, np.float64).reshape(n, -1)
    qfin = np.ascontiguousarray(qfin, np.float64).reshape(n, -1)
    ncond = qini.shape[1]
    sk = np.ascontiguousarray(iskip, np.int32)
    pr = np.ascontiguousarray([int(bool(x)) for x in pres], np.int32)
    codes = np.zeros(cap, np.int64)
    fin = np.zeros(cap * ncond, np.int32)
    ini = np.zeros(ncond, np.int32)
    counts = np.zeros(cap, np.int64)
    cross, sd = np.zeros(cap), np.zeros(cap)
    nfs = L.orc_statistics(n, ncond, ip(sk), ip(pr), int(qnmax), dp(np.ascontiguousarray(bmax, np.float64)),
                           dp(np.ascontiguousarray(bsamp, np.float64)), dp(qini), dp(qfin), cap,
                           codes.ctypes.data_as(C.POINTER(C.c_int64)), ip(fin), ip(ini),
                           counts.ctypes.data_as(C.POINTER(C.c_int64)), dp(cross), dp(sd))
    if nfs < 0:
        raise ValueError("orc_statistics failed (%d)" % nfs)
    fin = fin.reshape(cap, ncond)
    return [(tuple(int(x) for x in fin[i]), int(counts[i]), float(cross[i]), float(sd[i])) for i in range(nfs)], \
        tuple(int(x) for x in ini)


def mean_velocity(ttra, xmu):
    return lib().orc_mean_velocity(float(ttra), float(xmu))
