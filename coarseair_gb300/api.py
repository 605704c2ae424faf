"""Host-side interface mirroring the reference's operators for the trajectory path.

    PES(system).Compute(R, Q)          -> V, dVdR, dVdQ      PES_Type%Compute   (PES_Class.F90:43-72)
    PES(system).Potential(R)           -> V                  PES_Type%Potential
    Collision(system).Hamiltonian(PaQ) -> H, Rpi             Collision_Type%Hamiltonian_1d
    Collision(system).EvaluateRHS(y)   -> dy/dt              HamiltonODESystem (RHS_Evaluation)
    Collision(system).ApplyTransformation(PaQ) -> PaQ with velocities
    ODE(system).Integrate(traj, n)     -> n BS attempts      ODE_Solver_Type%Integrate
    Integrator(system).Integrate(traj) -> to end of collision Integrator_Type%Integrate (propagation)
    MolecularState.FindState(PaQ)      -> final states       TrajectoryPoint%Analyze + FindState

All arrays are FP64 numpy arrays laid out as the Fortran arrays (PaQ per trajectory
contiguous).  Every call runs on the GPU through libcair_gpu.so; no CPU path exists.
"""
import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import dptr, iptr


class CairError(RuntimeError):
    pass


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


def _i32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int32)


def system_desc(cfg, tpq=None):
    """cair_system_desc of a SystemConfig; returns it with the arrays it points into (keep them alive)."""
    d = _lib.SystemDesc()
    d.abi_version = _lib.CAIR_ABI_VERSION
    d.natoms = cfg.natoms
    d.npes = len(cfg.surfaces)
    d.diat_model = cfg.diat_model
    for i, m in enumerate(cfg.masses):
        d.mass[i] = m
    keep = []
    for i, s in enumerate(cfg.surfaces):
        c = np.ascontiguousarray(s.coef, dtype=np.float64)
        keep.append(c)
        p = d.pes[i]
        p.model, p.ncoef, p.coef = s.model, c.size, dptr(c)
        p.a, p.ab, p.ra, p.rb, p.eref, p.totdiss = s.a, s.ab, s.ra, s.rb, s.eref, s.totdiss
    if tpq is not None:
        t = np.asfortranarray(tpq, dtype=np.float64).ravel(order="F")
        keep.append(t)
        d.tpq = dptr(t)
    d.dt0, d.eps, d.relax, d.rmax, d.tmax, d.ham_abs_tol = (cfg.dt0, cfg.eps, cfg.relax, cfg.rmax, cfg.tmax,
                                                            cfg.ham_abs_tol)
    d.nsteps, d.inc_step, d.ncall, d.nquad = cfg.nsteps, cfg.inc_step, cfg.ncall, cfg.nquad
    d.rsmal, d.rcent, d.rfact, d.tthresau = cfg.rsmal, cfg.rcent, cfg.rfact, cfg.tthresau
    return d, keep


class Handle:
    """Owns one cair_handle (device copies of the surfaces, stream, scratch)."""

    def __init__(self, cfg, tpq=None):
        lib = _lib.load()
        self.lib = lib
        self.cfg = cfg
        d, self._keep = system_desc(cfg, tpq)
        h = C.c_void_p()
        rc = lib.cair_create(C.byref(h), C.byref(d))
        self.h = h
        if rc != 0:
            msg = lib.cair_last_error(h).decode() if h else ""
            if h:
                lib.cair_destroy(h)
            self.h = None
            raise CairError("cair_create: %s (%s)" % (_lib.STATUS.get(rc, rc), msg))
        nv, ne, np_ = C.c_int32(), C.c_int32(), C.c_int32()
        lib.cair_dims(h, C.byref(nv), C.byref(ne), C.byref(np_))
        self.nv, self.ne, self.npairs = nv.value, ne.value, np_.value

    def check(self, rc, what):
        if rc != 0:
            raise CairError("%s: %s (%s)" % (what, _lib.STATUS.get(rc, rc), self.lib.cair_last_error(self.h).decode()))

    def close(self):
        if self.h:
            self.lib.cair_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def tpq(self):
        t = np.zeros(self.nv * self.nv)
        self.check(self.lib.cair_get_tpq(self.h, dptr(t)), "cair_get_tpq")
        return t.reshape(self.nv, self.nv, order="F")

    def flop_model(self, ipes=0):
        a, b, c, d = C.c_double(), C.c_double(), C.c_double(), C.c_double()
        self.check(self.lib.cair_flop_model(self.h, ipes, C.byref(a), C.byref(b), C.byref(c), C.byref(d)),
                   "cair_flop_model")
        return dict(grad=a.value, energy=b.value, attempt=c.value, exp=d.value)

    _MODES = {"thread": _lib.INTEGRATOR_THREAD, "warp": _lib.INTEGRATOR_WARP, "auto": _lib.INTEGRATOR_AUTO}

    @property
    def integrator_mode(self):
        """"thread" (a lane per trajectory, the default), "warp" (a warp per trajectory: the latency
        mode for small jobs; O3, N3, O4 and N4 UMN surfaces) or "auto" (warp for launches of fewer
        trajectories than twice the thread integrator's resident lanes, where it has programs)."""
        m = self.lib.cair_get_integrator_mode(self.h)
        return {v: k for k, v in self._MODES.items()}[m]

    def set_tail_handoff(self, below=-1):
        """AUTO mode's tail hand-off threshold (trajectories in flight): -1 the warp integrator's resident
        warps, 0 off."""
        self.check(self.lib.cair_set_tail_handoff(self.h, int(below)), "cair_set_tail_handoff")

    def last_handoffs(self):
        """Trajectories the last launch handed from the thread to the warp integrator."""
        return int(self.lib.cair_last_handoffs(self.h))

    @property
    def last_integrator(self):
        """The integrator ("thread" or "warp") the handle's last launch ran."""
        return "warp" if self.lib.cair_last_integrator(self.h) == _lib.INTEGRATOR_WARP else "thread"

    @integrator_mode.setter
    def integrator_mode(self, mode):
        m = self._MODES[mode]
        self.check(self.lib.cair_set_integrator_mode(self.h, m), "cair_set_integrator_mode")

    def counters(self):
        c = np.zeros(5, dtype=np.int64)
        self.check(self.lib.cair_last_counters(self.h, c.ctypes.data_as(C.POINTER(C.c_int64))), "counters")
        return dict(attempts=int(c[0]), accepted=int(c[1]), rejected=int(c[2]), grad_evals=int(c[3]),
                    energy_evals=int(c[4]))


class PES:
    """Batched PES_Type%Compute / %Potential."""

    def __init__(self, handle):
        self.H = handle

    def Compute(self, R, Qall, ipes=None):
        H = self.H
        R = _f64(R, (-1, H.npairs))
        n = R.shape[0]
        Qall = _f64(Qall, (n, 3 * H.cfg.natoms))
        V = np.zeros(n)
        dVdR = np.zeros((n, H.npairs))
        dVdQ = np.zeros((n, H.nv))
        H.check(H.lib.cair_pes_eval(H.h, n, iptr(_i32(ipes)), dptr(R), dptr(Qall), dptr(V), dptr(dVdR), dptr(dVdQ)),
                "cair_pes_eval")
        return V, dVdR, dVdQ

    def Potential(self, R, Qall=None, ipes=None):
        H = self.H
        R = _f64(R, (-1, H.npairs))
        n = R.shape[0]
        if Qall is None:
            Qall = np.zeros((n, 3 * H.cfg.natoms))
        Qall = _f64(Qall, (n, 3 * H.cfg.natoms))
        V = np.zeros(n)
        H.check(H.lib.cair_pes_eval(H.h, n, iptr(_i32(ipes)), dptr(R), dptr(Qall), dptr(V), None, None),
                "cair_pes_eval")
        return V


class Collision:
    def __init__(self, handle):
        self.H = handle

    def EvaluateRHS(self, y, ipes=None):
        H = self.H
        y = _f64(y, (-1, H.ne))
        yp = np.zeros_like(y)
        H.check(H.lib.cair_rhs(H.h, y.shape[0], iptr(_i32(ipes)), dptr(y), dptr(yp)), "cair_rhs")
        return yp

    def Hamiltonian(self, paq, ipes=None):
        H = self.H
        paq = _f64(paq, (-1, H.ne))
        n = paq.shape[0]
        h = np.zeros(n)
        rpi = np.zeros((n, H.npairs))
        H.check(H.lib.cair_hamiltonian(H.h, n, iptr(_i32(ipes)), dptr(paq), dptr(h), dptr(rpi)), "cair_hamiltonian")
        return h, rpi

    def ApplyTransformation(self, paq):
        H = self.H
        paq = _f64(paq, (-1, H.ne))
        out = np.zeros_like(paq)
        H.check(H.lib.cair_apply_transformation(H.h, paq.shape[0], dptr(paq), dptr(out)), "cair_apply_transformation")
        return out


@dataclass
class Trajectories:
    """Trajectories_Type state (Trajectories_Class.F90:34-68), one row per trajectory."""
    paq: np.ndarray
    t: np.ndarray
    dt: np.ndarray
    erra: np.ndarray
    ipes: np.ndarray
    H: np.ndarray = None
    smax: np.ndarray = None
    smin: np.ndarray = None
    irej: np.ndarray = None
    iste: np.ndarray = None
    status: np.ndarray = None

    @classmethod
    def start(cls, paq, erra, dt0, ipes=None):
        """Initial state as SetIniCondForward sets it (Collision_Class.F90:1100-1108)."""
        paq = _f64(paq)
        n = paq.shape[0]
        return cls(paq=paq.copy(), t=np.zeros(n), dt=np.full(n, float(dt0)), erra=_f64(erra).copy(),
                   ipes=np.zeros(n, np.int32) if ipes is None else _i32(ipes).copy(),
                   H=np.zeros(n), smax=np.full(n, -np.finfo(np.float64).max),
                   smin=np.full(n, np.finfo(np.float64).max), irej=np.zeros(n, np.int32),
                   iste=np.zeros(n, np.int32), status=np.zeros(n, np.int32))


class ODE:
    def __init__(self, handle):
        self.H = handle

    def Integrate(self, traj, nattempts):
        """Exactly `nattempts` Bulirsch-Stoer attempts per trajectory (no end checks)."""
        H = self.H
        n = traj.paq.shape[0]
        H.check(H.lib.cair_bs_steps(H.h, n, iptr(traj.ipes), dptr(traj.paq), dptr(traj.t), dptr(traj.dt),
                                    dptr(traj.erra), int(nattempts)), "cair_bs_steps")
        return traj


class Integrator:
    def __init__(self, handle):
        self.H = handle

    def Integrate(self, traj, max_attempts=None):
        """Propagate to the end of the collision; fills H (last end check) and status."""
        H = self.H
        n = traj.paq.shape[0]
        ma = int(max_attempts if max_attempts is not None else H.cfg.max_attempts)
        H.check(H.lib.cair_integrate(H.h, n, iptr(traj.ipes), dptr(traj.paq), dptr(traj.t), dptr(traj.dt),
                                     dptr(traj.erra), dptr(traj.H), dptr(traj.smax), dptr(traj.smin),
                                     iptr(traj.irej), iptr(traj.iste), iptr(traj.status), ma), "cair_integrate")
        return traj


class MolecularState:
    def __init__(self, handle):
        self.H = handle

    def FindState(self, paq_vel):
        """Analyse trajectory points given velocities+coordinates; returns a structured array."""
        H = self.H
        paq_vel = _f64(paq_vel, (-1, H.ne))
        n = paq_vel.shape[0]
        out = np.zeros(n, dtype=_lib.TRAJ_POINT_DTYPE)
        H.check(H.lib.cair_find_state(H.h, n, dptr(paq_vel), out.ctypes.data_as(C.POINTER(_lib.TrajPoint))),
                "cair_find_state")
        return out


def level_table(levels):
    """Level rows (systems.load_levels) as the C struct array cair_level[]."""
    out = np.zeros(len(levels), dtype=_lib.LEVEL_DTYPE)
    for c in _lib.LEVEL_DTYPE.names:
        out[c] = levels[c]
    return out


def work_items(entries):
    """entries: iterable of (ilevel, ipes, ntraj, seed, ttra, bmax, dinit[, ilevel2[, b_mode, bmin, skip]])
    -> cair_work_item[] tiling the batch in order; ilevel2 is the projectile diatom's level of a
    diatom + diatom system; b_mode, bmin, skip describe an impact-parameter ring (ring_entries)."""
    entries = list(entries)
    out = np.zeros(len(entries), dtype=_lib.ITEM_DTYPE)
    first = 0
    for i, e in enumerate(entries):
        il, ip, nt, seed, ttra, bmax, dinit = e[:7]
        il2 = e[7] if len(e) > 7 else 0
        mode, bmin, skip = (e[8], e[9], e[10]) if len(e) > 8 else (0, 0.0, 0)
        out[i] = (il, ip, first, nt, seed, ttra, bmax, dinit, il2, mode, bmin, skip)
        first += nt
    return out


STRATA = {"Circles": 0, "Rings": 1, "Segments": 2}


def ring_entries(ilevel, ipes, ntraj, seed, ttra, dinit, bring, ntring, strata="Circles", ilevel2=0):
    """Work-item entries for one stream of `ntraj` trajectories stratified in impact-parameter rings,
    as InitializeImpactParameter and GetImpactParamValue split it (ImpactParameter_Class.F90:55-221):
    ring r gets int(ntring_r x ntraj / sum(ntring)) trajectories, the first ring the remainder,
    and draws its impact parameter from the ring's input value bring_r (negative: sampled by the
    strata type up to |bring_r|; positive: that fixed value) with the previous ring's value as
    bmin.  The rings continue one random-number stream (skip = trajectories of the earlier rings)."""
    bring, ntring = list(bring), [int(x) for x in ntring]
    if len(bring) != len(ntring) or not bring:
        raise ValueError("one weight per ring")
    if any(w < 0 for w in ntring):
        raise ValueError("negative ring weights leave the reference's rings without trajectories")
    total = sum(ntring)
    counts = [int(float(w * ntraj) / total) for w in ntring]
    counts[0] += ntraj - sum(counts)
    out, skip = [], 0
    for r, (b, n) in enumerate(zip(bring, counts)):
        bmin = -bring[r - 1] if r > 0 else 0.0
        out.append((ilevel, ipes, n, seed, ttra, -float(b), dinit, ilevel2, STRATA[strata], float(bmin), skip))
        skip += n
    return out


def degeneracy_blocks(ntraj, degeneracies):
    """Trajectories per surface of a batch, as SetPESIndx assigns them (Collision_Class.F90:2468-2507):
    contiguous blocks of int(g_k / sum(g) * ntraj) for every surface but the last, which takes the rest."""
    g = np.asarray(degeneracies, dtype=np.float64)
    g = g / g.sum()
    counts = [int(x * ntraj) for x in g[:-1]]
    return counts + [ntraj - sum(counts)]


def process_seed(iseed, iproc, npes=1, inode=1, rndnb=0):
    """Stream seed of process iProc (Collision_Class.F90:295-296)."""
    return int(iseed * (1 + (iproc - 1) * (npes + 1) + (inode - 1) * 200.0 * (npes + 1)) +
               rndnb * 200.0 * 100.0 * (npes + 2))


class InitialConditions:
    """SetIniCondForward for diatom + atom and diatom + diatom work items, on the GPU."""

    def __init__(self, handle):
        self.H = handle

    def sample(self, levels, items):
        H = self.H
        lv = np.ascontiguousarray(levels, dtype=_lib.LEVEL_DTYPE)
        it = np.ascontiguousarray(items, dtype=_lib.ITEM_DTYPE)
        n = int(it["ntraj"].sum())
        paq, paq0, erra = np.zeros((n, H.ne)), np.zeros((n, H.ne)), np.zeros((n, H.ne))
        H0, b, ipes = np.zeros(n), np.zeros(n), np.zeros(n, np.int32)
        H.check(H.lib.cair_sample_ics(H.h, len(lv), lv.ctypes.data, len(it), it.ctypes.data, n, dptr(paq),
                                      dptr(paq0), dptr(erra), dptr(H0), dptr(b), iptr(ipes)), "cair_sample_ics")
        return dict(paq=paq, paq0=paq0, erra=erra, H0=H0, b=b, ipes=ipes)


class RunTrajectories:
    """RunTrajectories for work items, end to end on the GPU; returns trajectories.out rows."""

    def __init__(self, handle):
        self.H = handle

    def run(self, levels, items, max_attempts=None):
        H = self.H
        lv = np.ascontiguousarray(levels, dtype=_lib.LEVEL_DTYPE)
        it = np.ascontiguousarray(items, dtype=_lib.ITEM_DTYPE)
        n = int(it["ntraj"].sum())
        out = np.zeros(n, dtype=_lib.RESULT_DTYPE)
        ma = int(max_attempts if max_attempts is not None else H.cfg.max_attempts)
        H.check(H.lib.cair_run_queue(H.h, len(lv), lv.ctypes.data, len(it), it.ctypes.data, n, ma, out.ctypes.data),
                "cair_run_queue")
        return out


def autotune(handle, levels, items, sample=65536, cap_attempts=300):
    """The project's autotuner (cair_autotune): measures every launch shape of the persistent
    integrator on a capped sample of these work items and keeps the fastest on the handle.  Returns
    (chosen (block, per_sm), the measured points)."""
    H = handle
    lv = np.ascontiguousarray(levels, dtype=_lib.LEVEL_DTYPE)
    it = np.ascontiguousarray(items, dtype=_lib.ITEM_DTYPE)
    pts = np.zeros(32, dtype=_lib.TUNE_POINT_DTYPE)
    n = C.c_int32()
    H.check(H.lib.cair_autotune(H.h, len(lv), lv.ctypes.data, len(it), it.ctypes.data, int(sample), int(cap_attempts),
                                pts.ctypes.data, len(pts), C.byref(n)), "cair_autotune")
    b, p = C.c_int32(), C.c_int32()
    H.check(H.lib.cair_get_launch_shape(H.h, C.byref(b), C.byref(p)), "cair_get_launch_shape")
    return (b.value, p.value), pts[:n.value].copy()


def _nint(x):
    """Fortran nint: nearest integer, halves away from zero."""
    x = np.asarray(x, dtype=np.float64)
    return (np.sign(x) * np.floor(np.abs(x) + 0.5)).astype(np.int64)


def histogram_assign(j, v, arr):
    """Final (J, v, arrangement) integers of the histogram method (Statistics_Class.F90:626-656)."""
    return _nint(np.asarray(j) - 0.5), _nint(np.asarray(v) - 0.5), _nint(np.asarray(arr) - 0.5)


def format_rows(rows, idx_offset=0, header=True, nmol=1):
    """trajectories.out text of result rows (Integrator_Class.F90:884-933); nmol is NInitMolecules
    (1: diatom + atom, 2: diatom + diatom)."""
    lib = _lib.load()
    rw = np.ascontiguousarray(rows, dtype=_lib.RESULT_DTYPE)
    n = C.c_int64(0)
    lib.cair_format_rows(rw.ctypes.data, len(rw), int(idx_offset), int(nmol), int(header), None, 0, C.byref(n))
    buf = C.create_string_buffer(n.value + 1)
    rc = lib.cair_format_rows(rw.ctypes.data, len(rw), int(idx_offset), int(nmol), int(header), buf, n.value,
                              C.byref(n))
    if rc != 0:
        raise CairError("cair_format_rows: %s" % _lib.STATUS.get(rc, rc))
    return buf.raw[:n.value].decode()


def write_trajectories(directory, rows, ham_abs_tol, idx_offset=0, binary=None, nmol=1):
    """Write trajectories.out and trajectories_HNotCons.out (and trajectories.bin if `binary` is a
    path); returns (rows in trajectories.out, rows in trajectories_HNotCons.out).  nmol is
    NInitMolecules (1: diatom + atom, 2: diatom + diatom)."""
    lib = _lib.load()
    rw = np.ascontiguousarray(rows, dtype=_lib.RESULT_DTYPE)
    cnt = (C.c_int64 * 2)()
    rc = lib.cair_write_trajectories(str(directory).encode(), rw.ctypes.data, len(rw), int(idx_offset), int(nmol),
                                     float(ham_abs_tol), cnt)
    if rc != 0:
        raise CairError("cair_write_trajectories: %s" % _lib.STATUS.get(rc, rc))
    if binary is not None:
        rc = lib.cair_write_trajectories_bin(str(binary).encode(), rw.ctypes.data, len(rw), int(idx_offset),
                                             int(nmol), float(ham_abs_tol))
        if rc != 0:
            raise CairError("cair_write_trajectories_bin: %s" % _lib.STATUS.get(rc, rc))
    return cnt[0], cnt[1]


def merge_trajectories(src_dirs, out_dir):
    """MergeTrajectories (ComputeRates.sh:406-472): append each directory's trajectories.out and
    trajectories_HNotCons.out to out_dir/trajectories.csv and out_dir/trajectories_HNotCons.out
    (one header line), write out_dir/NConvTraj.dat; returns the merged row count."""
    lib = _lib.load()
    src = [str(d).encode() for d in src_dirs]
    arr = (C.c_char_p * max(1, len(src)))(*src)
    n = C.c_int64(0)
    rc = lib.cair_merge_trajectories(len(src), arr, str(out_dir).encode(), C.byref(n))
    if rc != 0:
        raise CairError("cair_merge_trajectories: %s" % _lib.STATUS.get(rc, rc))
    return n.value


class Statistics:
    """TrajectoriesStats for state-specific runs (Statistics_Class.F90, Histogram assignment):
    final-state cross sections [bohr^2] and rate coefficients [cm^3/s] per work item, counted on
    the GPU.  Conditions are J, v, arrangement for diatom + atom and J1, v1, J2, v2, arrangement for
    diatom + diatom (the reference's N4/O4 inputs, Identical Diatoms = no).  Defaults are the
    reference's (QuantumNumberMax 300, Iskip 1, no even/oddness preserved); shorter iskip and
    pres_even_odd tuples are padded with those defaults."""

    def __init__(self, handle, qn_max=300, iskip=(1, 1, 1, 1, 1), pres_even_odd=(0, 0, 0, 0, 0), ham_abs_tol=None,
                 xmu=None):
        self.H = handle
        cfg = handle.cfg
        m = cfg.masses
        ncond = 5 if cfg.natoms == 4 else 3
        iskip = tuple(iskip) + (1,) * (5 - len(iskip))
        pres_even_odd = tuple(pres_even_odd) + (0,) * (5 - len(pres_even_odd))
        p = _lib.StatsParams()
        p.qn_max = int(qn_max)
        p.ncond = ncond
        for i in range(5):
            p.iskip[i] = int(iskip[i]) if i < ncond else 0
            p.pres_even_odd[i] = int(bool(pres_even_odd[i])) if i < ncond else 0
        p.ham_abs_tol = float(cfg.ham_abs_tol if ham_abs_tol is None else ham_abs_tol)
        # RedMass of the relative translation, target against projectile (Collision_Class.F90:454):
        # diatom (atoms 1, 2) against atom 3, or against the diatom (atoms 3, 4)
        if xmu is None:
            mt, mp = m[0] + m[1], sum(m[2:])
            xmu = mt * mp / (mt + mp)
        p.xmu = float(xmu)
        self.ncond = ncond
        self.params = p

    def compute(self, items, rows, runs=None, cap=None):
        """Final states of every run.  runs[i] is the run of work item i: the items (surfaces,
        impact-parameter rings) whose rows the reference's statistics read together for one
        initial state and temperature; None makes each item its own run."""
        H = self.H
        it = np.ascontiguousarray(items, dtype=_lib.ITEM_DTYPE)
        rw = np.ascontiguousarray(rows, dtype=_lib.RESULT_DTYPE)
        rn = None if runs is None else np.ascontiguousarray(runs, dtype=np.int32)
        if rn is not None and len(rn) != len(it):
            raise ValueError("runs must have one entry per work item")
        cap = int(cap if cap is not None else max(64, len(rw)))
        out = np.zeros(cap, dtype=_lib.FINAL_STATE_DTYPE)
        n = C.c_int64(0)
        H.check(H.lib.cair_statistics(H.h, len(it), it.ctypes.data, None if rn is None else rn.ctypes.data, len(rw),
                                      rw.ctypes.data, C.byref(self.params), out.ctypes.data, cap, C.byref(n)),
                "cair_statistics")
        return out[:n.value].copy()

    # -- replicas: step 1 and step 2 of the host-side exchange (statistics_finish is step 3) --
    def replica_items(self, nitems, rows):
        """This replica's counted rows and smallest initial-state code per item."""
        H = self.H
        rw = np.ascontiguousarray(rows, dtype=_lib.RESULT_DTYPE)
        item_rows = np.zeros(int(nitems), np.uint64)
        item_ini = np.zeros(int(nitems), np.int64)
        H.check(H.lib.cair_statistics_items(H.h, int(nitems), len(rw), rw.ctypes.data, C.byref(self.params),
                                            item_rows.ctypes.data, item_ini.ctypes.data), "cair_statistics_items")
        return item_rows, item_ini

    def replica_counts(self, items, rows, item_rows, item_ini, runs=None, cap=None):
        """This replica's (run, ring, code) counts under the rings of the replicas' totals, and its rows
        per (run, ring) as an nruns x 64 array."""
        H = self.H
        it = np.ascontiguousarray(items, dtype=_lib.ITEM_DTYPE)
        rw = np.ascontiguousarray(rows, dtype=_lib.RESULT_DTYPE)
        rn = None if runs is None else np.ascontiguousarray(runs, dtype=np.int32)
        ir = np.ascontiguousarray(item_rows, dtype=np.uint64)
        ii = np.ascontiguousarray(item_ini, dtype=np.int64)
        nruns = len(it) if rn is None else int(rn.max()) + 1
        cap = int(cap if cap is not None else max(64, len(rw)))
        out = np.zeros(cap, dtype=_lib.STATS_COUNT_DTYPE)
        ring_rows = np.zeros((nruns, _lib.STATS_MAX_RINGS), np.uint64)
        n = C.c_int64(0)
        H.check(H.lib.cair_statistics_counts(H.h, len(it), it.ctypes.data, None if rn is None else rn.ctypes.data,
                                             ir.ctypes.data, ii.ctypes.data, len(rw), rw.ctypes.data,
                                             C.byref(self.params), out.ctypes.data, cap, C.byref(n),
                                             ring_rows.ctypes.data), "cair_statistics_counts")
        return out[:n.value].copy(), ring_rows

    def replica_compute(self, items, rows, runs=None, group=None, cap=None):
        """Lines of every replica's rows together, on every rank of a torch.distributed group that ran
        the same items from disjoint streams (see replica_statistics)."""
        return replica_statistics(self.params, items, rows, runs, self.replica_items, self.replica_counts,
                                  group=group, cap=cap)


def statistics_finish(params, items, item_rows, item_ini, counts, ring_rows, runs=None, cap=None):
    """Step 3 of the replicas' statistics (cair_statistics_finish, host code): the lines from the summed
    totals and counts."""
    lib = _lib.load()
    it = np.ascontiguousarray(items, dtype=_lib.ITEM_DTYPE)
    rn = None if runs is None else np.ascontiguousarray(runs, dtype=np.int32)
    ir = np.ascontiguousarray(item_rows, dtype=np.uint64)
    ii = np.ascontiguousarray(item_ini, dtype=np.int64)
    ct = np.ascontiguousarray(counts, dtype=_lib.STATS_COUNT_DTYPE)
    rr = np.ascontiguousarray(ring_rows, dtype=np.uint64)
    cap = int(cap if cap is not None else max(64, len(ct)))
    out = np.zeros(cap, dtype=_lib.FINAL_STATE_DTYPE)
    n = C.c_int64(0)
    msg = C.create_string_buffer(256)
    rc = lib.cair_statistics_finish(len(it), it.ctypes.data, None if rn is None else rn.ctypes.data, ir.ctypes.data,
                                    ii.ctypes.data, C.byref(params), len(ct), ct.ctypes.data, rr.ctypes.data,
                                    out.ctypes.data, cap, C.byref(n), msg, 256)
    if rc != 0:
        raise CairError("cair_statistics_finish: %s (%s)" % (_lib.STATUS.get(rc, rc), msg.value.decode()))
    return out[:n.value].copy()


def replica_statistics(params, items, rows, runs, items_pass, counts_pass, group=None, cap=None):
    """The statistics of torch.distributed replicas that ran the same work items from disjoint streams,
    with two host-side sums as the only exchange (the reference merges its processes' trajectories.out
    files instead): items_pass(nitems, rows) -> (item_rows, item_ini); the totals summed (rows) and
    minimised (initial codes) over ranks; counts_pass(items, rows, item_rows, item_ini, runs) -> (counts,
    ring_rows) under the rings those totals define; the ring rows summed, the counts gathered; and
    statistics_finish.  Every rank returns the same lines."""
    import torch
    import torch.distributed as dist
    ir, ii = items_pass(len(items), rows)
    t = torch.from_numpy(np.asarray(ir, np.int64).copy())
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    ir = t.numpy().astype(np.uint64)
    t = torch.from_numpy(np.asarray(ii, np.int64).copy())
    dist.all_reduce(t, op=dist.ReduceOp.MIN, group=group)
    ii = t.numpy()
    counts, ring_rows = counts_pass(items, rows, ir, ii, runs)
    t = torch.from_numpy(np.asarray(ring_rows, np.int64).copy())
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    ring_rows = t.numpy().astype(np.uint64)
    parts = [None] * dist.get_world_size(group)
    dist.all_gather_object(parts, np.asarray(counts, dtype=_lib.STATS_COUNT_DTYPE), group=group)
    return statistics_finish(params, items, ir, ii, np.concatenate(parts), ring_rows, runs, cap=cap)
