"""Learned surrogate of the N3 UMN three-body term (host side of cair_sur_* in include/cair_gpu.h).

The reference has no learned surface on this path; this module builds one for the N2 + N queue:

* `record_training_set` runs the FP64 queue with the integrator's geometry recorder on, so the
  training geometries lie along the method's own trajectories, and `targets` evaluates the FP64
  surface's three-body term and its gradient there (both on the GPU).
* `Surrogate` holds the two ensemble members; `train` runs the hand-written training kernels
  (forward, input gradient, tangent and reverse passes on the tensor cores, then Adam).
* `Surrogate.attach(handle)` makes every integrator launch of the handle run on the surrogate, with
  the per-attempt gate back to the FP64 surface.

Device memory is held in torch tensors (plumbing only: every computation is a library kernel).
"""
import ctypes as C

import numpy as np

from . import _lib
from .api import CairError

NINV = _lib.SUR_NINV


def _torch():
    import torch
    return torch


def _stream():
    torch = _torch()
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class Surrogate:
    """Two ensemble members (0 = A drives the dynamics, 1 = B is the gate's second opinion) and the
    constants they share."""

    def __init__(self, device=0):
        torch = _torch()
        if not torch.cuda.is_available():
            raise CairError("the surrogate needs a CUDA device")
        self.lib = _lib.load()
        h = C.c_void_p()
        rc = self.lib.cair_sur_create(C.byref(h), int(device))
        if rc != 0:
            raise CairError("cair_sur_create: %s" % _lib.STATUS.get(rc, rc))
        self.h = h
        self.device = torch.device("cuda", device)
        self.nparam = self.lib.cair_sur_nparam()
        self.history = []

    def check(self, rc, what):
        if rc != 0:
            raise CairError("%s: %s (%s)" % (what, _lib.STATUS.get(rc, rc),
                                             self.lib.cair_sur_last_error(self.h).decode()))

    def close(self):
        if getattr(self, "h", None):
            self.lib.cair_sur_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- constants and parameters --
    def set_consts(self, mu, isd, fmin, fmax, sigma_d=2e-3, gate_ev=1e-3, gate_dmin=1e-3):
        c = _lib.SurConsts()
        for i in range(NINV):
            c.mu[i], c.isd[i], c.fmin[i], c.fmax[i] = float(mu[i]), float(isd[i]), float(fmin[i]), float(fmax[i])
        c.sigma_d, c.gate_ev, c.gate_dmin = float(sigma_d), float(gate_ev), float(gate_dmin)
        self.check(self.lib.cair_sur_set_consts(self.h, C.byref(c)), "cair_sur_set_consts")

    def consts(self):
        c = _lib.SurConsts()
        self.check(self.lib.cair_sur_get_consts(self.h, C.byref(c)), "cair_sur_get_consts")
        return dict(mu=np.array(c.mu[:]), isd=np.array(c.isd[:]), fmin=np.array(c.fmin[:]), fmax=np.array(c.fmax[:]),
                    sigma_d=c.sigma_d, gate_ev=c.gate_ev, gate_dmin=c.gate_dmin)

    def set_params(self, member, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        assert p.size == self.nparam
        self.check(self.lib.cair_sur_set_params(self.h, int(member), p.ctypes.data_as(C.POINTER(C.c_float))),
                   "cair_sur_set_params")

    def params(self, member):
        p = np.zeros(self.nparam, dtype=np.float32)
        self.check(self.lib.cair_sur_get_params(self.h, int(member), p.ctypes.data_as(C.POINTER(C.c_float))),
                   "cair_sur_get_params")
        return p

    def grad(self, member):
        g = np.zeros(self.nparam, dtype=np.float32)
        self.check(self.lib.cair_sur_get_grad(self.h, int(member), g.ctypes.data_as(C.POINTER(C.c_float))),
                   "cair_sur_get_grad")
        return g

    # -- evaluation --
    def eval(self, R):
        """At pair distances R[n][3] (numpy or a CUDA tensor): yA, yB [eV], g = dyA/df [n][16],
        V3 [Eh], dV3/dR [n][3] [Eh/bohr], as numpy arrays."""
        torch = _torch()
        Rt = torch.as_tensor(np.ascontiguousarray(R, dtype=np.float64) if isinstance(R, np.ndarray) else R,
                             dtype=torch.float64, device=self.device).reshape(-1, 3).contiguous()
        n = Rt.shape[0]
        ya = torch.empty(n, dtype=torch.float32, device=self.device)
        yb = torch.empty_like(ya)
        g = torch.empty((n, 16), dtype=torch.float32, device=self.device)
        v3 = torch.empty(n, dtype=torch.float64, device=self.device)
        dv3 = torch.empty((n, 3), dtype=torch.float64, device=self.device)
        self.check(self.lib.cair_sur_eval_dev(self.h, n, C.c_void_p(Rt.data_ptr()), C.c_void_p(ya.data_ptr()),
                                              C.c_void_p(yb.data_ptr()), C.c_void_p(g.data_ptr()),
                                              C.c_void_p(v3.data_ptr()), C.c_void_p(dv3.data_ptr()), _stream()),
                   "cair_sur_eval_dev")
        return ya.cpu().numpy(), yb.cpu().numpy(), g.cpu().numpy(), v3.cpu().numpy(), dv3.cpu().numpy()

    # -- training --
    def grad_step(self, member, samples, idx, w_e, w_f):
        """Adds the gradient of the batch samples[idx] (device tensors) to the member's gradient."""
        self.check(self.lib.cair_sur_grad_dev(self.h, int(member), int(idx.numel()), C.c_void_p(samples.data_ptr()),
                                              C.c_void_p(idx.data_ptr()), float(w_e), float(w_f), _stream()),
                   "cair_sur_grad_dev")

    def adam(self, member, lr):
        self.check(self.lib.cair_sur_adam_dev(self.h, int(member), float(lr), _stream()), "cair_sur_adam_dev")

    def take_loss(self):
        out = np.zeros(2)
        self.check(self.lib.cair_sur_take_loss(self.h, out.ctypes.data_as(C.POINTER(C.c_double)), _stream()),
                   "cair_sur_take_loss")
        return out

    def fit_normalisation(self, R, margin=0.02):
        """Feature normalisation and training range from the training geometries R[n][3]."""
        raw = raw_features_np(R)
        mu = raw.mean(0)
        sd = raw.std(0)
        isd = 1.0 / np.where(sd > 0, sd, 1.0)
        fn = (raw - mu) * isd
        lo, hi = fn.min(0), fn.max(0)
        span = hi - lo
        return mu, isd, lo - margin * span, hi + margin * span

    def train(self, samples, epochs=20, batch=8192, lr0=2e-3, lr1=2e-5, w_e=1.0, w_f=1.0, members=(0, 1),
              seeds=(11, 12), init=True, log_every=1):
        """Adam on both members over `samples` (a CUDA uint8 tensor of cair_sur_sample rows), the
        learning rate decaying geometrically from lr0 to lr1.  Returns the per-epoch mean losses
        [epoch][member][energy, force]."""
        torch = _torch()
        n = samples.numel() // _lib.SUR_SAMPLE_DTYPE.itemsize
        nb = max(1, n // batch)
        total = epochs * nb
        if init:
            for m, sd in zip(members, seeds):
                self.set_params(m, init_params(sd))
        curves = []
        step = 0
        gens = {m: torch.Generator(device=self.device).manual_seed(1000 + m) for m in members}
        for ep in range(epochs):
            row = []
            for m in members:
                perm = torch.randperm(n, generator=gens[m], device=self.device)
                acc = np.zeros(2)
                for b in range(nb):
                    lr = lr0 * (lr1 / lr0) ** (min(step + b, total - 1) / max(1, total - 1))
                    idx = perm[b * batch:(b + 1) * batch]
                    self.grad_step(m, samples, idx, w_e, w_f)
                    self.adam(m, lr)
                acc += self.take_loss()
                row.append(acc / nb)
            step += nb
            curves.append(row)
        self.history.extend(curves)
        return np.array(curves)

    # -- integration --
    def attach(self, handle):
        """Every integrator launch of `handle` (an api.Handle) now runs on the surrogate."""
        handle.check(self.lib.cair_sur_attach(handle.h, self.h), "cair_sur_attach")
        handle._sur = self

    @staticmethod
    def detach(handle):
        handle.check(_lib.load().cair_sur_attach(handle.h, None), "cair_sur_attach")
        handle._sur = None

    def counters(self, reset=False):
        """Gate counters: attempts on the FP64 surface, on the surrogate, range-gated, ensemble-gated."""
        c = np.zeros(4, dtype=np.int64)
        self.check(self.lib.cair_sur_counters(self.h, c.ctypes.data_as(C.POINTER(C.c_int64)), int(bool(reset))),
                   "cair_sur_counters")
        return dict(fp64=int(c[0]), surrogate=int(c[1]), range_gated=int(c[2]), ensemble_gated=int(c[3]))


NH, NF = 128, 16


def init_params(seed):
    """Initial parameters of one member: Glorot-uniform hidden weights (the first layer's bias column
    uniform in +-0.1), zero hidden biases, a Glorot-uniform output row and zero output bias."""
    rng = np.random.default_rng(seed)
    a1 = np.sqrt(6.0 / (NINV + 1 + NH))
    W1 = np.zeros((NH, NF))
    W1[:, :NINV] = rng.uniform(-a1, a1, (NH, NINV))
    W1[:, NF - 1] = rng.uniform(-0.1, 0.1, NH)
    a = np.sqrt(6.0 / (2 * NH))
    W2 = rng.uniform(-a, a, (NH, NH))
    W3 = rng.uniform(-a, a, (NH, NH))
    w4 = rng.uniform(-a, a, NH)
    return np.concatenate([W1.ravel(), W2.ravel(), W3.ravel(), np.zeros(NH), np.zeros(NH), w4, [0.0]]).astype(
        np.float32)


def raw_features_np(R):
    """The ten raw orbit-sum invariants at R[n][3] in float64 (the host's copy of the device feature
    map, used only to fix the normalisation constants)."""
    R = np.asarray(R, dtype=np.float64).reshape(-1, 3)
    d = R * 0.52917721092 - 1.098
    x = np.exp(-d - d * d / 1.5)
    s1 = x.sum(1)
    x2, x3 = x * x, x * x * x
    s2, s3 = x2.sum(1), x3.sum(1)
    p11 = x[:, 0] * x[:, 1] + x[:, 0] * x[:, 2] + x[:, 1] * x[:, 2]
    p111 = x[:, 0] * x[:, 1] * x[:, 2]
    s4 = (x2 * x2).sum(1)
    return np.stack([s1, s2, p11, s3, s2 * s1 - s3, p111, s4, s3 * s1 - s4,
                     x2[:, 0] * x2[:, 1] + x2[:, 0] * x2[:, 2] + x2[:, 1] * x2[:, 2], p111 * s1], 1)


def record_training_set(handle, levels, items, cap, modulus=4, rcut=9.0, max_attempts=None):
    """Runs the queue of `items` on the FP64 surface with the geometry recorder on and returns the
    recorded pair distances as a CUDA float64 tensor [m][3] (m <= cap) and the queue's rows."""
    torch = _torch()
    from .api import RunTrajectories
    lib = handle.lib
    rec = torch.empty((int(cap), 3), dtype=torch.float64, device="cuda")
    handle.check(lib.cair_record_samples(handle.h, C.c_void_p(rec.data_ptr()), int(cap), int(modulus), float(rcut)),
                 "cair_record_samples")
    try:
        rows = RunTrajectories(handle).run(levels, items, max_attempts=max_attempts)
        n = lib.cair_recorded_samples(handle.h)
    finally:
        handle.check(lib.cair_record_samples(handle.h, None, 0, 1, 0.0), "cair_record_samples")
    return rec[:min(int(n), int(cap))].clone(), rows


def targets(handle, R):
    """cair_sur_sample rows (a CUDA uint8 tensor) at the pair distances R (CUDA float64 [n][3]):
    V3 [eV] and dV3/dR [eV/bohr] from the FP64 surface."""
    torch = _torch()
    R = R.contiguous()
    n = R.shape[0]
    out = torch.empty(n * _lib.SUR_SAMPLE_DTYPE.itemsize, dtype=torch.uint8, device=R.device)
    handle.check(handle.lib.cair_sur_targets_dev(handle.h, n, C.c_void_p(R.data_ptr()), C.c_void_p(out.data_ptr()),
                                                 _stream()), "cair_sur_targets_dev")
    return out


def samples_numpy(samples):
    """cair_sur_sample rows of a CUDA uint8 tensor as a numpy structured array."""
    return np.frombuffer(samples.cpu().numpy().tobytes(), dtype=_lib.SUR_SAMPLE_DTYPE)
