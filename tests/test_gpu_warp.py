"""The warp integrator (a warp per trajectory, cair_set_integrator_mode) against the oracle on the GPU.

1. Its lane-parallel right-hand-side and energy programs at phase-space points, under the GPU
   right-hand-side parity criterion (tests/test_warp_host.py runs the same programs on the host).
2. Whole collisions through the persistent warp integrator against the oracle's: final (v, J,
   arrangement) on the oracle-stable trajectories, energy conservation, the device counters.
3. NSteps 2 and 4 (their half-warp schedules differ from NSteps 3's).
4. O3 NN (the networks as programs) end to end, the AUTO mode's choice, and the mode refused where the
   programs do not apply."""
import numpy as np
import pytest

from coarseair_gb300 import api, systems
from test_gpu_parity import PROCS, _final_qn, _gpu_final_qn, _ics, _setup
from test_warp_host import CFGS as HOST_CFGS, DEPTH, U, _phase_points

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", list(HOST_CFGS))
def test_warp_programs_on_the_gpu_match_the_oracle(gpu_lib, oracle_lib, name):
    torch = pytest.importorskip("torch")
    from oracle import Oracle
    cfg = HOST_CFGS[name]()
    o = Oracle(cfg)
    H = api.Handle(cfg, tpq=o.tpq)
    y = _phase_points(o, name, 161, 12)     # odd: a diatom + atom warp ends with one point
    ipes = np.arange(len(y), dtype=np.int32) % len(cfg.surfaces)
    dev = torch.device("cuda")
    yd = torch.from_numpy(np.ascontiguousarray(y)).to(dev)
    ipd = torch.from_numpy(ipes).to(dev)
    ypd = torch.zeros_like(yd)
    Hd = torch.zeros(len(y), dtype=torch.float64, device=dev)
    Rd = torch.zeros((len(y), o.npairs), dtype=torch.float64, device=dev)
    H.check(H.lib.cair_internal_warp_eval(H.h, len(y), ipd.data_ptr(), yd.data_ptr(), ypd.data_ptr(), Hd.data_ptr(),
                                          Rd.data_ptr()), "cair_internal_warp_eval")
    yp, h, ri = ypd.cpu().numpy(), Hd.cpu().numpy(), Rd.cpu().numpy()
    yp_o = o.rhs(y, ipes=ipes)
    R, _ = o.rp(y[:, o.nv:])
    cs = o.condition_scale(R, ipes=ipes)
    ROUND_U = 2 * DEPTH[name] * U
    sc = np.maximum(1e-12 * np.abs(yp_o).max(axis=1, keepdims=True), ROUND_U * cs[:, 1:].max(axis=1, keepdims=True))
    print("%s warp programs on the GPU: worst/bound %.2e" % (name, (np.abs(yp - yp_o) / sc).max()))
    assert np.all(np.abs(yp - yp_o) <= sc)
    h_o, r_o = o.hamiltonian(y, ipes=ipes)
    hs = np.maximum(1e-12 * np.maximum(np.abs(h_o), 0.1), ROUND_U * cs[:, 0])
    assert np.all(np.abs(h - h_o) <= hs)
    assert np.allclose(ri, r_o, rtol=4e-16, atol=0)
    H.close()


def test_warp_integrator_o4_to_the_end(gpu_lib, oracle_lib):
    """O2 + O2 (a whole warp per trajectory, three surfaces): the thread integrator's O4 criterion,
    final points within 1e-6 of the oracle's on its stable trajectories and H conserved."""
    from test_gpu_o4 import _collision_points
    from test_gpu_o4 import _setup as o4_setup
    cfg, o, H = o4_setup()
    H.integrator_mode = "warp"
    y, erra = _collision_points(o, cfg, 32, 13)
    ip = np.arange(len(y), dtype=np.int32) % 3
    ref = o.integrate(y, erra, ipes=ip, procs=PROCS)
    pert = o.integrate(y * (1 + 1e-14), erra, ipes=ip, procs=PROCS)
    tr = api.Trajectories.start(y, erra, cfg.dt0, ipes=ip)
    api.Integrator(H).Integrate(tr)
    assert np.all(tr.status == 0) and np.all(ref["status"] == 0)
    scale = np.abs(ref["paq"]).max(axis=1)
    stable = np.abs(pert["paq"] - ref["paq"]).max(axis=1) / scale < 1e-9
    rel = np.abs(tr.paq - ref["paq"]).max(axis=1) / scale
    print("O4 warp integrator to the end: %d of %d stable, max rel on stable %.2e" % (stable.sum(), len(y),
                                                                                     rel[stable].max()))
    assert stable.sum() >= 4
    assert np.all(rel[stable] < 1e-6)
    h_o, _ = o.hamiltonian(tr.paq, ipes=ip)
    assert np.max(np.abs(tr.H - h_o)) < 1e-9
    assert np.max(np.abs(tr.H - o.hamiltonian(y, ipes=ip)[0])) < cfg.ham_abs_tol
    c = H.counters()
    assert c["attempts"] == int(np.sum(tr.iste + tr.irej))
    H.close()


def _end_to_end(name, n, seed=None, **kw):
    cfg, o, H = _setup(name, **kw)
    H.integrator_mode = "warp"
    assert H.integrator_mode == "warp"
    ic = _ics(o, name, n, seed=seed)
    ref = o.integrate(ic["paq"], ic["erra"], procs=PROCS)
    pert = o.integrate(ic["paq"] * (1 + 1e-14), ic["erra"], procs=PROCS)
    tr = api.Trajectories.start(ic["paq"], ic["erra"], cfg.dt0)
    api.Integrator(H).Integrate(tr)
    assert np.all(tr.status == 0) and np.all(ref["status"] == 0)
    assert np.max(np.abs(tr.H - ic["H0"])) < cfg.ham_abs_tol
    Jo, vo, ao = _final_qn(o.analyze(o.apply_transformation(ref["paq"])))
    Jp, vp, ap = _final_qn(o.analyze(o.apply_transformation(pert["paq"])))
    Jg, vg, ag = _gpu_final_qn(api.MolecularState(H).FindState(api.Collision(H).ApplyTransformation(tr.paq)))
    same = (Jo == Jg) & (vo == vg) & (ao == ag)
    stable = (Jo == Jp) & (vo == vp) & (ao == ap)
    c = H.counters()
    return cfg, H, tr, ref, same, stable, c


@pytest.mark.parametrize("name", ["O3", "N3"])
def test_warp_integrator_end_to_end(gpu_lib, oracle_lib, name):
    """Same bar as the thread integrator's end-to-end test: >= 99.5 % of the oracle-stable
    trajectories end in the oracle's (v, J, arrangement), overall no worse than the oracle's own
    reproducibility minus 1 %; the attempt counters add up."""
    cfg, H, tr, ref, same, stable, c = _end_to_end(name, 400)
    print("%s warp integrator: GPU vs oracle %.4f overall, %.4f on oracle-stable (%.4f stable); attempts %d vs %d" %
          (name, same.mean(), same[stable].mean(), stable.mean(), int(np.sum(tr.iste + tr.irej)),
           int(np.sum(ref["iste"] + ref["irej"])) if "iste" in ref else -1))
    assert same[stable].mean() >= 0.995
    assert same.mean() >= stable.mean() - 0.01
    assert c["attempts"] == int(np.sum(tr.iste + tr.irej))
    assert c["grad_evals"] == 13 * c["attempts"]
    H.close()


@pytest.mark.parametrize("nsteps", [2, 4])
def test_warp_integrator_other_step_counts(gpu_lib, oracle_lib, nsteps):
    cfg, H, tr, ref, same, stable, c = _end_to_end("N3", 64, seed=4321, nsteps=nsteps)
    assert stable.sum() >= 48
    assert np.all(same[stable])
    nseq = {2: 1 + 2 + 4, 4: 1 + 2 + 4 + 6 + 8}[nsteps]
    assert c["grad_evals"] == nseq * c["attempts"]
    H.close()


def test_warp_mode_refused_where_not_built(gpu_lib):
    """An O3 UMN surface given the N2 diatomic: its programs evaluate the O2 curve, so the warp mode is
    refused and the handle stays on the thread integrator."""
    import dataclasses
    cfg = dataclasses.replace(systems.o3_config(), diat_model=systems.DIAT_N2_UMN_FORN4)
    H = api.Handle(cfg)
    with pytest.raises(api.CairError, match="CAIR_EUNSUPPORTED"):
        H.integrator_mode = "warp"
    assert H.integrator_mode == "thread"
    H.close()


def test_warp_integrator_o3_nn_end_to_end(gpu_lib, oracle_lib):
    """O3 NN through the warp integrator (its Compute and Potential networks as programs, tanh as an
    instruction): both sides stop at the same attempt cap, final (v, J, arrangement) and whether the cap
    was reached agree on >= 99.5 % of the oracle-stable trajectories; H is the Potential network's at
    the returned point (the reference's Hamiltonian, which is not conserved for this surface)."""
    from test_gpu_parity import ROUND_U
    cfg, o, H = _setup("O3NN")
    H.integrator_mode = "warp"
    # the thread integrator's O3 NN sample and cap (test_gpu_parity): 400 trajectories, so that one chaotic
    # trajectory the oracle's 1e-14 perturbation misses is within the 0.5 % the bar allows
    n, cap = 400, 30000
    ic = _ics(o, "O3NN", n)
    ref = o.integrate(ic["paq"], ic["erra"], procs=PROCS, max_attempts=cap)
    pert = o.integrate(ic["paq"] * (1 + 1e-14), ic["erra"], procs=PROCS, max_attempts=cap)
    tr = api.Trajectories.start(ic["paq"], ic["erra"], cfg.dt0)
    api.Integrator(H).Integrate(tr, max_attempts=cap)
    assert H.last_integrator == "warp"
    assert np.all(np.isin(tr.status, (0, 1))) and np.all(np.isin(ref["status"], (0, 1)))
    h_o, _ = o.hamiltonian(tr.paq)
    hs = np.maximum(1e-12 * np.maximum(np.abs(h_o), 0.1), ROUND_U * o.condition_scale(o.rp(tr.paq[:, 6:])[0])[:, 0])
    assert np.all(np.abs(tr.H - h_o) <= hs)
    Jo, vo, ao = _final_qn(o.analyze(o.apply_transformation(ref["paq"])))
    Jp, vp, ap = _final_qn(o.analyze(o.apply_transformation(pert["paq"])))
    Jg, vg, ag = _gpu_final_qn(api.MolecularState(H).FindState(api.Collision(H).ApplyTransformation(tr.paq)))
    same = (Jo == Jg) & (vo == vg) & (ao == ag) & (tr.status == ref["status"])
    stable = (Jo == Jp) & (vo == vp) & (ao == ap) & (pert["status"] == ref["status"])
    print("O3NN warp integrator: GPU vs oracle %.4f overall, %.4f on oracle-stable (%.4f stable), %d capped" %
          (same.mean(), same[stable].mean(), stable.mean(), int(np.sum(ref["status"] == 1))))
    assert same[stable].mean() >= 0.995
    assert same.mean() >= stable.mean() - 0.01
    H.close()


def test_auto_mode_picks_by_job_size(gpu_lib, oracle_lib):
    """CAIR_INTEGRATOR_AUTO: a launch below twice the thread integrator's resident lanes runs on the
    warp integrator, a larger one on the thread integrator; both give the same attempt counts as the
    explicit modes on the same trajectories."""
    cfg, o, H = _setup("N3")
    H.integrator_mode = "auto"
    assert H.integrator_mode == "auto"
    ic = _ics(o, "N3", 64, seed=99)
    tr = api.Trajectories.start(ic["paq"], ic["erra"], cfg.dt0)
    api.Integrator(H).Integrate(tr, max_attempts=200)
    assert H.last_integrator == "warp"
    big = 2 * 152 * 8 * 64 + 1     # above twice the resident lanes of any launch shape
    paq = np.repeat(ic["paq"], big // 64 + 1, axis=0)[:big]
    erra = np.repeat(ic["erra"], big // 64 + 1, axis=0)[:big]
    tr2 = api.Trajectories.start(paq, erra, cfg.dt0)
    api.Integrator(H).Integrate(tr2, max_attempts=20)
    assert H.last_integrator == "thread"
    assert np.all(tr2.iste + tr2.irej == 20)
    H.integrator_mode = "thread"
    api.Integrator(H).Integrate(api.Trajectories.start(ic["paq"], ic["erra"], cfg.dt0), max_attempts=20)
    assert H.last_integrator == "thread"
    H.close()


def test_tail_handoff_to_the_warp_integrator(gpu_lib, oracle_lib):
    """AUTO on a launch above twice the thread integrator's resident lanes (a 32 x 1 launch shape keeps 4,864
    lanes): the thread integrator runs it and hands the queue's tail to the warp integrator.  12,000
    trajectories (64 initial conditions of 930 to 11,550 attempts, repeated) capped at 3,000 attempts, against
    the thread integrator alone: a trajectory that never left the thread integrator ran the same arithmetic,
    so at least n - (hand-offs) end bit for bit where the thread run ends; every one conserves H; statuses
    agree; the counters add up.  The queue path (its hand-off buffers carved from the batch) the same way."""
    cfg, o, H = _setup("N3")
    H.check(H.lib.cair_set_launch_shape(H.h, 32, 1), "cair_set_launch_shape")
    ic = _ics(o, "N3", 64, seed=7)
    n, cap = 12000, 3000
    paq, erra = np.resize(ic["paq"], (n, 12)), np.resize(ic["erra"], (n, 12))
    H0 = np.resize(ic["H0"], n)
    H.integrator_mode = "thread"
    ref = api.Trajectories.start(paq, erra, cfg.dt0)
    api.Integrator(H).Integrate(ref, max_attempts=cap)
    H.integrator_mode = "auto"
    tr = api.Trajectories.start(paq, erra, cfg.dt0)
    api.Integrator(H).Integrate(tr, max_attempts=cap)
    handed = H.last_handoffs()
    assert H.last_integrator == "thread"
    c = H.counters()
    assert c["attempts"] == int(np.sum(tr.iste + tr.irej))
    exact = np.all(tr.paq == ref.paq, axis=1) & (tr.iste == ref.iste) & (tr.irej == ref.irej)
    print("tail hand-off: %d of %d trajectories finished on warps; %d end bit for bit as on the thread "
          "integrator alone; statuses equal on %.4f" % (handed, n, int(exact.sum()), np.mean(tr.status == ref.status)))
    assert handed > 0
    assert exact.sum() >= n - handed
    assert np.max(np.abs(tr.H - H0)) < cfg.ham_abs_tol
    assert np.mean(tr.status == ref.status) >= 0.98
    # the queue path
    lv = systems.load_levels("N2")
    table = api.level_table(lv[(lv["vqn"] == 0) & (lv["jqn"] == 10)])
    items = api.work_items([(0, 0, n, api.process_seed(5, 1), 10000.0, 7.0, 15.0)])
    H.integrator_mode = "thread"
    rows_t = api.RunTrajectories(H).run(table, items, max_attempts=cap)
    H.integrator_mode = "auto"
    rows_a = api.RunTrajectories(H).run(table, items, max_attempts=cap)
    handed = H.last_handoffs()
    same = np.ones(n, bool)
    for key in ("j_f", "v_f", "arr_f", "t", "dH", "iste", "irej"):
        same &= rows_a[key] == rows_t[key]
    print("queue path: %d handed off, %d rows bit for bit" % (handed, int(same.sum())))
    assert handed > 0 and same.sum() >= n - handed
    assert np.mean(rows_a["status"] == rows_t["status"]) >= 0.98
    assert np.max(np.abs(rows_a["dH"])) < cfg.ham_abs_tol
    H.close()
