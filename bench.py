#!/usr/bin/env python3
"""Throughput of the trajectory hot path on one GB300: trajectories/s for N2 + N on the N3 UMN surface.

Workload (one "step"): a batch of trajectories over 64 initial (v, J) levels drawn uniformly (seed 2)
from the N2 UMN_ForN4 level list x translational temperatures {5000, 10000, 20000} K (192 work items,
each one state-specific RunTrajectories run with its own random-number stream), b = 7 bohr sqrt(U),
separation 15 bohr, masses 14.0067 amu, plain FP64.  A step samples the initial conditions on the
device, integrates every trajectory to the end of the collision with the persistent queue-refilled
kernel, and analyses the initial and final points into trajectories.out rows.  The default step is
the full 1M-trajectory configuration as one queue: trajectory lengths span 30x (slow collisions run
to tmax), and on GB300 a lone FP64 thread barely speeds up once its SM empties, so the longest
trajectories start at the beginning of the job (the queue is ordered longest-first) and, in the default
AUTO integrator mode, the queue's last trajectories move to the warp integrator (a warp per trajectory)
once fewer are left than it has resident warps.  Steps below twice the thread integrator's resident lanes
(--ntraj, --system o3) run on the warp integrator from the start.

value: device-resident inputs, CUDA events on the launch stream around K steps.
e2e:   the public host entry point cair_run_queue from pinned host buffers (level table and work
       items in, result rows out) with the copies inside the timed region.
cpu_baseline / --impl reference: the CPU oracle (C restatement of the reference path; the reference's
Fortran cannot be built here) on the host cores, one process per core, on a bounded sample of the
same work items.
"""
import argparse
import ctypes
import json
import multiprocessing as mp
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

# DRAM bytes per trajectory of the persistent integrator, measured with ncu (dram__bytes_read.sum +
# dram__bytes_write.sum = 69.13 MB for a 98,304-trajectory launch of this workload); the state is read
# and written once per trajectory, so the full launch's traffic scales with the trajectory count
DRAM_BYTES_PER_TRAJ = 703.0
# --integrator auto (CAIR_INTEGRATOR_AUTO): the library runs a warp per trajectory below twice the lanes the thread
# integrator keeps resident; the autotuner runs for jobs at least this large (twice 152 SMs x 4 warps x 32 lanes)
WARP_MODE_MAX_TRAJ = 2 * 19456

TEMPS = (5000.0, 10000.0, 20000.0)


def workload(ntraj, rank=0, seed_levels=2, nlevels=64, iseed=2, bmax=7.0, dinit=15.0, temps=TEMPS):
    """Level table and work items of the N2 + N configuration.  Replica `rank` draws its streams as
    processes rank * nitems + 1 ... of the run (Collision_Class.F90:295-296), so replicas never repeat
    each other's trajectories."""
    from coarseair_gb300 import api, systems
    lv = systems.load_levels("N2")
    rng = np.random.default_rng(seed_levels)
    pick = np.sort(rng.choice(len(lv), nlevels, replace=False))
    table = api.level_table(lv[pick])
    nitems = nlevels * len(temps)
    base, extra = divmod(ntraj, nitems)
    entries = []
    for il in range(nlevels):
        for it, T in enumerate(temps):
            k = il * len(temps) + it
            n = base + (1 if k < extra else 0)
            entries.append((il, 0, n, api.process_seed(iseed, rank * nitems + k + 1), T, bmax, dinit))
    return table, api.work_items(entries)


def workload_o3(ntraj, rank=0):
    """O2(v=0, J=1) + O on UMN_11A1: one state-specific run, seed 1, 10,000 K, b = 6 sqrt(U) bohr."""
    from coarseair_gb300 import api, systems
    lv = systems.load_levels("O2")
    row = lv[(lv["vqn"] == 0) & (lv["jqn"] == 1)]
    return api.level_table(row), api.work_items([(0, 0, ntraj, api.process_seed(1, rank + 1), 10000.0, 6.0, 15.0)])


def workload_o4(ntraj, rank=0, npairs=64, seed_levels=3):
    """O2 + O2 on the three O4 UMN surfaces: 64 (level, level) pairs drawn uniformly (seed 3) from the
    first 200 O2 levels, 10,000 K, b = 8 sqrt(U) bohr, Dinit 18 bohr; each pair's trajectories are
    split over the singlet, triplet and quintet surfaces in proportion to their degeneracies 1:3:5
    (contiguous blocks per surface, Collision_Class.F90:2468-2507)."""
    from coarseair_gb300 import api, systems
    lv = systems.load_levels("O2")[:200]
    rng = np.random.default_rng(seed_levels)
    pairs = rng.integers(0, 200, size=(npairs, 2))
    table = api.level_table(lv)
    per_pair = [ntraj // npairs + (1 if k < ntraj % npairs else 0) for k in range(npairs)]
    entries = []
    for k, (a, b) in enumerate(pairs):
        n = per_pair[k]
        split = [n * 1 // 9, n * 3 // 9]
        split.append(n - split[0] - split[1])
        for ip in range(3):
            entries.append((int(a), ip, split[ip], api.process_seed(3, rank * 3 * npairs + 3 * k + ip + 1), 10000.0,
                            8.0, 18.0, int(b)))
    return table, api.work_items(entries)


def config(system="n3"):
    """System of the workload.  N3 and O3 use the end-of-collision criterion stated for the atom-diatom
    configurations (any pair beyond 16 bohr, attempt cap 1e6); O4 the reference's O4 input
    (35 bohr, tmax 5e5)."""
    from coarseair_gb300 import systems
    if system == "o3":
        return systems.o3_config(dinit=15.0, bmax=6.0, rmax=16.0)
    if system == "o4":
        return systems.o4_config()
    return systems.n3_config(dinit=15.0, bmax=7.0, rmax=16.0, tmax=4.0e5)


SYSTEMS = {
    "n3": dict(workload=workload, ntraj=1000000,
               text="N2+N on N3 UMN (N4 PIP), plain FP64: 64 levels (seed 2) x {5000,10000,20000} K, "
                    "b = 7 sqrt(U) bohr, Dinit 15 bohr, rmax 16 bohr, m = 14.0067 amu"),
    "o3": dict(workload=workload_o3, ntraj=10000,
               text="O2(v=0,J=1)+O on O3 UMN_11A1, plain FP64: seed 1, 10000 K, b = 6 sqrt(U) bohr, Dinit 15 bohr, "
                    "rmax 16 bohr, m = 15.9994 amu"),
    "o4": dict(workload=workload_o4, ntraj=500000,
               text="O2+O2 on O4 UMN singlet/triplet/quintet (1:3:5), plain FP64: 64 level pairs from the first 200 "
                    "O2 levels (seed 3), 10000 K, b = 8 sqrt(U) bohr, Dinit 18 bohr, rmax 35 bohr, m = 15.9994 amu"),
}


# ------------------------------------------------------------------------------------------------
# CPU side: the oracle on host cores (one process per core, spawned before any GPU work)
# ------------------------------------------------------------------------------------------------
def _oracle_level(table, il):
    lv = table[il:il + 1]
    lvs = np.zeros(1, dtype=[(c, "f8") for c in ("vqn", "jqn", "eint", "egam", "rmin", "rmax", "vmin", "vmax",
                                                   "tau", "ri", "ro", "rlim")])
    for c in lvs.dtype.names:
        lvs[c] = lv[c] if c in lv.dtype.names else 0.0
    return lvs


def _cpu_worker(args):
    items, table, wall, system = args
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle
    o = Oracle(config(system))
    done, t0 = 0, time.perf_counter()
    for (il, ntraj, seed, ttra, bmax, dinit, ipes, il2) in items:
        if system == "o4":
            ic = o.sample_ics4(ntraj, _oracle_level(table, il)[0], _oracle_level(table, il2)[0], ttra=ttra,
                               bmax=bmax, dinit=dinit, seed=seed)
        else:
            ic = o.sample_ics(ntraj, _oracle_level(table, il), seed=seed, ttra=ttra, bmax=bmax, dinit=dinit)
        for k in range(ntraj):
            res = o.integrate(ic["paq"][k:k + 1], ic["erra"][k:k + 1], ipes=np.array([ipes], np.int32))
            o.analyze(ic["paq0"][k:k + 1])
            o.analyze(o.apply_transformation(res["paq"]))
            done += 1
            if time.perf_counter() - t0 > wall:
                return done, time.perf_counter() - t0
    return done, time.perf_counter() - t0


def cpu_baseline(table, items, cores, wall, system="n3"):
    """Trajectories/s of the oracle on `cores` processes, each running trajectories of its own
    work items for about `wall` seconds (a bounded sample of the same workload)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    per = [[] for _ in range(cores)]
    if len(items) >= cores:
        for k, it in enumerate(items):
            per[k % cores].append((int(it["ilevel"]), int(it["ntraj"]), int(it["seed"]), float(it["ttra"]),
                                   float(it["bmax"]), float(it["dinit"]), int(it["ipes"]), int(it["ilevel2"])))
    else:  # fewer items than cores: every process runs the first item's stream from its own seed
        it = items[0]
        for k in range(cores):
            per[k].append((int(it["ilevel"]), int(it["ntraj"]), int(it["seed"]) + 2 * k, float(it["ttra"]),
                           float(it["bmax"]), float(it["dinit"]), int(it["ipes"]), int(it["ilevel2"])))
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        out = pool.map(_cpu_worker, [(p, table, wall, system) for p in per])
    n = sum(o[0] for o in out)
    t = max(o[1] for o in out)
    return n / t, n, t


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


# ------------------------------------------------------------------------------------------------
# clocks during the timed region
# ------------------------------------------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, path):
        self.path = path
        self.p = None

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
            self.f.close()

    def summary(self):
        if not self.p or not os.path.exists(self.path):
            return None
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9 or not f[0].isdigit():
                continue
            try:
                sm.append(float(f[1].split()[0]))
                mx = float(f[2].split()[0])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------------------------------------
def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--system", default="n3", choices=sorted(SYSTEMS),
                    help="n3: N2+N 1M (the headline); o3: O2+O 10k; o4: O2+O2 500k")
    ap.add_argument("--ntraj", type=int, default=None, help="trajectories per step (one queue)")
    ap.add_argument("--inflight", type=int, default=1, help="steps in flight on separate streams")
    ap.add_argument("--e2e-ntraj", type=int, default=None, help="trajectories of the e2e host call")
    ap.add_argument("--max-attempts", type=int, default=1000000)
    ap.add_argument("--cpu-wall", type=float, default=20.0, help="seconds of CPU work per core for the baseline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--clocks-csv", default=None, help="keep the nvidia-smi clock samples of the timed region here")
    ap.add_argument("--surrogate", default="on", choices=["on", "off", "only"],
                    help="the learned-surrogate arm (N2 + N): trained on the GPU, then timed on the same queue")
    ap.add_argument("--sur-train-ntraj", type=int, default=200000,
                    help="FP64 trajectories at 10,000 K whose end-check geometries form the training set")
    ap.add_argument("--sur-cap", type=int, default=20000000, help="training geometries kept")
    ap.add_argument("--sur-epochs", type=int, default=12)
    ap.add_argument("--sur-steps", type=int, default=1, help="timed surrogate steps")
    ap.add_argument("--integrator", default="auto", choices=["auto", "thread", "warp"],
                    help="persistent integrator: a lane per trajectory (thread), a warp per trajectory (warp), or "
                         "the library's choice by job size, with the thread integrator's tail on warps (auto)")
    args = ap.parse_args()
    spec = SYSTEMS[args.system]
    if args.ntraj is None:
        args.ntraj = spec["ntraj"]
    if args.e2e_ntraj is None:
        args.e2e_ntraj = args.ntraj

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    table, items = spec["workload"](args.ntraj, rank)
    cores = host_cores()
    metric = "trajectories/s"
    cfg_json = {"workload": spec["text"],
                "trajectories_per_step": int(args.ntraj), "work_items": int(len(items)),
                "full_config_trajectories": spec["ntraj"], "parallelism": "replicas" if world > 1 else "single",
                "l2": "inputs stay resident; each step re-samples initial conditions and rewrites all state "
                      "(state per step %.0f MB, above the 129 MB L2 from 1M trajectories)" % (args.ntraj * 0.4e-3)}

    if args.impl == "reference":
        if rank != 0:
            return
        K, W = args.steps, args.warmup
        times, total = [], 0
        for s in range(W + K):
            rate, n, t = cpu_baseline(table, items, cores, max(2.0, args.cpu_wall / 4), args.system)
            if s >= W:
                times.append(t)
                total += n
        value = total / sum(times)
        line = {"impl": "reference", "metric": metric, "value": value, "unit": "trajectories/s", "n_gpus": 0,
                "steps": K, "warmup": W, "ms_per_step": 1e3 * sum(times) / K, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": cfg_json,
                "cpu_baseline": {"value": value, "unit": "trajectories/s", "cores": cores, "kind": "port",
                                 "sample": "each step: %d processes x ~%.0f s of the same work items "
                                           "(C restatement of the reference CPU path)" % (cores, max(2.0, args.cpu_wall / 4))},
                "e2e": {"value": value, "unit": "trajectories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    # CPU baseline first (spawned processes before any GPU call)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        rate, n, t = cpu_baseline(table, items, cores, args.cpu_wall, args.system)
        cpu = {"value": rate, "unit": "trajectories/s", "cores": cores, "kind": "port",
               "sample": "%d trajectories of the same work items in %.1f s on %d processes "
                         "(C restatement of the reference CPU path, -O3 no FMA)" % (n, t, cores)}

    import torch
    from coarseair_gb300 import api, _lib
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dev = torch.device("cuda", torch.cuda.current_device())
    cfg = config(args.system)
    H = api.Handle(cfg)
    lib = H.lib
    n = int(items["ntraj"].sum())
    d_lv = torch.from_numpy(table.view(np.uint8).copy()).to(dev)
    d_it = torch.from_numpy(items.view(np.uint8).copy()).to(dev)
    # several batches in flight on their own streams: later steps fill the SMs that an earlier
    # step's longest trajectories leave idle
    ws_bytes = int(lib.cair_queue_workspace_bytes(n))
    streams = [torch.cuda.Stream(device=dev) for _ in range(max(1, args.inflight))]
    ws = [torch.empty(ws_bytes + 256, dtype=torch.uint8, device=dev) for _ in streams]
    res_bufs = [torch.empty(n * _lib.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=dev) for _ in streams]

    def aligned(t):
        p = t.data_ptr()
        return (p + 255) & ~255

    mode = args.integrator
    # the project's autotuner picks the thread integrator's launch shape on a capped sample of this job
    # (in THREAD mode: AUTO would hand the sample's tail to the warp integrator)
    H.integrator_mode = "thread"
    tune = None
    runs_thread = mode == "thread" or (mode == "auto" and n >= WARP_MODE_MAX_TRAJ)
    if runs_thread and args.surrogate != "only" and (args.system != "o4" or args.ntraj <= 200000):
        # eight times the most lanes any shape keeps resident (152 SMs x 8 warps x 32), so that every
        # shape's sample runs in several full rounds of its lanes
        ns = min(n, 8 * 38912)
        shape, pts = api.autotune(H, table, items, sample=ns, cap_attempts=100)
        tune = {"block": shape[0], "blocks_per_sm": shape[1],
                "points": [[int(p["block"]), int(p["per_sm"]), float(p["attempts_per_s"])] for p in pts],
                "sample": "%d trajectories of the job's items, each capped at 100 attempts" % ns}

    # CAIR_INTEGRATOR_AUTO: a warp per trajectory below twice the thread integrator's resident lanes; above,
    # a lane per trajectory that hands the queue's tail to the warp integrator
    H.integrator_mode = mode

    def step(i):
        j = i % len(streams)
        H.check(lib.cair_run_queue_dev(H.h, len(table), d_lv.data_ptr(), len(items), d_it.data_ptr(), n,
                                       args.max_attempts, res_bufs[j].data_ptr(), aligned(ws[j]),
                                       streams[j].cuda_stream), "cair_run_queue_dev")

    if args.surrogate == "only":
        # the surrogate arm alone (a profiling command): no plain timing, no rate comparison
        out = surrogate_arm(args, H, table, items, None, rank)
        if rank == 0:
            print(json.dumps({"surrogate": out}))
        return
    for i in range(args.warmup):
        step(i)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = Clocks(args.clocks_csv or os.path.join(tempfile.gettempdir(), "bench_clocks_%d.csv" % os.getpid()))
    ev0 = torch.cuda.Event(enable_timing=True)
    ev_end = [torch.cuda.Event(enable_timing=True) for _ in streams]
    H.check(lib.cair_set_integrate_timing(H.h, 1), "cair_set_integrate_timing")
    # the integrator's warp timeline (start and end of every warp of the launch) for the tail figures
    wt = torch.zeros(4 * 65536, dtype=torch.int64, device=dev)
    H.check(lib.cair_set_warp_timeline(H.h, wt.data_ptr(), 65536), "cair_set_warp_timeline")
    with clocks:
        torch.cuda.synchronize()
        ev0.record(streams[0])
        for st in streams[1:]:
            st.wait_event(ev0)
        for i in range(args.steps):
            step(i)
        for e, st in zip(ev_end, streams):
            e.record(st)
        torch.cuda.synchronize()
    ms = max(ev0.elapsed_time(e) for e in ev_end)
    # the persistent integrator's own launches, timed by the library with events on their stream
    kt = (ctypes.c_float * max(1, args.steps))()
    nk = ctypes.c_int32(0)
    H.check(lib.cair_integrate_timings(H.h, kt, args.steps, ctypes.byref(nk)), "cair_integrate_timings")
    H.check(lib.cair_set_integrate_timing(H.h, 0), "cair_set_integrate_timing")
    integ_ms = float(np.mean(list(kt)[:nk.value]))
    ran = H.last_integrator
    handoffs = H.last_handoffs() if ran == "thread" else 0
    nw = int(lib.cair_warp_timeline_count(H.h))
    H.check(lib.cair_set_warp_timeline(H.h, None, 0), "cair_set_warp_timeline")
    tail = tail_figures(wt[:4 * nw].cpu().numpy().reshape(-1, 4)) if nw else None
    if world > 1:
        ms = max_over_ranks(ms, dist, torch.tensor([0.0], device=dev))
    value = aggregate_rate(n, args.steps, world, ms)
    res = np.frombuffer(res_bufs[(args.steps - 1) % len(streams)].cpu().numpy().tobytes(), dtype=_lib.RESULT_DTYPE)
    per_traj = res["iste"].astype(np.int64) + res["irej"]
    att = int(np.sum(per_traj))
    counters = {"attempts": att, "grad_evals": 13 * att, "energy_evals": att // cfg.ncall}
    fm = H.flop_model()
    flops_step = (counters["grad_evals"] * fm["grad"] + counters["energy_evals"] * fm["energy"] +
                  counters["attempts"] * fm["attempt"])

    # e2e through the host entry point with pinned buffers
    e2e = None
    if not args.no_e2e:
        etab, eitems = spec["workload"](args.e2e_ntraj, rank)
        ne = int(eitems["ntraj"].sum())
        pin_res = torch.empty(ne * _lib.RESULT_DTYPE.itemsize, dtype=torch.uint8, pin_memory=True)
        pin_lv = torch.from_numpy(etab.view(np.uint8).copy()).pin_memory()
        pin_it = torch.from_numpy(eitems.view(np.uint8).copy()).pin_memory()
        t0 = time.perf_counter()
        H.check(lib.cair_run_queue(H.h, len(etab), pin_lv.data_ptr(), len(eitems), pin_it.data_ptr(), ne,
                                   args.max_attempts, pin_res.data_ptr()), "cair_run_queue")
        t1 = time.perf_counter()
        e2e = {"value": ne / (t1 - t0), "unit": "trajectories/s", "steps": 1, "trajectories": ne,
               "note": "one synchronous cair_run_queue call on a %d-trajectory job, host buffers pinned" % ne,
               "h2d_bytes_per_step": int(etab.nbytes + eitems.nbytes),
               "d2h_bytes_per_step": int(ne * _lib.RESULT_DTYPE.itemsize)}

    # dominant kernel: the persistent integrator; its share of the step is measured in profiles/
    peak_fp64 = fp64_peak_probe(lib, H)
    ms_step = ms / args.steps
    achieved = flops_step / (integ_ms / 1e3) / 1e12
    line = {"metric": metric, "value": value, "unit": "trajectories/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg_json,
            "gpu_launches": (9 if handoffs else 8) * args.steps,
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak_fp64["tflops"], "unit": "TFLOP/s",
                         "frac": achieved / peak_fp64["tflops"],
                         "traffic": DRAM_BYTES_PER_TRAJ * n if args.system == "n3" else None,
                         "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of one ncu capture of a "
                                           "98,304-trajectory launch (703 B per trajectory), scaled by trajectories"
                                           if args.system == "n3" else "not captured for this system",
                         "peak_source": peak_fp64["source"],
                         "kernel": ("k_integrate (persistent Bulirsch-Stoer integrator, a lane per trajectory)" +
                                    (", its tail on k_integrate_warp" if handoffs else ""))
                                   if ran == "thread" else
                                   "k_integrate_warp (persistent Bulirsch-Stoer integrator, a warp per trajectory)",
                         "kernel_ms_per_launch": integ_ms, "kernel_share_of_step": integ_ms * args.steps / ms,
                         "work": "executed FP64 operations of the pruned formulation per step "
                                 "(exp, division and sqrt counted as one operation each)"},
            "pes_evals_per_s": counters["grad_evals"] / (ms_step / 1e3),
            "attempts_per_trajectory": counters["attempts"] / n,
            "attempts_per_trajectory_quantiles": {q: int(np.quantile(per_traj, float(q))) for q in
                                                  ("0.5", "0.9", "0.99", "0.999", "1.0")},
            "inflight_batches": len(streams),
            "integrator": {"mode": mode, "ran": ran, "tail_handoffs": handoffs},
            "autotune": tune,
            "tail": tail,
            "converged_fraction": float(np.mean(res["status"] == 0)),
            "energy_not_conserved_fraction": float(np.mean(np.abs(res["dH"]) > cfg.ham_abs_tol))}
    line.update(outcome_summary(res, cfg.ncall))
    if args.surrogate == "on" and args.system == "n3":
        sur = surrogate_arm(args, H, table, items, res, rank)
        sur["vs_plain"]["throughput_ratio"] = sur["value"] / value
        line["surrogate"] = sur
    if e2e:
        line["e2e"] = e2e
    if cpu:
        line["cpu_baseline"] = cpu
    cs = clocks.summary()
    if cs:
        line["clocks"] = cs
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


EV_PER_EH = 27.211386245988


def surrogate_arm(args, H, table, items, plain_res, rank):
    """The learned surrogate on the N2 + N queue.  Training set: the end-check geometries of
    args.sur_train_ntraj FP64 trajectories at 10,000 K over the same 64 levels (streams of seed 4),
    with FP64 three-body targets; both ensemble members trained on the GPU.  Then args.sur_steps
    timed steps of the same queue as the plain arm with the surrogate attached (device-resident
    inputs, CUDA events), judged against the plain arm's rows: per-trajectory energy drift on the FP64
    surface, the attempts the gate sent to FP64, and every final state's rate within 2 sigma."""
    import torch
    from coarseair_gb300 import _lib, api, surrogate
    lib = H.lib
    dev = torch.device("cuda", torch.cuda.current_device())
    ttab, titems = workload(args.sur_train_ntraj, rank, iseed=4, temps=(10000.0,))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    R, _ = surrogate.record_training_set(H, ttab, titems, cap=args.sur_cap, modulus=2, rcut=9.0,
                                         max_attempts=args.max_attempts)
    smp = surrogate.targets(H, R)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    S = surrogate.Surrogate()
    sub = R[torch.randperm(R.shape[0], device=R.device)[:min(R.shape[0], 2000000)]].cpu().numpy()
    mu, isd, lo, hi = S.fit_normalisation(sub)
    S.set_consts(mu, isd, lo, hi)
    t0 = time.perf_counter()
    curves = S.train(smp, epochs=args.sur_epochs, batch=32768, lr0=3e-3, lr1=2e-5)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del smp
    n = int(items["ntraj"].sum())
    d_lv = torch.from_numpy(table.view(np.uint8).copy()).to(dev)
    d_it = torch.from_numpy(items.view(np.uint8).copy()).to(dev)
    ws = torch.empty(int(lib.cair_queue_workspace_bytes(n)) + 256, dtype=torch.uint8, device=dev)
    res_buf = torch.empty(n * _lib.RESULT_DTYPE.itemsize, dtype=torch.uint8, device=dev)
    st = torch.cuda.Stream(device=dev)
    S.attach(H)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    S.counters(reset=True)
    torch.cuda.synchronize()
    ev0.record(st)
    for _ in range(args.sur_steps):
        H.check(lib.cair_run_queue_dev(H.h, len(table), d_lv.data_ptr(), len(items), d_it.data_ptr(), n,
                                       args.max_attempts, res_buf.data_ptr(), (ws.data_ptr() + 255) & ~255,
                                       st.cuda_stream), "cair_run_queue_dev (surrogate)")
    ev1.record(st)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.sur_steps
    gate = S.counters()
    S.detach(H)
    rows = np.frombuffer(res_buf.cpu().numpy().tobytes(), dtype=_lib.RESULT_DTYPE)
    de = np.abs(rows["dH"]) * EV_PER_EH
    att = rows["iste"].astype(np.int64) + rows["irej"]
    out = {"value": n / (ms / 1e3), "unit": "trajectories/s", "steps": args.sur_steps, "ms_per_step": ms,
           "attempts_per_trajectory": float(att.mean()),
           "dE_eV": {"median": float(np.median(de)), "p90": float(np.quantile(de, 0.9)), "max": float(de.max())},
           "fp64_attempt_fraction": gate["fp64"] / max(1, gate["fp64"] + gate["surrogate"]),
           "gate": gate, "converged_fraction": float(np.mean(rows["status"] == 0)),
           "training": {"geometries": int(R.shape[0]), "record_and_targets_s": t_data, "train_s": t_train,
                        "epochs": args.sur_epochs, "batch": 32768,
                        "final_loss_member_A": [float(x) for x in curves[-1][0]],
                        "final_loss_member_B": [float(x) for x in curves[-1][1]],
                        "loss_curve_A": [[float(x) for x in c[0]] for c in curves]},
           "precision": "hidden layers: BF16 weights, activations split exactly into three BF16 parts, FP32 "
                        "accumulation (tcgen05); FP32 output layer; FP64 integrator state, diatomics, gate "
                        "fallback and energy check"}
    out["hnotcons_fraction_at_reference_tolerance"] = float(np.mean(np.abs(rows["dH"]) > H.cfg.ham_abs_tol))
    if plain_res is not None:
        # both runs' rows counted with a tolerance above the surrogate's drift (its fit error, reported
        # as dE_eV), so that the rates compare the same trajectories
        sp = api.Statistics(H, pres_even_odd=(1, 0, 0), ham_abs_tol=1e-3)
        a = {(int(r["run"]),) + tuple(int(x) for x in r["fin"][:3]): (r["rate"], r["rate_sd"])
             for r in sp.compute(items, plain_res)}
        b = {(int(r["run"]),) + tuple(int(x) for x in r["fin"][:3]): (r["rate"], r["rate_sd"])
             for r in sp.compute(items, rows)}
        z = []
        for k in set(a) | set(b):
            ka, sa = a.get(k, (0.0, 0.0))
            kb, sb = b.get(k, (0.0, 0.0))
            s2 = np.hypot(sa, sb)
            if s2 > 0:
                z.append(abs(ka - kb) / s2)
        z = np.array(z)
        pde = np.abs(plain_res["dH"]) * EV_PER_EH
        out["vs_plain"] = {"rates_compared": int(len(z)), "beyond_2_sigma": int(np.sum(z > 2.0)),
                           "rates_ham_abs_tol_eh": 1e-3,
                           "fraction_beyond_2_sigma": float(np.mean(z > 2.0)) if len(z) else 0.0,
                           "plain_dE_eV_median": float(np.median(pde))}
    S.close()
    return out


def tail_figures(t):
    """Queue-tail figures of one integrator launch from its warp timeline t[warp] = (start [ns], end [ns],
    lane-blocks, blocks):
    the fraction of warp-time idle after each warp ran out of work (launch length x warps - busy time),
    and when (as fractions of the launch) 90 %, 50 % and 10 % of the warps were still busy."""
    t = t.astype(np.float64)
    t0, t1 = t[:, 0].min(), t[:, 1].max()
    T = t1 - t0
    busy = (t[:, 1] - t0) / T
    q = np.sort(busy)[::-1]
    at = lambda f: float(q[min(len(q) - 1, int(f * len(q)))])
    # lanes without a trajectory inside busy warps, weighted by ncall-attempt blocks (an attempt costs
    # the same whatever the trajectory, so blocks measure time)
    lane_idle = float(1.0 - t[:, 2].sum() / (32.0 * t[:, 3].sum()))
    return {"warps": int(len(t)), "launch_ms": T / 1e6, "idle_warp_time_fraction": float(1.0 - busy.mean()),
            "idle_lane_time_fraction_in_busy_warps": lane_idle,
            "time_fraction_when_busy_warps_fall_to": {"90%": at(0.1), "50%": at(0.5), "10%": at(0.9)},
            "source": "%globaltimer at each warp's start and at its last lane's end (cair_set_warp_timeline)"}


def max_over_ranks(value, dist, buf):
    """The slowest replica's time: all_reduce(MAX) of one number through the tensor `buf` (a CUDA tensor
    under NCCL, a CPU tensor under gloo)."""
    buf.fill_(float(value))
    dist.all_reduce(buf, op=dist.ReduceOp.MAX)
    return float(buf.item())


def outcome_summary(res, ncall):
    """Outcome figures of one step's result rows: the fraction of trajectories that ended at the first
    end check, i.e. after ncall attempts (with Dinit 15 and rmax 16 bohr a pair can start beyond rmax,
    Integrator_Class.F90:441-465), and, with more than one surface, per surface the trajectories, their
    mean attempts and the converged fraction."""
    per_traj = res["iste"].astype(np.int64) + res["irej"]
    out = {"first_check_fraction": float(np.mean((per_traj <= ncall) & (res["status"] == 0)))}
    surfaces = np.unique(res["ipes"])
    if len(surfaces) > 1:
        out["per_surface"] = {
            str(int(p)): {"trajectories": int(np.sum(res["ipes"] == p)),
                          "attempts_per_trajectory": float(per_traj[res["ipes"] == p].mean()),
                          "converged_fraction": float(np.mean(res["status"][res["ipes"] == p] == 0))}
            for p in surfaces}
    return out


def aggregate_rate(ntraj_per_rank, steps, world, ms):
    """Whole-job trajectories/s: every replica's trajectories over the slowest replica's time."""
    return ntraj_per_rank * steps * world / (ms / 1e3)


def fp64_peak_probe(lib, H):
    """FP64 FMA throughput of this GPU, measured live (MEASURED_PEAKS.json carries bf16 and HBM only)."""
    import ctypes
    g = ctypes.c_double()
    rc = lib.cair_fp64_peak_probe(H.h, ctypes.byref(g))
    if rc == 0 and g.value > 0:
        return {"tflops": g.value / 1e3, "source": "live DFMA probe (cair_fp64_peak_probe)"}
    return {"tflops": 1.2, "source": "fallback"}


if __name__ == "__main__":
    main()
