"""O2 + O on the nine O3 UMN surfaces of the reference's O3 input (degeneracies 1/1/3/3/5/5/1/3/5):
every surface against the oracle at the same points, and a queue run split into contiguous
per-surface blocks as SetPESIndx assigns them, each block drawing the same stream (the reference's
default: every PES stream starts from the same seed)."""
import os

import numpy as np
import pytest

from coarseair_gb300 import api, systems

pytestmark = pytest.mark.gpu
PROCS = min(16, os.cpu_count() or 1)


def _setup():
    from oracle import Oracle
    cfg = systems.o3_mix_config()
    o = Oracle(cfg)
    return cfg, o, api.Handle(cfg, tpq=o.tpq)


def test_nine_surfaces_match_the_oracle(gpu_lib, oracle_lib):
    from test_gpu_parity import _check_rounding_level, _geometries
    cfg, o, H = _setup()
    R, Qall = _geometries(o, 9 * 64, 31)
    ip = np.arange(len(R), dtype=np.int32) % 9
    for k in range(9):
        sel = ip == k
        V_o, g_o, _ = o.compute(R[sel], Qall[sel], ipes=ip[sel])
        V_g, g_g, _ = api.PES(H).Compute(R[sel], Qall[sel], ipes=ip[sel])
        _check_rounding_level(o_k(o, k), R[sel], V_o, g_o, [(V_g, g_g)], systems.O3_MIX[k][0])
    H.close()


class o_k:
    """The oracle's condition scale of surface k for _check_rounding_level."""

    def __init__(self, o, k):
        self.o, self.k = o, k

    def condition_scale(self, R):
        return self.o.condition_scale(R, ipes=np.full(len(R), self.k, np.int32))


def test_degeneracy_blocks_through_the_queue(gpu_lib, oracle_lib):
    cfg, o, H = _setup()
    lv = systems.load_levels("O2")
    row = lv[(lv["vqn"] == 0) & (lv["jqn"] == 1)]
    table = api.level_table(row)
    counts = api.degeneracy_blocks(270, cfg.degeneracy)
    seed = api.process_seed(1, 1)
    items = api.work_items([(0, k, n, seed, 10000.0, 6.0, 15.0) for k, n in enumerate(counts)])
    res = api.RunTrajectories(H).run(table, items)
    assert np.all(res["status"] == 0)
    assert list(np.bincount(res["ipes"], minlength=9)) == counts
    same, stable = [], []
    lvo = np.zeros(1, dtype=[(c, "f8") for c in ("vqn", "jqn", "eint", "egam", "rmin", "rmax", "vmin", "vmax", "tau",
                                                   "ri", "ro", "rlim")])
    for c in lvo.dtype.names:
        lvo[c] = row[c] if c in row.dtype.names else 0.0
    for k, n in enumerate(counts):
        ic = o.sample_ics(n, lvo, seed=seed, ttra=10000.0, bmax=6.0, dinit=15.0)
        ipv = np.full(n, k, np.int32)
        a = o.integrate(ic["paq"], ic["erra"], ipes=ipv, procs=PROCS)
        b = o.integrate(ic["paq"] * (1 + 1e-14), ic["erra"], ipes=ipv, procs=PROCS)
        fa = api.histogram_assign(*[np.array([f[c] for f in o.analyze(o.apply_transformation(a["paq"]))])
                                    for c in ("angmom", "viba")],
                                  np.array([16 * f["ipair"] + f["itype"] + 0.5
                                            for f in o.analyze(o.apply_transformation(a["paq"]))]))
        fb = api.histogram_assign(*[np.array([f[c] for f in o.analyze(o.apply_transformation(b["paq"]))])
                                    for c in ("angmom", "viba")],
                                  np.array([16 * f["ipair"] + f["itype"] + 0.5
                                            for f in o.analyze(o.apply_transformation(b["paq"]))]))
        r = res[res["ipes"] == k]
        fg = api.histogram_assign(r["j_f"], r["v_f"], r["arr_f"])
        same.append((fa[0] == fg[0]) & (fa[1] == fg[1]) & (fa[2] == fg[2]))
        stable.append((fa[0] == fb[0]) & (fa[1] == fb[1]) & (fa[2] == fb[2]))
    same, stable = np.concatenate(same), np.concatenate(stable)
    print("O3 9 surfaces: GPU vs oracle %.4f overall, %.4f on oracle-stable (%.4f stable)" %
          (same.mean(), same[stable].mean(), stable.mean()))
    assert same[stable].mean() >= 0.995
    H.close()
