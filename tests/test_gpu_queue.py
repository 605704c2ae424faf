"""GPU tests of the device initial-condition sampler and the end-to-end queue path (cair_run_queue)
against the oracle on the same work items."""
import os

import numpy as np
import pytest

from coarseair_gb300 import api, systems

pytestmark = pytest.mark.gpu


def _oracle_levels(table_rows):
    out = np.zeros(len(table_rows), dtype=[(c, "f8") for c in ("vqn", "jqn", "eint", "egam", "rmin", "rmax",
                                                               "vmin", "vmax", "tau", "ri", "ro", "rlim")])
    for c in out.dtype.names:
        out[c] = table_rows[c] if c in table_rows.dtype.names else 0.0
    return out


def _setup(name):
    from oracle import Oracle
    cfg = systems.n3_config(rmax=30.0) if name == "N3" else systems.o3_config()
    o = Oracle(cfg)
    H = api.Handle(cfg, tpq=o.tpq)
    lv = systems.load_levels("N2" if name == "N3" else "O2")
    return cfg, o, H, lv


@pytest.mark.parametrize("name", ["N3", "O3"])
def test_device_initial_conditions_match_oracle(gpu_lib, oracle_lib, name):
    cfg, o, H, lv = _setup(name)
    rows = lv[[0, 17, 250, 1200]] if name == "N3" else lv[[0, 1, 40, 700]]
    table = api.level_table(rows)
    entries = [(i, 0, 24, api.process_seed(3, i + 1), T, 7.0, 15.0) for i, T in enumerate((5000., 10000., 20000., 8000.))]
    items = api.work_items(entries)
    ic = api.InitialConditions(H).sample(table, items)
    for i, (il, _, nt, seed, T, bmax, dinit) in enumerate(entries):
        ref = o.sample_ics(nt, _oracle_levels(rows[il:il + 1]), seed=seed, ttra=T, bmax=bmax, dinit=dinit)
        sl = slice(int(items["first"][i]), int(items["first"][i] + nt))
        for key in ("paq", "paq0", "erra"):
            sc = np.abs(ref[key]).max(axis=1, keepdims=True)
            assert np.all(np.abs(ic[key][sl] - ref[key]) <= 1e-10 * sc), key
        assert np.all(np.abs(ic["H0"][sl] - ref["H0"]) <= 1e-11 * np.maximum(np.abs(ref["H0"]), 0.1))
        assert np.allclose(ic["b"][sl], ref["b"], rtol=1e-14, atol=0)


def test_quasibound_level_consumes_rejection_draws(gpu_lib, oracle_lib):
    """The shipped lists hold no quasi-bound rows; a synthetic one (egam > 0) exercises the
    rejection sampling of ComputeKineticEnergy, whose draws shift the rest of the stream."""
    cfg, o, H, lv = _setup("N3")
    rows = lv[[40]].copy()
    rows["egam"] = 2.0e-3
    rows["vmax"] = rows["eint"] + 1.0e-3
    items = api.work_items([(0, 0, 16, 5, 10000.0, 7.0, 15.0)])
    ic = api.InitialConditions(H).sample(api.level_table(rows), items)
    ref = o.sample_ics(16, _oracle_levels(rows), seed=5, ttra=10000.0, bmax=7.0, dinit=15.0)
    assert np.allclose(ic["b"], ref["b"], rtol=1e-14, atol=0)


@pytest.mark.parametrize("name", ["N3", "O3"])
def test_run_queue_matches_oracle_path(gpu_lib, oracle_lib, name):
    cfg, o, H, lv = _setup(name)
    rows = lv[[3, 60]] if name == "N3" else lv[[1, 30]]
    table = api.level_table(rows)
    entries = [(0, 0, 60, api.process_seed(2, 1), 10000.0, 7.0, 15.0),
               (1, 0, 60, api.process_seed(2, 2), 20000.0, 7.0, 15.0)]
    items = api.work_items(entries)
    res = api.RunTrajectories(H).run(table, items)
    assert np.all(res["status"] == 0)
    assert np.max(np.abs(res["dH"])) < cfg.ham_abs_tol
    Ji, vi, ai = api.histogram_assign(res["j_i"], res["v_i"], res["arr_i"])
    Jf, vf, af = api.histogram_assign(res["j_f"], res["v_f"], res["arr_f"])
    same_f, same_i = [], []
    for i, (il, _, nt, seed, T, bmax, dinit) in enumerate(entries):
        ref = o.sample_ics(nt, _oracle_levels(rows[il:il + 1]), seed=seed, ttra=T, bmax=bmax, dinit=dinit)
        out = o.integrate(ref["paq"], ref["erra"], procs=min(16, os.cpu_count() or 1))
        fi = o.analyze(ref["paq0"])
        ff = o.analyze(o.apply_transformation(out["paq"]))
        sl = slice(int(items["first"][i]), int(items["first"][i] + nt))
        ji, vi_, ai_ = api.histogram_assign([f["angmom"] for f in fi], [f["viba"] for f in fi],
                                            [16 * f["ipair"] + f["itype"] + 0.5 for f in fi])
        jf, vf_, af_ = api.histogram_assign([f["angmom"] for f in ff], [f["viba"] for f in ff],
                                            [16 * f["ipair"] + f["itype"] + 0.5 for f in ff])
        same_i.append((ji == Ji[sl]) & (vi_ == vi[sl]) & (ai_ == ai[sl]))
        same_f.append((jf == Jf[sl]) & (vf_ == vf[sl]) & (af_ == af[sl]))
        assert np.allclose(res["t"][sl][res["status"][sl] == 0] > 0, True)
        assert np.array_equal(res["idx"][sl], np.arange(1, nt + 1))
    assert np.concatenate(same_i).all()
    assert np.concatenate(same_f).mean() >= 0.995
