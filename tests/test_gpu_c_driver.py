"""The C ABI from a compiled caller: examples/cair_run.c (built with the library) runs N2 + N for two
levels through cair_create / cair_run_queue / cair_write_trajectories, with no Python in the
process, and its trajectories.out matches the Python-bound call on the same inputs row for row."""
import os
import subprocess

import numpy as np
import pytest

from coarseair_gb300 import api, build, systems

pytestmark = pytest.mark.gpu


def test_c_driver_matches_python_binding(gpu_lib, tmp_path):
    exe = build.build_example()
    assert exe and os.path.exists(exe)
    lv = systems.load_levels("N2")[[12, 400]]
    with open(tmp_path / "levels.txt", "w") as f:
        for r in lv:
            f.write(" ".join(repr(float(r[c])) if c not in ("vqn", "jqn") else str(int(r[c]))
                             for c in ("vqn", "jqn", "eint", "egam", "rmin", "rmax", "vmin", "vmax", "tau", "ri", "ro"))
                    + "\n")
    out = tmp_path / "out"
    out.mkdir()
    coef = os.path.join(os.path.dirname(build.__file__), "data", "N3_UMN.dat")
    r = subprocess.run([exe, coef, str(tmp_path / "levels.txt"), str(out), "150", "10000", "11"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert "300 trajectories" in r.stdout
    # the same run through the Python binding
    cfg = systems.n3_config(rmax=16.0)
    H = api.Handle(cfg)
    items = api.work_items([(0, 0, 150, 11, 10000.0, 7.0, 15.0), (1, 0, 150, 13, 10000.0, 7.0, 15.0)])
    rows = api.RunTrajectories(H).run(api.level_table(lv), items)
    ok = (rows["status"] == 0) & (np.abs(rows["dH"]) <= cfg.ham_abs_tol)
    text = (out / "trajectories.out").read_text()
    assert text == api.format_rows(rows[ok])
    H.close()
