"""CPU tests of the C-ABI boundary: the library builds for sm_103a, loads, exports every entry point
declared in include/cair_gpu.h, and the Python mirror of its structs matches the C layout.
No kernel is launched here."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "cair_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cair_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for n in ("cair_create", "cair_destroy", "cair_pes_eval", "cair_rhs", "cair_bs_steps", "cair_integrate",
              "cair_integrate_dev", "cair_find_state", "cair_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol(gpu_lib):
    lib = ctypes.CDLL(gpu_lib)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_bindings_cover_every_declared_symbol():
    from coarseair_gb300 import _lib
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert set(declared_functions()) <= bound


PROBE = r"""
#include <stdio.h>
#include <stddef.h>
#include "cair_gpu.h"
#define P(T, F) printf(#T "." #F " %zu\n", offsetof(T, F))
int main(void) {
  printf("sizeof.cair_system_desc %zu\n", sizeof(cair_system_desc));
  printf("sizeof.cair_pes_desc %zu\n", sizeof(cair_pes_desc));
  printf("sizeof.cair_traj_point %zu\n", sizeof(cair_traj_point));
  P(cair_system_desc, mass); P(cair_system_desc, tpq); P(cair_system_desc, pes); P(cair_system_desc, dt0);
  P(cair_system_desc, nsteps); P(cair_system_desc, nquad); P(cair_system_desc, rsmal); P(cair_system_desc, tthresau);
  P(cair_pes_desc, coef); P(cair_pes_desc, totdiss);
  P(cair_traj_point, b); P(cair_traj_point, vrel); P(cair_traj_point, nmol);
  printf("sizeof.cair_level %zu\n", sizeof(cair_level));
  printf("sizeof.cair_work_item %zu\n", sizeof(cair_work_item));
  printf("sizeof.cair_traj_result %zu\n", sizeof(cair_traj_result));
  printf("sizeof.cair_final_state %zu\n", sizeof(cair_final_state));
  printf("sizeof.cair_stats_params %zu\n", sizeof(cair_stats_params));
  P(cair_level, eint); P(cair_level, ro); P(cair_work_item, first); P(cair_work_item, dinit);
  P(cair_work_item, b_mode); P(cair_work_item, bmin); P(cair_work_item, skip);
  P(cair_final_state, nrings); P(cair_final_state, count); P(cair_final_state, rate_sd);
  P(cair_stats_params, pres_even_odd); P(cair_stats_params, ham_abs_tol); P(cair_stats_params, xmu);
  P(cair_traj_result, status); P(cair_traj_result, bmax); P(cair_traj_result, dH);
  return 0;
}
"""


def test_struct_layout_matches_c(tmp_path):
    from coarseair_gb300 import _lib
    src = tmp_path / "probe.c"
    exe = tmp_path / "probe"
    src.write_text(PROBE)
    r = subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True).stdout.splitlines())
    assert int(out["sizeof.cair_system_desc"]) == ctypes.sizeof(_lib.SystemDesc)
    assert int(out["sizeof.cair_pes_desc"]) == ctypes.sizeof(_lib.PesDesc)
    assert int(out["sizeof.cair_traj_point"]) == ctypes.sizeof(_lib.TrajPoint) == _lib.TRAJ_POINT_DTYPE.itemsize
    assert int(out["sizeof.cair_level"]) == _lib.LEVEL_DTYPE.itemsize
    assert int(out["sizeof.cair_work_item"]) == _lib.ITEM_DTYPE.itemsize
    assert int(out["sizeof.cair_traj_result"]) == _lib.RESULT_DTYPE.itemsize
    assert int(out["sizeof.cair_final_state"]) == _lib.FINAL_STATE_DTYPE.itemsize
    assert int(out["sizeof.cair_stats_params"]) == ctypes.sizeof(_lib.StatsParams)
    dt = {"cair_level": _lib.LEVEL_DTYPE, "cair_work_item": _lib.ITEM_DTYPE, "cair_traj_result": _lib.RESULT_DTYPE,
          "cair_final_state": _lib.FINAL_STATE_DTYPE}
    for key, val in out.items():
        if key.startswith("sizeof"):
            continue
        T, F = key.split(".")
        if T in dt:
            assert dt[T].fields[F][1] == int(val), key
            continue
        cls = {"cair_system_desc": _lib.SystemDesc, "cair_pes_desc": _lib.PesDesc, "cair_traj_point": _lib.TrajPoint,
               "cair_stats_params": _lib.StatsParams}[T]
        assert getattr(cls, F).offset == int(val), key


def test_product_fails_loudly_without_a_gpu(gpu_lib):
    """No CPU fallback: creating a handle without a usable GPU raises."""
    import numpy as np
    from coarseair_gb300 import api, systems
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except Exception:
        pass
    with pytest.raises(api.CairError, match="CAIR_ECUDA"):
        api.Handle(systems.n3_config())


def test_model_constants_match_the_header():
    """The surface and diatomic model numbers the Python side passes are the header's enums."""
    import re
    from coarseair_gb300 import systems
    text = open(os.path.join(ROOT, "include", "cair_gpu.h")).read()
    enums = {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(CAIR_(?:PES|DIAT)_[A-Z0-9_]+)\s*=\s*(\d+)", text)}
    names = {n: getattr(systems, n) for n in dir(systems) if re.match(r"^(PES|DIAT)_[A-Z0-9_]+$", n)}
    assert len(names) == len(enums) == 10
    for n, v in names.items():
        assert enums["CAIR_" + n] == v, n
