"""trajectories.out / trajectories_HNotCons.out / trajectories.bin writers (host code in the
library; no GPU).  Expected rows are written out by hand from the reference's format
(I10, A, I5, 2(A, ES11.5), *(A, ES14.8)) (Integrator_Class.F90:933) and Fortran's edit-descriptor
rules: a field too narrow for its value prints as asterisks, a three-digit exponent drops the E."""
import numpy as np

from coarseair_gb300 import _lib, api

HEADER = ("#    iTraj, iPES,       bmax,        b_i,           j_i,           v_i,         arr_i,           j_f,"
          "           v_f,         arr_f\n")


def _rows():
    r = np.zeros(4, dtype=_lib.RESULT_DTYPE)
    r["idx"] = [7, 8, 9, 10]
    r["ipes"] = [0, 2, 0, 0]
    r["bmax"] = 7.0
    r["b"] = [3.25, 0.0, 6.999999999, 1.0e100]
    r["j_i"], r["v_i"], r["arr_i"] = 10.5, 0.5, 16.5
    r["j_f"] = [11.49, 2.0, np.nan, 1.0e-100]
    r["v_f"] = [-1.0, 3.5, 0.5, 12.25]
    r["arr_f"] = [32.5, 16.5, 18.5, 48.5]
    r["status"] = [0, 0, 0, 1]
    r["dH"] = [1e-9, 2e-5, 0.0, 0.0]
    return r


EXPECTED = [
    "         7,    1,7.00000E+00,3.25000E+00,1.05000000E+01,5.00000000E-01,1.65000000E+01,1.14900000E+01,"
    "**************,3.25000000E+01\n",
    "         8,    3,7.00000E+00,0.00000E+00,1.05000000E+01,5.00000000E-01,1.65000000E+01,2.00000000E+00,"
    "3.50000000E+00,1.65000000E+01\n",
    "         9,    1,7.00000E+00,7.00000E+00,1.05000000E+01,5.00000000E-01,1.65000000E+01,           NaN,"
    "5.00000000E-01,1.85000000E+01\n",
    "        10,    1,7.00000E+00,1.00000+100,1.05000000E+01,5.00000000E-01,1.65000000E+01,1.00000000-100,"
    "1.22500000E+01,4.85000000E+01\n",
]


def test_rows_follow_the_reference_format():
    assert api.format_rows(_rows(), header=False) == "".join(EXPECTED)
    assert api.format_rows(_rows()[:1], idx_offset=1000, header=True) == HEADER + EXPECTED[0].replace(
        "         7,", "      1007,")


def test_files_split_by_energy_conservation(tmp_path):
    rows = _rows()
    n_ok, n_not = api.write_trajectories(tmp_path, rows, ham_abs_tol=1e-5, binary=tmp_path / "trajectories.bin")
    assert (n_ok, n_not) == (2, 2)
    assert (tmp_path / "trajectories.out").read_text() == HEADER + EXPECTED[0] + EXPECTED[2]
    assert (tmp_path / "trajectories_HNotCons.out").read_text() == HEADER + EXPECTED[1] + EXPECTED[3]
    raw = (tmp_path / "trajectories.bin").read_bytes()
    assert np.frombuffer(raw[:8], "<i8")[0] == 2
    recs = np.frombuffer(raw[8:], dtype=[("idx", "<i8"), ("ipes", "<i8"), ("v", "<f8", 8)])
    assert list(recs["idx"]) == [7, 9] and list(recs["ipes"]) == [1, 1]
    assert recs["v"][0].tolist() == [7.0, 3.25, 10.5, 0.5, 16.5, 11.49, -1.0, 32.5]


HEADER2 = ("#    iTraj, iPES,       bmax,        b_i,          j1_i,          v1_i,          j2_i,          v2_i,"
           "         arr_i,          j1_f,          v1_f,          j2_f,          v2_f,         arr_f\n")


def _rows2():
    """Two diatom + diatom rows: a four-atom cluster (negative J2, arrangement -65.5) and an exchange."""
    r = np.zeros(2, dtype=_lib.RESULT_DTYPE)
    r["idx"] = [3, 4]
    r["ipes"] = [1, 0]
    r["bmax"] = 8.0
    r["b"] = [2.5, 0.125]
    r["j_i"], r["v_i"], r["j2_i"], r["v2_i"], r["arr_i"] = 1.5, 0.5, 3.5, 1.5, 26.5
    r["j_f"] = [12.25, 40.0]
    r["v_f"] = [0.5, 3.0]
    r["j2_f"] = [-0.5, 7.0]
    r["v2_f"] = [2.5, 0.0]
    r["arr_f"] = [-65.5, 58.5]
    r["status"] = [0, 0]
    r["dH"] = [1e-9, 1e-3]
    return r


EXPECTED2 = [
    "         3,    2,8.00000E+00,2.50000E+00,1.50000000E+00,5.00000000E-01,3.50000000E+00,1.50000000E+00,"
    "2.65000000E+01,1.22500000E+01,5.00000000E-01,**************,2.50000000E+00,**************\n",
    "         4,    1,8.00000E+00,1.25000E-01,1.50000000E+00,5.00000000E-01,3.50000000E+00,1.50000000E+00,"
    "2.65000000E+01,4.00000000E+01,3.00000000E+00,7.00000000E+00,0.00000000E+00,5.85000000E+01\n",
]


def test_two_molecule_rows_follow_the_reference_format():
    assert api.format_rows(_rows2(), header=True, nmol=2) == HEADER2 + "".join(EXPECTED2)


def test_two_molecule_files(tmp_path):
    n_ok, n_not = api.write_trajectories(tmp_path, _rows2(), ham_abs_tol=1e-5, binary=tmp_path / "trajectories.bin",
                                         nmol=2)
    assert (n_ok, n_not) == (1, 1)
    assert (tmp_path / "trajectories.out").read_text() == HEADER2 + EXPECTED2[0]
    assert (tmp_path / "trajectories_HNotCons.out").read_text() == HEADER2 + EXPECTED2[1]
    raw = (tmp_path / "trajectories.bin").read_bytes()
    assert np.frombuffer(raw[:8], "<i8")[0] == 1
    recs = np.frombuffer(raw[8:], dtype=[("idx", "<i8"), ("ipes", "<i8"), ("v", "<f8", 12)])
    assert list(recs["idx"]) == [3] and list(recs["ipes"]) == [2]
    assert recs["v"][0].tolist() == [8.0, 2.5, 1.5, 0.5, 3.5, 1.5, 26.5, 12.25, 0.5, -0.5, 2.5, -65.5]


def test_bad_molecule_count_is_refused():
    import pytest
    with pytest.raises(api.CairError):
        api.format_rows(_rows2(), nmol=3)


def test_merge_follows_merge_trajectories(tmp_path):
    """Two replicas' outputs (plus a directory without output) merge into one trajectories.csv with
    the first header only, HNotCons likewise, and NConvTraj.dat holds the row count."""
    rows = _rows()
    dirs = [tmp_path / "Proc_1", tmp_path / "Proc_2", tmp_path / "Proc_3"]
    for d in dirs:
        d.mkdir()
    api.write_trajectories(dirs[0], rows, ham_abs_tol=1e-5)
    api.write_trajectories(dirs[2], rows[:3], ham_abs_tol=1e-5, idx_offset=1000)
    out = tmp_path / "merged"
    out.mkdir()
    (out / "trajectories_HNotCons.out").write_text("stale\n")
    n = api.merge_trajectories(dirs, out)
    second = [e.replace("         %d," % i, "      %d," % (1000 + i), 1) for e, i in zip(EXPECTED, (7, 8, 9, 10))]
    assert n == 4
    assert (out / "trajectories.csv").read_text() == HEADER + EXPECTED[0] + EXPECTED[2] + second[0] + second[2]
    assert (out / "trajectories_HNotCons.out").read_text() == HEADER + EXPECTED[1] + EXPECTED[3] + second[1]
    assert (out / "NConvTraj.dat").read_text() == "4\n"
    # a later merge appends to the existing trajectories.csv, as the script does
    assert api.merge_trajectories(dirs[:1], out) == 6


def test_empty_inputs(tmp_path):
    """No rows: the files hold the header alone; merging nothing writes NConvTraj.dat = 0."""
    rows = _rows()[:0]
    assert api.format_rows(rows) == HEADER and api.format_rows(rows, header=False) == ""
    assert api.write_trajectories(tmp_path, rows, ham_abs_tol=1e-5, binary=tmp_path / "t.bin") == (0, 0)
    assert (tmp_path / "trajectories.out").read_text() == HEADER
    assert np.frombuffer((tmp_path / "t.bin").read_bytes(), "<i8").tolist() == [0]
    out = tmp_path / "merged"
    out.mkdir()
    assert api.merge_trajectories([], out) == 0
    assert (out / "NConvTraj.dat").read_text() == "0\n" and not (out / "trajectories.csv").exists()


def test_large_files_are_the_rows_in_order(tmp_path):
    """Many chunks' worth of rows (the writer formats them in parallel chunks): each file is the header and
    its rows in their original order, as cair_format_rows formats them one by one."""
    rng = np.random.default_rng(3)
    n = 70001
    r = np.zeros(n, dtype=_lib.RESULT_DTYPE)
    r["idx"] = np.arange(1, n + 1)
    r["ipes"] = rng.integers(0, 9, n)
    r["status"] = np.where(rng.random(n) < 0.02, 1, 0)
    for f in ("bmax", "b", "j_i", "v_i", "arr_i", "j_f", "v_f", "arr_f"):
        r[f] = rng.normal(size=n) * 30
    r["dH"] = rng.normal(size=n) * 1e-5
    ok = (r["status"] == 0) & (np.abs(r["dH"]) <= 1e-5)
    assert api.write_trajectories(tmp_path, r, ham_abs_tol=1e-5, idx_offset=5) == (ok.sum(), n - ok.sum())
    assert (tmp_path / "trajectories.out").read_text() == api.format_rows(r[ok], idx_offset=5)
    assert (tmp_path / "trajectories_HNotCons.out").read_text() == api.format_rows(r[~ok], idx_offset=5)
