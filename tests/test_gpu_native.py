"""Compiled callers of the library through include/ alone (tests/native/, built by
the package build): a C program on chimes_gb300.h and a C++ program on the ZCalc /
ZCalc_Deriv drop-ins of chimes_gb300_zcalc.hpp, run as separate processes.

Checked against the reference's fixtures: the design matrix of tests/golden/water3b
(reference chimes_lsq's A; 1e-12 of the entry and its column's scale) and the MD
forces of tests/golden/md_ch4b (reference chimes_md's first-step forces; 1e-10 of
the largest component).
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _write_frame(path, types, xyz, cell):
    with open(path, "wb") as f:
        f.write(np.int32(len(types)).tobytes())
        f.write(np.ascontiguousarray(types, dtype=np.int32).tobytes())
        f.write(np.ascontiguousarray(xyz, dtype=np.float64).tobytes())
        f.write(np.ascontiguousarray(cell, dtype=np.float64).reshape(9).tobytes())


def _write_coef(path, x):
    with open(path, "wb") as f:
        f.write(np.int32(len(x)).tobytes())
        f.write(np.ascontiguousarray(x, dtype=np.float64).tobytes())


def _close(A, R):
    colmax = np.abs(R).max(axis=0)
    return bool(np.all(np.abs(A - R) <= 1e-12 * np.abs(R) + 1e-12 * colmax[None, :]))


@pytest.fixture(scope="module")
def programs(cg):
    cg.build()
    d = os.path.dirname(cg.LIB_PATH)
    p = {n: os.path.join(d, n) for n in ("capi_check", "zcalc_check")}
    for v in p.values():
        assert os.path.exists(v), v
    return p


@pytest.fixture(scope="module")
def md_inputs(tmp_path_factory):
    d = np.load(os.path.join(GOLDEN, "md_ch4b", "md_ref.npz"))
    tmp = tmp_path_factory.mktemp("native")
    _write_frame(tmp / "md_frame.bin", d["types"], d["xyz"], d["cell"])
    _write_coef(tmp / "md_coef.bin", d["x"])
    return tmp, d


def test_c_program_assembles_and_evaluates_forces(programs, md_inputs):
    tmp, md = md_inputs
    r = subprocess.run([programs["capi_check"], os.path.join(GOLDEN, "water3b", "fm_setup.in"), str(tmp / "A.bin"),
                        os.path.join(GOLDEN, "md_ch4b", "fm_setup.in"), str(tmp / "md_frame.bin"),
                        str(tmp / "md_coef.bin"), str(tmp / "F.bin")], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    raw = open(tmp / "A.bin", "rb").read()
    rows, cols = np.frombuffer(raw[:16], dtype=np.int64)
    A = np.frombuffer(raw[16:], dtype=np.float64).reshape(rows, cols)
    R = np.load(os.path.join(GOLDEN, "water3b", "ref.npz"))["A"]
    assert A.shape == R.shape and _close(A, R)
    n = len(md["types"])
    F = np.fromfile(tmp / "F.bin", dtype=np.float64)
    ref = md["forces"][0]
    assert np.abs(F[:3 * n].reshape(n, 3) - ref).max() <= 1e-10 * np.abs(ref).max()


def test_zcalc_dropins_match_reference(programs, md_inputs):
    tmp, md = md_inputs
    synth = __import__("importlib").import_module("chimes_lsq-myllfork_gb300.synth")
    nat, types, xyz, cell = synth.frames_arrays(os.path.join(GOLDEN, "water3b", "traj.xyzf"), 1, ["O", "H"])[:4]
    _write_frame(tmp / "lsq_frame.bin", types, xyz, cell[0])
    r = subprocess.run([programs["zcalc_check"], os.path.join(GOLDEN, "md_ch4b", "fm_setup.in"),
                        str(tmp / "md_frame.bin"), str(tmp / "md_coef.bin"), str(tmp / "Fz.bin"),
                        os.path.join(GOLDEN, "water3b", "fm_setup.in"), str(tmp / "lsq_frame.bin"),
                        str(tmp / "Az.bin")], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    n = len(md["types"])
    F = np.fromfile(tmp / "Fz.bin", dtype=np.float64)
    assert F.shape == (3 * n + 11,)
    ref = md["forces"][0]
    assert np.abs(F[:3 * n].reshape(n, 3) - ref).max() <= 1e-10 * np.abs(ref).max()
    R = np.load(os.path.join(GOLDEN, "water3b", "ref.npz"))["A"]
    A = np.fromfile(tmp / "Az.bin", dtype=np.float64).reshape(R.shape[0], -1)
    assert _close(A, R[:, :A.shape[1]])
    assert A.shape[1] == R.shape[1] - 2   # the short-range columns (the two energy-offset columns come later)
