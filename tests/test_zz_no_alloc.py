"""The allocation-free assembly entry point (cg_assemble_device_noalloc).

Callers that cannot allocate device memory during a run -- an MD engine or a
serving loop that reserves its memory at start-up, or an application with its own
device pool -- use this entry point; its work buffers live in a fixed device array
inside the library.  It must give the same A as cg_assemble_device, call after call
(the shared array keeps the previous call's contents, so stale data would show up on
the second call), and must refuse inputs whose work lists exceed the array.
Named test_zz_* so that pytest collects it last.
"""
import ctypes
import importlib
import os

import numpy as np
import pytest

from conftest import fixture_dir

pytestmark = pytest.mark.gpu


def _close(A, R, prec):
    """FP64: 1e-12 of the entry and of its column's scale; FP32: 2e-5 of the column's
    scale (the tolerances of the assembly parity tests)."""
    colmax = np.abs(R).max(axis=0)
    if prec == 0:
        return bool(np.all(np.abs(A - R) <= 1e-12 * np.abs(R) + 1e-12 * colmax[None, :]))
    return bool(np.all(np.abs(A - R) <= 2e-5 * (colmax[None, :] + 1e-300)))


@pytest.mark.parametrize("prec", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("name", ["water3b", "ch4b"])
def test_noalloc_matches_device_entry_point(cg, name, prec):
    torch = pytest.importorskip("torch")
    lib = cg.lib()
    model = cg.Model(os.path.join(fixture_dir(name), "fm_setup.in"))
    frames = cg.Frames.read(model)
    sess = cg.Session(model, 0)
    dfr = sess.upload(frames)
    nrows, ncols = frames.nrows, model.ncols
    dt = torch.float64 if prec == cg.CG_FP64 else torch.float32
    ref = torch.empty((nrows, ncols), dtype=dt, device="cuda")
    sess.assemble_device(dfr, prec, ref.data_ptr(), ncols)
    torch.cuda.synchronize()
    R = ref.double().cpu().numpy()
    for _ in range(2):
        out = torch.full((nrows, ncols), float("nan"), dtype=dt, device="cuda")
        rc = lib.cg_assemble_device_noalloc(sess._h, dfr._h, prec, ctypes.c_void_p(out.data_ptr()), ncols)
        assert rc == 0, lib.cg_last_error().decode()
        torch.cuda.synchronize()
        assert _close(out.double().cpu().numpy(), R, prec)


def test_noalloc_rejects_oversize_input(cg, tmp_path):
    torch = pytest.importorskip("torch")
    synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
    fm = synth.make_workload("water-3b", str(tmp_path), nframes=40, seed=7, labels=False)
    model = cg.Model(fm)
    frames = cg.Frames.read(model)
    sess = cg.Session(model, 0)
    dfr = sess.upload(frames)
    out = torch.empty((frames.nrows, model.ncols), dtype=torch.float64, device="cuda")
    lib = cg.lib()
    rc = lib.cg_assemble_device_noalloc(sess._h, dfr._h, cg.CG_FP64, ctypes.c_void_p(out.data_ptr()), model.ncols)
    assert rc == 4
    assert "scratch capacity" in lib.cg_last_error().decode()
