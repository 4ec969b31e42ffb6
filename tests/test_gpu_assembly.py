"""GPU parity of the design-matrix assembly, through the C ABI.

Tolerances (FP64 form): |gpu - ref| <= 1e-12 |ref| + 1e-12 max|ref[:, col]| per
entry -- the GPU sums the same terms in a different order, so the bound is
relative to the entry and to its column's scale.  The FP32 (mixed) form is held to
2e-5 of the column scale.  Cluster sets themselves are integer work: a missing or
extra pair/triplet/quadruplet shifts entries by O(column scale), far above these
bounds.
"""
import os

import numpy as np
import pytest

from conftest import FIXTURES, fixture_dir, frame_part

pytestmark = pytest.mark.gpu


def close_fp64(A, R):
    colmax = np.abs(R).max(axis=0)
    err = np.abs(A - R)
    tol = 1e-12 * np.abs(R) + 1e-12 * colmax[None, :]
    return bool(np.all(err <= tol)), float(err.max())


@pytest.fixture(scope="module")
def session_for(cg):
    cache = {}

    def get(fm):
        if fm not in cache:
            m = cg.Model(fm)
            cache[fm] = (m, cg.Session(m, 0))
        return cache[fm]
    return get


@pytest.mark.parametrize("name", FIXTURES)
def test_fixture_fp64_matches_reference(cg, session_for, name):
    fm = os.path.join(fixture_dir(name), "fm_setup.in")
    model, sess = session_for(fm)
    frames = cg.Frames.read(model)
    A = sess.assemble(frames, cg.CG_FP64)
    R, rb, _, _ = frame_part(model, np.load(os.path.join(fixture_dir(name), "ref.npz")))
    assert A.shape == R.shape
    ok, err = close_fp64(A, R)
    assert ok, f"{name}: max |gpu - reference| = {err}"
    assert np.array_equal(frames.labels(), rb)


@pytest.mark.parametrize("name", FIXTURES)
def test_fixture_fp32_close_to_reference(cg, session_for, name):
    fm = os.path.join(fixture_dir(name), "fm_setup.in")
    model, sess = session_for(fm)
    frames = cg.Frames.read(model)
    A = sess.assemble(frames, cg.CG_FP32).astype(np.float64)
    R = frame_part(model, np.load(os.path.join(fixture_dir(name), "ref.npz")))[0]
    colmax = np.abs(R).max(axis=0) + 1e-300
    rel = (np.abs(A - R) / colmax[None, :]).max()
    assert rel < 2e-5, f"{name}: FP32 column-relative error {rel}"


def test_deterministic(cg, session_for):
    fm = os.path.join(fixture_dir("ch4b"), "fm_setup.in")
    model, sess = session_for(fm)
    frames = cg.Frames.read(model)
    A1 = sess.assemble(frames, cg.CG_FP64)
    A2 = sess.assemble(frames, cg.CG_FP64)
    assert np.array_equal(A1, A2)


def _workload(tmp_path_factory, cg, name, nframes, seed, **over):
    import importlib
    synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
    d = tmp_path_factory.mktemp(name)
    return synth.make_workload(name, str(d), nframes=nframes, seed=seed, **over)


def test_water3b_matches_oracle(cg, oracle, session_for, tmp_path_factory):
    fm = _workload(tmp_path_factory, cg, "water-3b", 6, 101)
    model, sess = session_for(fm)
    frames = cg.Frames.read(model)
    A = sess.assemble(frames, cg.CG_FP64)
    O, b = oracle.assemble(fm, nthreads=8)
    ok, err = close_fp64(A, O)
    assert ok, f"max |gpu - oracle| = {err}"
    assert np.array_equal(frames.labels(), b)
    c = sess.last_counts()
    assert c["triplets"] > 0


@pytest.mark.parametrize("form,threads", [(1, 512), (0, 512), (0, 1024)])
def test_chno4b_matches_oracle(cg, oracle, tmp_path_factory, form, threads):
    """The full 4-body basis (3,861 allowed powers per quadruplet type) with the range
    form of the force-row kernel and both launch shapes of the per-power form."""
    fm = _workload(tmp_path_factory, cg, "chno-4b", 1, 202)
    model = cg.Model(fm)
    sess = cg.Session(model, 0)
    sess.tune("force_range", form)
    sess.tune("force4_threads", threads)
    frames = cg.Frames.read(model)
    A = sess.assemble(frames, cg.CG_FP64)
    O, _ = oracle.assemble(fm, nthreads=8)
    assert A.shape == O.shape == (780, 51209)
    ok, err = close_fp64(A, O)
    assert ok, f"max |gpu - oracle| = {err}"
    A32 = sess.assemble(frames, cg.CG_FP32).astype(np.float64)
    colmax = np.abs(O).max(axis=0) + 1e-300
    assert (np.abs(A32 - O) / colmax[None, :]).max() < 2e-5


@pytest.mark.parametrize("form", [2, 0])
def test_dense_3body_matches_oracle(cg, oracle, tmp_path_factory, form):
    """A 6 A 3-body cut-off in liquid water: each owner meets its triplet types far
    more often than one shared-memory chunk holds, and more than one pass of
    incidences (above 1024), so the force rows are added over chunks and passes."""
    fm = _workload(tmp_path_factory, cg, "water-3b", 2, 303, smax=(5.0, 6.0, None))
    model = cg.Model(fm)
    sess = cg.Session(model, 0)
    sess.tune("force_range", form)
    frames = cg.Frames.read(model)
    A = sess.assemble(frames, cg.CG_FP64)
    c = sess.last_counts()
    assert 3 * c["triplets"] > 1024 * 384 * 2, c   # more than 1024 incidences per owner on average
    O, _ = oracle.assemble(fm, nthreads=8)
    ok, err = close_fp64(A, O)
    assert ok, f"max |gpu - oracle| = {err}"


def test_force_rows_sum_to_zero(cg, session_for, tmp_path_factory):
    """Newton's third law per column: the force rows of a frame sum to zero
    (every cluster contributes equal and opposite terms)."""
    fm = _workload(tmp_path_factory, cg, "water-3b", 3, 303)
    model, sess = session_for(fm)
    frames = cg.Frames.read(model)
    A = sess.assemble(frames, cg.CG_FP64)
    n = 384
    per = 3 * n + 9 + 3
    for f in range(3):
        F = A[f * per: f * per + 3 * n, : model.columns()["n2b"] + model.columns()["n3b"]]
        s = F.reshape(n, 3, -1).sum(axis=0)
        scale = np.abs(F).max(axis=0) + 1e-300
        assert (np.abs(s) / scale).max() < 1e-11


def test_arrays_path_equals_text_path(cg, session_for):
    import importlib
    synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
    d = fixture_dir("ch4b")
    fm = os.path.join(d, "fm_setup.in")
    model, sess = session_for(fm)
    nat, typ, xyz, cell, frc, st, en = synth.frames_arrays(os.path.join(d, "traj.xyzf"), 2, ["C", "H"])
    fa = cg.Frames.from_arrays(model, nat, typ, xyz, cell, frc, st, en)
    ft = cg.Frames.read(model)
    assert np.array_equal(sess.assemble(fa), sess.assemble(ft))


def test_streamed_host_assembly_equals_device_assembly(cg, session_for, tmp_path_factory):
    """cg_assemble_stream (row blocks to pinned host memory while the next block
    assembles) and cg_assemble (the same pipeline into the caller's buffer) give the
    device assembly's A bit for bit; a sink that asks to stop ends the call with
    status 1."""
    torch = pytest.importorskip("torch")
    fm = _workload(tmp_path_factory, cg, "water-3b", 7, 505)
    model, sess = session_for(fm)
    frames = cg.Frames.read(model)
    dfr = sess.upload(frames)
    dA = torch.empty((frames.nrows, model.ncols), dtype=torch.float64, device="cuda")
    sess.assemble_device(dfr, cg.CG_FP64, dA.data_ptr(), model.ncols)
    torch.cuda.synchronize()
    R = dA.cpu().numpy()
    got = []
    sess.assemble_stream(frames, cg.CG_FP64, lambda first, blk: got.append((first, blk.copy())) and False,
                         block_frames=2)
    assert [g[0] for g in got] == sorted(g[0] for g in got) and len(got) == 4
    assert np.array_equal(np.concatenate([g[1] for g in got]), R)
    assert np.array_equal(sess.assemble(frames, cg.CG_FP64), R)
    with pytest.raises(cg.ChimesError) as e:
        sess.assemble_stream(frames, cg.CG_FP64, lambda first, blk: True, block_frames=3)
    assert e.value.code == 1
    sess.tune("host_staging", 0)   # staging in huge-page memory registered with CUDA
    got = []
    sess.assemble_stream(frames, cg.CG_FP64, lambda first, blk: got.append((first, blk.copy())) and False,
                         block_frames=2)
    assert np.array_equal(np.concatenate([g[1] for g in got]), R)
    sess.tune("host_staging", 1)
