"""The mixed-precision fit on a 4-body problem against the FP64 oracle.

The mixed form assembles A in FP32, forms G with the split-BF16 tensor-core Gram,
factorises G + ridge I in FP64 and refines with conjugate gradients whose products
come from FP64 row blocks assembled again on every pass (cg_solve_streamed: no FP64
A is stored).  The FP64 oracle is numpy's FP64 solve of the same ridge system on the
CPU oracle's A (oracle/chimes_oracle.cpp, the reference's loops restated).

Tolerances (the fit targets): coefficients within 1e-8 relative, and the predicted
force rows within 1e-6 eV/A RMS (1 eV/A = 23.0605 kcal/mol/A; A's rows are in
kcal/mol/A).  Ridge: 1e-6 of the largest diagonal entry of A^T A.
"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EV_PER_KCAL = 1.0 / 23.0605


@pytest.fixture(scope="module")
def problem(cg, oracle, tmp_path_factory):
    torch = pytest.importorskip("torch")
    synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
    fm = synth.make_workload("chno-4b", str(tmp_path_factory.mktemp("mixed4b")), nframes=8, seed=505,
                             order=(8, 4, 3), species2=True)
    model = cg.Model(fm)
    frames = cg.Frames.read(model)
    A, b = oracle.assemble(fm, nthreads=8)
    assert A.shape == (frames.nrows, model.ncols)
    G = A.T @ A
    lam = 1e-6 * float(np.abs(np.diag(G)).max())
    xref = np.linalg.solve(G + lam * np.eye(G.shape[0]), A.T @ b)
    force = np.zeros(A.shape[0], bool)   # 256 atoms x 3 force rows, then 9 stress + 3 energy rows per frame
    for f in range(frames.nframes):
        force[f * 780: f * 780 + 768] = True
    return model, frames, A, b, lam, xref, force, torch


def _rel(u, v):
    return float(np.linalg.norm(u - v) / np.linalg.norm(v))


def _force_rms_eVA(A, force, dx):
    return float(np.sqrt(np.mean((A[force] @ dx) ** 2))) * EV_PER_KCAL


def test_mixed_streamed_fit_matches_fp64_oracle(cg, problem):
    model, frames, A, b, lam, xref, force, torch = problem
    sess = cg.Session(model, 0)
    C = model.ncols
    G = torch.zeros((C, C), dtype=torch.float64, device="cuda")
    h = torch.zeros(C, dtype=torch.float64, device="cuda")
    dfrs, labels = [], []
    for f0 in range(0, frames.nframes, 3):
        blk = frames.slice(f0, min(3, frames.nframes - f0))
        dfr = sess.upload(blk)
        lab = torch.from_numpy(blk.labels()).cuda()
        A32 = torch.empty((blk.nrows, C), dtype=torch.float32, device="cuda")
        sess.assemble_device(dfr, cg.CG_FP32, A32.data_ptr(), C)
        sess.gram(1, A32.data_ptr(), C, blk.nrows, C, lab.data_ptr(), 1, G.data_ptr(), h.data_ptr())
        dfrs.append(dfr)
        labels.append(lab)
    sess.gram_finish(G.data_ptr(), C)
    x0 = torch.zeros(C, dtype=torch.float64, device="cuda")
    sess.solve_streamed(G.data_ptr(), h.data_ptr(), C, lam, dfrs, [l.data_ptr() for l in labels], x0.data_ptr(),
                        max_iters=0)
    x = torch.zeros(C, dtype=torch.float64, device="cuda")
    info = sess.solve_streamed(G.data_ptr(), h.data_ptr(), C, lam, dfrs, [l.data_ptr() for l in labels],
                               x.data_ptr(), max_iters=100, tol=1e-13)
    xm, x0 = x.cpu().numpy(), x0.cpu().numpy()
    rel, rel0 = _rel(xm, xref), _rel(x0, xref)
    rms = _force_rms_eVA(A, force, xm - xref)
    print(f"\nmixed 4-body fit: {info['iters']} FP64 passes, coefficients {rel:.3e} relative "
          f"(Cholesky of the tensor-core Gram alone: {rel0:.3e}); force rows {rms:.3e} eV/A RMS", flush=True)
    assert info["iters"] < 100
    assert rel <= 1e-8
    assert rms <= 1e-6
    assert rel < rel0


def test_plain_fp64_fit_matches_fp64_oracle(cg, problem):
    """The plain form: FP64 assembly, this library's FP64 SYRK Gram and FP64 Cholesky."""
    model, frames, A, b, lam, xref, force, torch = problem
    sess = cg.Session(model, 0)
    C = model.ncols
    G = torch.zeros((C, C), dtype=torch.float64, device="cuda")
    h = torch.zeros(C, dtype=torch.float64, device="cuda")
    dA = torch.from_numpy(sess.assemble(frames, cg.CG_FP64)).cuda()
    db = torch.from_numpy(frames.labels()).cuda()
    sess.gram(0, dA.data_ptr(), C, dA.shape[0], C, db.data_ptr(), 0, G.data_ptr(), h.data_ptr())
    sess.gram_finish(G.data_ptr(), C)
    x = torch.zeros(C, dtype=torch.float64, device="cuda")
    sess.solve(G.data_ptr(), h.data_ptr(), C, lam, 0, C, 0, 0, 0, x.data_ptr())
    x64 = x.cpu().numpy()
    assert _rel(x64, xref) <= 1e-8
    assert _force_rms_eVA(A, force, x64 - xref) <= 1e-6


def test_large_cholesky_solve_matches_numpy(cg, problem):
    """n = 9000 > the single-CTA triangular solve: every multi-launch path of the
    blocked Cholesky (diagonal blocks, panel substitution, non-atomic trailing SYRK)
    and of the blocked triangular solves, on a random SPD matrix."""
    model, frames, A, b, lam, xref, force, torch = problem
    sess = cg.Session(model, 0)
    rng = np.random.default_rng(77)
    n = 9000
    M = rng.standard_normal((n + 500, n)) / np.sqrt(n)
    Gh = M.T @ M + 0.5 * np.eye(n)
    hh = rng.standard_normal(n)
    ref = np.linalg.solve(Gh, hh)
    G = torch.from_numpy(Gh).cuda()
    h = torch.from_numpy(hh).cuda()
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    sess.solve(G.data_ptr(), h.data_ptr(), n, 0.0, 0, n, 0, 0, 0, x.data_ptr())
    assert _rel(x.cpu().numpy(), ref) <= 1e-10
