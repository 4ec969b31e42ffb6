"""GPU checks of the normal equations (G = A^T A, h = A^T b) and the FP64 solve.

Tolerances: the FP64 library Gram matches numpy's A^T A to 1e-12 relative to
sqrt(G_ii G_jj); the split-BF16 tensor-core Gram (hi.hi + hi.lo + lo.hi, FP32
accumulation) to 1e-4 of sqrt(G_ii G_jj) (its products carry ~2^-16 relative error).
The FP64 solve matches numpy's FP64 solve of the same ridge-regularised system
within the system's conditioning; preconditioned CG with FP64 products through A
brings the mixed form (tensor-core Gram) to the same least-squares fit as the FP64
form (measured agreements are printed).
"""
import ctypes
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def system(cg, tmp_path_factory):
    torch = pytest.importorskip("torch")
    synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
    fm = synth.make_workload("water-3b", str(tmp_path_factory.mktemp("gram")), nframes=8, seed=404)
    model = cg.Model(fm)
    frames = cg.Frames.read(model)
    sess = cg.Session(model, 0)
    A = sess.assemble(frames, cg.CG_FP64)
    b = frames.labels()
    dA = torch.from_numpy(A).cuda()
    db = torch.from_numpy(b).cuda()
    return sess, A, b, dA, db, torch


def _gram(cg, sess, dA, db, mode, torch, prec=0):
    n = dA.shape[1]
    G = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    h = torch.zeros(n, dtype=torch.float64, device="cuda")
    src = dA if prec == 0 else dA.float()
    lib = cg.lib()
    rc = lib.cg_gram(sess._h, prec, ctypes.c_void_p(src.data_ptr()), src.shape[1], src.shape[0], n,
                     ctypes.c_void_p(db.data_ptr()), mode, ctypes.c_void_p(G.data_ptr()), ctypes.c_void_p(h.data_ptr()))
    assert rc == 0, lib.cg_last_error().decode()
    assert lib.cg_gram_finish(sess._h, ctypes.c_void_p(G.data_ptr()), n) == 0
    torch.cuda.synchronize()
    return G, h


def test_gram_fp64_and_tensor_core(cg, system):
    sess, A, b, dA, db, torch = system
    Gref = A.T @ A
    href = A.T @ b
    d = np.sqrt(np.maximum(np.diag(Gref), 1e-300))
    scale = np.outer(d, d)
    G64, h64 = _gram(cg, sess, dA, db, 0, torch)
    assert np.all(np.abs(G64.cpu().numpy() - Gref) <= 1e-12 * scale + 1e-300)
    assert np.allclose(h64.cpu().numpy(), href, rtol=1e-10, atol=1e-10 * np.abs(href).max())
    Gtc, htc = _gram(cg, sess, dA, db, 1, torch)
    err = np.abs(Gtc.cpu().numpy() - Gref)
    assert np.all(err <= 1e-4 * scale + 1e-300), (err / (scale + 1e-300)).max()
    # h of the mixed form: FP64 sums in another order (fused into the split pass)
    habs = np.abs(A).T @ np.abs(b)
    assert np.all(np.abs(htc.cpu().numpy() - href) <= 1e-13 * habs)
    # FP32 A input gives the same tensor-core Gram (the split starts from FP32 values);
    # its h is the float-float sum of the FP32 A's products (about 44 bits), checked
    # against the FP64 product of that same FP32 A
    Gtc32, htc32 = _gram(cg, sess, dA, db, 1, torch, prec=1)
    assert np.all(np.abs(Gtc32.cpu().numpy() - Gref) <= 1e-4 * scale + 1e-300)
    A32 = A.astype(np.float32).astype(np.float64)
    assert np.all(np.abs(htc32.cpu().numpy() - A32.T @ b) <= 1e-11 * habs)


def _solve(cg, sess, G, h, dA, db, ridge, iters, torch):
    n = G.shape[0]
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    info = (ctypes.c_double * 3)()
    lib = cg.lib()
    rc = lib.cg_solve(sess._h, ctypes.c_void_p(G.data_ptr()), ctypes.c_void_p(h.data_ptr()), n, ctypes.c_double(ridge),
                      ctypes.c_void_p(dA.data_ptr()), dA.shape[1], dA.shape[0], ctypes.c_void_p(db.data_ptr()), iters,
                      ctypes.c_void_p(x.data_ptr()), info)
    assert rc == 0, lib.cg_last_error().decode()
    torch.cuda.synchronize()
    return x.cpu().numpy(), info[0], info[1]


def test_solve_matches_numpy_and_mixed_refines(cg, system):
    """FP64 Cholesky solve vs numpy on the same ridge system, and the mixed form
    (tensor-core Gram + FP64 Cholesky preconditioner + CG with FP64 products through
    A) vs the FP64 form on the same ridge system: coefficients within 1e-8 relative,
    force-row RMSE within 1e-9 relative."""
    sess, A, b, dA, db, torch = system
    G64, h64 = _gram(cg, sess, dA, db, 0, torch)
    Gn = A.T @ A
    hn = A.T @ b
    ridge = 1e-9 * np.abs(np.diag(Gn)).max()
    Gr = Gn + ridge * np.eye(Gn.shape[0])
    xref = np.linalg.solve(Gr, hn)
    x64, _, _ = _solve(cg, sess, G64, h64, dA, db, ridge, 0, torch)
    res_ref = np.linalg.norm(Gr @ xref - hn) / np.linalg.norm(hn)
    res_64 = np.linalg.norm(Gr @ x64 - hn) / np.linalg.norm(hn)
    assert res_64 <= max(10 * res_ref, 1e-10)
    assert np.linalg.norm(x64 - xref) <= 1e-6 * np.linalg.norm(xref)
    # mixed form on a conditioned ridge system
    lam = 1e-6 * np.abs(np.diag(Gn)).max()
    Gtc, htc = _gram(cg, sess, dA, db, 1, torch)
    xd, _, _ = _solve(cg, sess, G64, h64, dA, db, lam, 0, torch)          # FP64 direct
    xf, rn_f, gn_f = _solve(cg, sess, G64, h64, dA, db, lam, 20, torch)   # FP64 + CG
    x0, _, _ = _solve(cg, sess, Gtc, htc, dA, db, lam, 0, torch)          # mixed direct
    xm, rn_m, gn_m = _solve(cg, sess, Gtc, htc, dA, db, lam, 400, torch)  # mixed + CG
    rel = lambda u, v: np.linalg.norm(u - v) / np.linalg.norm(v)
    rmse = lambda x: np.sqrt(np.mean((A @ x - b) ** 2))
    print(f"\nridge {lam:.3e}: mixed direct vs FP64 {rel(x0, xf):.3e}, mixed+CG vs FP64 {rel(xm, xf):.3e}; "
          f"FP64 direct vs FP64+CG {rel(xd, xf):.3e}; residual |A^T r - l x|: FP64 {gn_f:.3e}, mixed {gn_m:.3e}; "
          f"RMSE FP64 {rmse(xf):.9e} mixed {rmse(xm):.9e}", flush=True)
    assert rel(xm, xf) <= 1e-8
    assert abs(rmse(xm) - rmse(xf)) <= 1e-9 * rmse(xf)
    assert rel(xm, xf) < rel(x0, xf)


@pytest.mark.parametrize("n", [700, 1537])
def test_cholesky_tensor_updates_match_fp64(cg, system, n):
    """The blocked Cholesky with trailing updates from exact BF16 digit products on the
    tensor cores against the same factorisation with FP64 SYRK updates, on a random
    symmetric positive definite matrix whose columns span 12 orders of magnitude (n not
    a multiple of the 128-wide panel).  Tolerance: factors within 1e-13 of each
    column's diagonal scale, solves within 1e-10 (condition number about 1e5)."""
    sess, _, _, _, _, torch = system
    rng = np.random.default_rng(n)
    X = rng.standard_normal((3 * n, n)) * np.exp(rng.uniform(-14, 14, size=n))[None, :]
    G = X.T @ X
    G += 1e-5 * np.diag(np.diag(G))
    dG = torch.from_numpy(G).cuda()
    h = torch.from_numpy(rng.standard_normal(n)).cuda()
    out = {}
    for mode in (0, 1):
        sess.tune("cholesky_tensor_updates", mode)
        L = torch.empty((n, n), dtype=torch.float64, device="cuda")
        r = sess.cholesky(dG.data_ptr(), n, 0.0, L.data_ptr())
        assert r == 0.0
        x = torch.empty(n, dtype=torch.float64, device="cuda")
        sess.cholesky_solve(L.data_ptr(), n, h.data_ptr(), x.data_ptr())
        torch.cuda.synchronize()
        out[mode] = (torch.triu(L).cpu().numpy(), x.cpu().numpy())
    sess.tune("cholesky_tensor_updates", 1)
    L0, x0 = out[0]
    L1, x1 = out[1]
    d = np.sqrt(np.diag(G))
    fac = float(np.abs((L1 - L0) / d[None, :]).max())
    sol = float(np.abs(x1 - x0).max() / np.abs(x0).max())
    print(f"\nn={n}: tensor-update vs FP64 Cholesky factor {fac:.2e}, solve {sol:.2e}", flush=True)
    assert fac <= 1e-13
    assert sol <= 1e-10
