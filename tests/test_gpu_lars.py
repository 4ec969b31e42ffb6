"""Device LARS-lasso (cg_lars) against scikit-learn's LassoLars, the reference's
`--algorithm lassolars` solver (tests/golden/lars/sklearn_lassolars.npz).
Tolerance: coefficients within 1e-7 relative, the same number of steps, the same
support.  One case takes its normal equations from the library's own FP64 Gram."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
CASES = [("water2b", 1e-4), ("water2b", 1e-2), ("water3b", 1e-4), ("water3b", 1e-2), ("ch4b", 1e-4), ("ch4b", 1e-2)]


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(GOLDEN, "lars", "sklearn_lassolars.npz"))


@pytest.mark.parametrize("name,alpha", CASES)
def test_device_lars_matches_sklearn_lassolars(cg, golden, name, alpha):
    torch = pytest.importorskip("torch")
    d = np.load(os.path.join(GOLDEN, name, "ref.npz"))
    A, b = d["A"], d["b"]
    model = cg.Model(os.path.join(GOLDEN, name, "fm_setup.in"))
    sess = cg.Session(model, 0)
    G = torch.from_numpy(A.T @ A).cuda()
    h = torch.from_numpy(A.T @ b).cuda()
    x = torch.zeros(A.shape[1], dtype=torch.float64, device="cuda")
    steps, nact, cfin = sess.lars(G.data_ptr(), h.data_ptr(), A.shape[1], A.shape[0], alpha, x.data_ptr())
    torch.cuda.synchronize()
    xs = x.cpu().numpy()
    key = f"{name}_{alpha:.0e}"
    ref = golden[key + "_coef"]
    assert steps == int(golden[key + "_steps"])
    assert np.linalg.norm(xs - ref) <= 1e-7 * np.linalg.norm(ref)
    assert np.array_equal(xs != 0, ref != 0)
    assert abs(cfin - alpha) <= 1e-9 * alpha


def test_device_lars_on_library_gram(cg, golden):
    torch = pytest.importorskip("torch")
    name, alpha = "ch4b", 1e-4
    d = np.load(os.path.join(GOLDEN, name, "ref.npz"))
    model = cg.Model(os.path.join(GOLDEN, name, "fm_setup.in"))
    sess = cg.Session(model, 0)
    dA = torch.from_numpy(d["A"]).cuda()
    db = torch.from_numpy(d["b"]).cuda()
    n = dA.shape[1]
    G = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    h = torch.zeros(n, dtype=torch.float64, device="cuda")
    sess.gram(0, dA.data_ptr(), n, dA.shape[0], n, db.data_ptr(), 0, G.data_ptr(), h.data_ptr())
    sess.gram_finish(G.data_ptr(), n)
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    sess.lars(G.data_ptr(), h.data_ptr(), n, dA.shape[0], alpha, x.data_ptr())
    torch.cuda.synchronize()
    ref = golden[f"{name}_{alpha:.0e}_coef"]
    assert np.linalg.norm(x.cpu().numpy() - ref) <= 1e-7 * np.linalg.norm(ref)


def _dlars64_device(cg, torch):
    d = np.load(os.path.join(GOLDEN, "dlars64", "dlars64.npz"))
    X, y = d["X"], d["y"]
    m = cg.Model(os.path.join(GOLDEN, "water2b", "fm_setup.in"))   # any model: the session only hosts the solver
    sess = cg.Session(m, 0)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    G, h, colsum = dev(X.T @ X), dev(X.T @ y), dev(X.sum(0))
    n = X.shape[0]
    mu = X.mean(0)
    sig = np.sqrt(np.diag(X.T @ X) - n * mu * mu)
    return d, sess, G, h, colsum, float(y.sum()), float(y @ y), n, sig


@pytest.mark.parametrize("case", ["lars", "lasso", "maxnorm", "lambda", "iters"])
def test_dlars_options_match_reference_test_suite(cg, case):
    """cg_dlars_ex on the reference DLARS's 64 x 32 test problem (--normalize=y) with
    its --algorithm, --max_norm=20, --lambda=5e-3 and --iterations=10: final
    coefficients as printed (13 digits, normalised problem) within 1e-9 of the
    largest, and the same iteration count."""
    torch = pytest.importorskip("torch")
    d, sess, G, h, colsum, bsum, btb, n, sig = _dlars64_device(cg, torch)
    lasso, lam, mn, its = d[case + "_params"]
    x = torch.zeros(G.shape[0], dtype=torch.float64, device="cuda")
    it, _, _ = sess.dlars(G.data_ptr(), h.data_ptr(), G.shape[0], n, btb, lam, bool(lasso), x.data_ptr(),
                          max_iter=int(its), colsum_ptr=colsum.data_ptr(), bsum=bsum,
                          max_norm=mn if mn < 1e49 else 0.0)
    ref = d[case + "_beta"]
    assert np.abs(x.cpu().numpy() * sig - ref).max() <= 1e-9 * np.abs(ref).max()
    assert it == int(d[case + "_iterations"])


def test_dlars_restart_resumes_the_walk(cg, tmp_path):
    """A walk stopped after 15 iterations with a restart file (written every ten)
    and resumed from it ends where the uninterrupted walk ends."""
    torch = pytest.importorskip("torch")
    d, sess, G, h, colsum, bsum, btb, n, sig = _dlars64_device(cg, torch)
    p = G.shape[0]
    full = torch.zeros(p, dtype=torch.float64, device="cuda")
    sess.dlars(G.data_ptr(), h.data_ptr(), p, n, btb, 0.0, True, full.data_ptr(), colsum_ptr=colsum.data_ptr(),
               bsum=bsum)
    part = torch.zeros(p, dtype=torch.float64, device="cuda")
    rst = tmp_path / "restart.txt"
    it1, _, _ = sess.dlars(G.data_ptr(), h.data_ptr(), p, n, btb, 0.0, True, part.data_ptr(), max_iter=15,
                           colsum_ptr=colsum.data_ptr(), bsum=bsum, restart_out=rst)
    assert it1 == 15 and rst.exists() and "Iteration 10" in rst.read_text()
    res = torch.zeros(p, dtype=torch.float64, device="cuda")
    it2, _, _ = sess.dlars(G.data_ptr(), h.data_ptr(), p, n, btb, 0.0, True, res.data_ptr(),
                           colsum_ptr=colsum.data_ptr(), bsum=bsum, restart_in=rst)
    ref = full.cpu().numpy()
    assert it2 == int(d["lasso_iterations"])
    assert np.abs(res.cpu().numpy() - ref).max() <= 1e-9 * np.abs(ref).max()
