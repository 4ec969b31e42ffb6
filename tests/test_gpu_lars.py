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
