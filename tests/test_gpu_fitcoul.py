"""FITCOUL (Ewald charge columns + charge constraints) through the device path.

* the reference's own lsq2 case (tests/golden/lsq2/normal.npz: its A^T A, A^T b
  and the coefficients of its committed params.ridge.1.0e-03.txt and
  params.lassolars.1.0e-04.txt): the device ridge solve and LARS-lasso on those
  normal equations reproduce the reference's published coefficients.  The ridge
  system is ill-conditioned (kappa(A^T A + 1e-3 I) = 4e12); a QR solve of the
  augmented system lands 9.7e-9 from the published answer, LAPACK's Cholesky 1.4e-10,
  the device Cholesky 9.5e-8: tolerance 2e-7 of max|x|.  LARS: the same support and 1e-6 of max|x| (the
  numpy LARS oracle lands 8.6e-8 from it).
* device DLARS (lars and lasso) against the reference's published DLARS outputs
  (same support, objective 1e-7, coefficients 1e-4 of max|x|: the path is
  ill-conditioned and its vertices move with the arithmetic route).
* the fit driver on the FITCOUL fixture (charge columns assembled on the device,
  constraint rows appended) on the reference's own A: the ridge objective within
  1e-12 of the QR optimum; the coefficients within 1e-5 of LAPACK's Cholesky (the
  constraint rows' 1e4 weights make kappa = 2.5e12; LAPACK's own answer is 1.1e-7
  from the QR one).
"""
import importlib
import os
import shutil

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lsq2():
    d = np.load(os.path.join(GOLDEN, "lsq2", "normal.npz"))
    n = int(d["ncols"])
    G = np.zeros((n, n))
    G[np.triu_indices(n)] = d["G_upper"]
    G = G + np.triu(G, 1).T
    return G, d["h"], int(d["nrows"]), d


def _session(cg):
    return cg.Session(cg.Model(os.path.join(GOLDEN, "watercoul", "fm_setup.in")), 0)


def test_lsq2_ridge_matches_reference_output(cg, lsq2):
    torch = pytest.importorskip("torch")
    G, h, nrows, d = lsq2
    n = G.shape[0]
    sess = _session(cg)
    dG, dh = torch.from_numpy(G).cuda(), torch.from_numpy(h).cuda()
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    sess.solve(dG.data_ptr(), dh.data_ptr(), n, 1e-3, 0, n, nrows, 0, 0, x.data_ptr())
    torch.cuda.synchronize()
    ref = d["x_ridge_1e-3"]
    err = np.abs(x.cpu().numpy() - ref).max() / np.abs(ref).max()
    print(f"\nlsq2 ridge: device vs the reference's params.ridge.1.0e-03.txt {err:.2e}", flush=True)
    assert err <= 2e-7


def test_lsq2_lassolars_matches_reference_output(cg, lsq2):
    torch = pytest.importorskip("torch")
    G, h, nrows, d = lsq2
    n = G.shape[0]
    sess = _session(cg)
    dG, dh = torch.from_numpy(G).cuda(), torch.from_numpy(h).cuda()
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    sess.lars(dG.data_ptr(), dh.data_ptr(), n, nrows, 1e-4, x.data_ptr())
    torch.cuda.synchronize()
    xs = x.cpu().numpy()
    ref = d["x_lassolars_1e-4"]
    err = np.abs(xs - ref).max() / np.abs(ref).max()
    print(f"\nlsq2 lassolars: device vs the reference's params.lassolars.1.0e-04.txt {err:.2e}", flush=True)
    assert np.array_equal(xs != 0, ref != 0)
    assert err <= 1e-6


@pytest.mark.parametrize("algorithm", ["dlars", "dlasso"])
def test_lsq2_dlars_matches_reference_output(cg, lsq2, algorithm):
    """Device DLARS (cg_dlars) on lsq2's normal equations against the reference's
    params.dlars / params.dlasso.1.0e-04.txt: the same support, objective within 1e-7,
    RMS within 1e-6, coefficients within 1e-4 of max|x| (the CPU restatement lands
    1.0e-6 / 2.7e-5 from the published coefficients; see test_cpu_lars.py)."""
    torch = pytest.importorskip("torch")
    G, h, nrows, d = lsq2
    n = G.shape[0]
    btb = float(d["btb"])
    sess = _session(cg)
    dG, dh = torch.from_numpy(G).cuda(), torch.from_numpy(h).cuda()
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    it, nact, _ = sess.dlars(dG.data_ptr(), dh.data_ptr(), n, nrows, btb, 1e-4, algorithm == "dlasso", x.data_ptr())
    torch.cuda.synchronize()
    xs = x.cpu().numpy()
    ref = d[f"x_{algorithm}_1e-4"]
    sq = lambda v: btb - 2 * v @ h + v @ G @ v
    obj = lambda v: 0.5 * sq(v) / nrows + 1e-4 * np.abs(v).sum()
    err = np.abs(xs - ref).max() / np.abs(ref).max()
    print(f"\nlsq2 {algorithm}: {it} iterations; device vs the reference's output {err:.2e}, objective "
          f"{abs(obj(xs) - obj(ref)) / obj(ref):.2e}", flush=True)
    assert np.array_equal(xs != 0, ref != 0)
    assert abs(obj(xs) - obj(ref)) <= 1e-7 * obj(ref)
    assert abs(np.sqrt(sq(xs) / nrows) - np.sqrt(sq(ref) / nrows)) <= 1e-6 * np.sqrt(sq(ref) / nrows)
    assert err <= 1e-4


def test_lsq2_dlasso_normalized_matches_reference_output(cg, lsq2):
    """Device DLARS --normalize=y (columns centred and scaled on the device) against
    the reference's params.dlasso.norm.txt: same support, 1e-8 of max|x| (the
    scaled problem is well conditioned; the CPU restatement lands 5.7e-12 away)."""
    torch = pytest.importorskip("torch")
    G, h, nrows, d = lsq2
    n = G.shape[0]
    sess = _session(cg)
    dG, dh = torch.from_numpy(G).cuda(), torch.from_numpy(h).cuda()
    dcs = torch.from_numpy(d["colsum"]).cuda()
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    it, _, _ = sess.dlars(dG.data_ptr(), dh.data_ptr(), n, nrows, float(d["btb"]), 1e-4, True, x.data_ptr(),
                          colsum_ptr=dcs.data_ptr(), bsum=float(d["bsum"]))
    torch.cuda.synchronize()
    xs = x.cpu().numpy()
    ref = d["x_dlasso_norm_1e-4"]
    err = np.abs(xs - ref).max() / np.abs(ref).max()
    print(f"\nlsq2 dlasso --normalize: {it} iterations; device vs the reference's output {err:.2e}", flush=True)
    assert np.array_equal(xs != 0, ref != 0)
    assert err <= 1e-8


def test_fitcoul_fit_driver_matches_fp64_ridge(cg, tmp_path):
    sl = pytest.importorskip("scipy.linalg")
    for f in ("fm_setup.in", "traj.xyzf"):
        shutil.copy(os.path.join(GOLDEN, "watercoul", f), tmp_path)
    fit = importlib.import_module("chimes_lsq-myllfork_gb300.fit")
    x, y = fit.main([str(tmp_path / "fm_setup.in"), "--out", str(tmp_path / "out"), "--algorithm", "ridge",
                     "--alpha", "1e-3", "--write-a"])
    d = np.load(os.path.join(GOLDEN, "watercoul", "ref.npz"))
    A, b = d["A"], d["b"]   # frames' rows and the two constraint rows, as the reference wrote them
    n = A.shape[1]
    ref = sl.solve(A.T @ A + 1e-3 * np.eye(n), A.T @ b, assume_a="pos")
    xq = np.linalg.lstsq(np.vstack([A, np.sqrt(1e-3) * np.eye(n)]), np.concatenate([b, np.zeros(n)]), rcond=None)[0]
    obj = lambda v: float(np.sum((A @ v - b) ** 2) + 1e-3 * np.sum(v * v))
    rel_obj = abs(obj(x) - obj(xq)) / obj(xq)
    rel_x = np.linalg.norm(x - ref) / np.linalg.norm(ref)
    print(f"\nwatercoul ridge: objective vs the QR optimum {rel_obj:.2e}, coefficients vs LAPACK Cholesky {rel_x:.2e}",
          flush=True)
    assert rel_obj <= 1e-12          # the ridge objective both minimise
    assert rel_x <= 1e-5             # kappa(A^T A + 1e-3 I) = 2.5e12: LAPACK itself is 1.1e-7 from the QR answer
    assert y.shape[0] == A.shape[0]
    model = cg.Model(str(tmp_path / "fm_setup.in"))
    text = open(tmp_path / "out" / "params.txt").read()
    assert "q_O x q_H" in text
    assert np.allclose(model.params_read(text), x, rtol=1e-12, atol=0)
    Aw = np.loadtxt(tmp_path / "out" / "A.txt")   # written from the device A, constraint rows appended
    colmax = np.abs(A).max(axis=0) + 1e-300
    assert Aw.shape == A.shape and (np.abs(Aw - A) / colmax).max() <= 1e-12
