"""The fit driver (chimes_lsq-myllfork_gb300/fit.py, the drop-in for `chimes_lsq` +
`chimes_lsq.py`) against scikit-learn's Ridge / LassoLars on the fixtures' design
matrices (the reference's --algorithm ridge / lassolars solvers), and its output
files against the library's own writers.  Tolerances: ridge coefficients 1e-9
relative (FP64) and 1e-8 (mixed Gram refined with FP64 products), LARS 1e-7."""
import importlib
import os
import shutil

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

pytestmark = pytest.mark.gpu


def _run(tmp_path, name, *args):
    for f in ("fm_setup.in", "traj.xyzf"):
        shutil.copy(os.path.join(GOLDEN, name, f), tmp_path)
    fit = importlib.import_module("chimes_lsq-myllfork_gb300.fit")
    return fit.main([str(tmp_path / "fm_setup.in"), "--out", str(tmp_path / "out"), *args])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fit_ridge_matches_sklearn_ridge(cg, tmp_path, precision):
    gold = np.load(os.path.join(GOLDEN, "lars", "sklearn_lassolars.npz"))
    ref = gold["water2b_ridge_1e-03_coef"]
    x, y = _run(tmp_path, "water2b", "--algorithm", "ridge", "--alpha", "1e-3", "--precision", precision,
                "--refine", "60")
    tol = 1e-9 if precision == "fp64" else 1e-8
    assert np.linalg.norm(x - ref) <= tol * np.linalg.norm(ref)
    model = cg.Model(str(tmp_path / "fm_setup.in"))
    out = tmp_path / "out"
    assert open(out / "params.header").read() == model.params_header()
    assert np.allclose(model.params_read(open(out / "params.txt").read()), x, rtol=1e-12, atol=0)
    d = np.load(os.path.join(GOLDEN, "water2b", "ref.npz"))
    f = np.loadtxt(out / "force.txt")
    assert np.allclose(f, d["A"] @ ref, rtol=2e-6, atol=2e-6 * np.abs(f).max())


def test_fit_lassolars_matches_sklearn(cg, tmp_path):
    gold = np.load(os.path.join(GOLDEN, "lars", "sklearn_lassolars.npz"))
    ref = gold["ch4b_1e-04_coef"]
    x, _ = _run(tmp_path, "ch4b", "--algorithm", "lassolars", "--alpha", "1e-4", "--write-a")
    assert np.linalg.norm(x - ref) <= 1e-7 * np.linalg.norm(ref)
    A = np.loadtxt(tmp_path / "out" / "A.txt", ndmin=2)
    d = np.load(os.path.join(GOLDEN, "ch4b", "ref.npz"))
    assert A.shape[0] == d["A"].shape[0]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fit_with_row_weights_matches_weighted_normal_equations(cg, tmp_path, precision):
    """--weights (chimes_lsq.py multiplies the rows of A and b by them): the ridge
    coefficients solve (A^T W^2 A + alpha I) x = A^T W^2 b on the reference's A, and
    force.txt stays the unweighted A x."""
    d = np.load(os.path.join(GOLDEN, "water2b", "ref.npz"))
    A, b = d["A"], d["b"]
    w = np.random.default_rng(21).uniform(0.5, 2.0, A.shape[0])
    np.savetxt(tmp_path / "weights.dat", w)
    Aw, bw = A * w[:, None], b * w
    ref = np.linalg.solve(Aw.T @ Aw + 1e-3 * np.eye(A.shape[1]), Aw.T @ bw)
    x, y = _run(tmp_path, "water2b", "--algorithm", "ridge", "--alpha", "1e-3", "--precision", precision,
                "--refine", "60", "--weights", str(tmp_path / "weights.dat"))
    tol = 1e-9 if precision == "fp64" else 1e-8
    assert np.linalg.norm(x - ref) <= tol * np.linalg.norm(ref)
    f = np.loadtxt(tmp_path / "out" / "force.txt")
    assert np.allclose(f, A @ ref, rtol=2e-6, atol=2e-6 * np.abs(f).max())
    assert "! Using weighting file:" in open(tmp_path / "out" / "params.txt").read()
    np.savetxt(tmp_path / "short.dat", w[:-1])
    with pytest.raises(SystemExit):
        _run(tmp_path, "water2b", "--weights", str(tmp_path / "short.dat"))
