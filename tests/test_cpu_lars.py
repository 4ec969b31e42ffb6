"""The oracle's LARS-lasso restatement (oracle/lars.py) against scikit-learn's
LassoLars -- the reference's `--algorithm lassolars` solver -- on the
design-matrix fixtures (tests/golden/lars/sklearn_lassolars.npz, made by
tests/golden/make_lars_fixtures.py).  Tolerance: coefficients within 1e-7
relative (the 910-step water case is the most sensitive: 1.3e-8 measured), the
same number of steps."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

CASES = [("water2b", 1e-4), ("water2b", 1e-2), ("water3b", 1e-4), ("water3b", 1e-2), ("ch4b", 1e-4), ("ch4b", 1e-2)]


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(GOLDEN, "lars", "sklearn_lassolars.npz"))


@pytest.mark.parametrize("name,alpha", CASES)
def test_oracle_lars_matches_sklearn_lassolars(golden, name, alpha):
    import lars
    d = np.load(os.path.join(GOLDEN, name, "ref.npz"))
    A, b = d["A"], d["b"]
    x, steps = lars.lars_lasso(A.T @ A, A.T @ b, A.shape[0], alpha)
    key = f"{name}_{alpha:.0e}"
    ref = golden[key + "_coef"]
    assert steps == int(golden[key + "_steps"])
    assert np.linalg.norm(x - ref) <= 1e-7 * np.linalg.norm(ref)
    assert np.array_equal(x != 0, ref != 0)


def test_cholesky_delete_matches_refactorisation():
    import lars
    rng = np.random.default_rng(0)
    X = rng.standard_normal((40, 12))
    G = X.T @ X
    L = np.linalg.cholesky(G)
    for k in (0, 5, 11):
        Ld = lars._chol_delete(L, k)
        keep = [i for i in range(12) if i != k]
        assert np.allclose(Ld @ Ld.T, G[np.ix_(keep, keep)], rtol=1e-12, atol=1e-12)


def test_oracle_lars_matches_reference_lsq2_output():
    """The LARS oracle on the normal equations of the reference's lsq2 case reproduces
    the coefficients of the reference's params.lassolars.1.0e-04.txt (its
    chimes_lsq.py --algorithm lassolars output): same support, 1e-6 of max|x|."""
    import lars
    d = np.load(os.path.join(GOLDEN, "lsq2", "normal.npz"))
    n = int(d["ncols"])
    G = np.zeros((n, n))
    G[np.triu_indices(n)] = d["G_upper"]
    G = G + np.triu(G, 1).T
    out = lars.lars_lasso(G, d["h"], int(d["nrows"]), 1e-4)
    x = out[0] if isinstance(out, tuple) else out
    ref = d["x_lassolars_1e-4"]
    assert np.array_equal(x != 0, ref != 0)
    assert np.abs(x - ref).max() <= 1e-6 * np.abs(ref).max()


@pytest.mark.parametrize("algorithm", ["dlars", "dlasso"])
def test_oracle_dlars_matches_reference_lsq2_output(algorithm):
    """The DLARS oracle (oracle/dlars.py) on lsq2's normal equations against the
    reference's params.dlars / params.dlasso.1.0e-04.txt (DLARS run on the A matrix
    by 36 MPI ranks).  The problem is ill-conditioned (singular values of A from
    6.5e4 down to 1.6e-12), and the path's vertices move with the arithmetic route: an
    A-based restatement lands 4.9e-6 / 1.7e-5 from the published coefficients, this
    normal-equation one 1.0e-6 / 2.7e-5.  Checked: the same support, the objective
    within 1e-7 relative, the RMS error within 1e-6, coefficients within 1e-4 of max|x|."""
    import dlars
    d = np.load(os.path.join(GOLDEN, "lsq2", "normal.npz"))
    n = int(d["ncols"])
    G = np.zeros((n, n))
    G[np.triu_indices(n)] = d["G_upper"]
    G = G + np.triu(G, 1).T
    h, btb, N = d["h"], float(d["btb"]), int(d["nrows"])
    x, it, stop = dlars.dlars(G, h, btb, N, 1e-4, algorithm == "dlasso")
    ref = d[f"x_{algorithm}_1e-4"]
    sq = lambda v: btb - 2 * v @ h + v @ G @ v
    obj = lambda v: 0.5 * sq(v) / N + 1e-4 * np.abs(v).sum()
    assert stop == "objective increased"
    assert np.array_equal(x != 0, ref != 0)
    assert abs(obj(x) - obj(ref)) <= 1e-7 * obj(ref)
    assert abs(np.sqrt(sq(x) / N) - np.sqrt(sq(ref) / N)) <= 1e-6 * np.sqrt(sq(ref) / N)
    assert np.abs(x - ref).max() <= 1e-4 * np.abs(ref).max()


def test_oracle_dlars_normalized_matches_reference_lsq2_output():
    """DLARS --normalize=y (columns centred and scaled, b centred) on lsq2 against the
    reference's params.dlasso.norm.txt: well conditioned after the scaling, the
    coefficients agree to 1e-9 of max|x| (5.7e-12 measured)."""
    import dlars
    d = np.load(os.path.join(GOLDEN, "lsq2", "normal.npz"))
    n = int(d["ncols"])
    G = np.zeros((n, n))
    G[np.triu_indices(n)] = d["G_upper"]
    G = G + np.triu(G, 1).T
    x, it, stop = dlars.dlars_normalized(G, d["h"], d["colsum"], float(d["bsum"]), float(d["btb"]), int(d["nrows"]),
                                         1e-4, True)
    ref = d["x_dlasso_norm_1e-4"]
    assert stop == "objective increased"
    assert np.array_equal(x != 0, ref != 0)
    assert np.abs(x - ref).max() <= 1e-9 * np.abs(ref).max()


def _dlars64():
    import os
    from conftest import GOLDEN
    d = np.load(os.path.join(GOLDEN, "dlars64", "dlars64.npz"))
    X, y = d["X"], d["y"]
    return d, X.T @ X, X.T @ y, X.sum(0), float(y.sum()), float(y @ y), X.shape[0]


@pytest.mark.parametrize("case", ["lars", "lasso", "maxnorm", "lambda", "iters"])
def test_dlars_restatement_matches_reference_test_suite(case):
    """The reference DLARS's own 64 x 32 test problem (contrib/dlars/tests, --normalize=y)
    with its --algorithm, --max_norm=20, --lambda=5e-3 and --iterations=10 runs: the
    final coefficients it printed (13 significant digits) and its iteration count."""
    import dlars
    d, G, h, colsum, bsum, btb, n = _dlars64()
    lasso, lam, mn, its = d[case + "_params"]
    x, it, stop = dlars.dlars_normalized(G, h, colsum, bsum, btb, n, lam, bool(lasso), int(its), mn)
    mu = colsum / n
    sig = np.sqrt(np.diag(G) - n * mu * mu)
    ref = d[case + "_beta"]
    assert np.abs(x * sig - ref).max() <= 1e-11 * np.abs(ref).max()
    assert it == int(d[case + "_iterations"])
