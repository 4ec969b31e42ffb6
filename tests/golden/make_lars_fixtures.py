"""Golden LARS-lasso and ridge coefficients from scikit-learn, the solvers the
reference's `chimes_lsq.py --algorithm lassolars / ridge` call (src/chimes_lsq.py:
216-263): `linear_model.LassoLars(alpha, fit_intercept=False, fit_path=False,
max_iter=100000)` and `linear_model.Ridge(alpha, fit_intercept=False)`.

Run where scikit-learn is installed (here: 1.9.0):
    python tests/golden/make_lars_fixtures.py
For each design-matrix fixture (tests/golden/<name>/ref.npz, made by the reference
binary) and penalty, tests/golden/lars/sklearn_lassolars.npz keeps the coefficients
and the number of LARS steps.
"""
import os

import numpy as np
import sklearn
from sklearn import linear_model

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = [("water2b", 1e-4), ("water2b", 1e-2), ("water3b", 1e-4), ("water3b", 1e-2), ("ch4b", 1e-4), ("ch4b", 1e-2)]


def main():
    out = {"sklearn_version": np.array(sklearn.__version__)}
    for name, alpha in CASES:
        d = np.load(os.path.join(HERE, name, "ref.npz"))
        reg = linear_model.LassoLars(alpha=alpha, fit_intercept=False, fit_path=False, max_iter=100000)
        reg.fit(d["A"], d["b"])
        key = f"{name}_{alpha:.0e}"
        out[key + "_coef"] = np.asarray(reg.coef_).ravel()
        out[key + "_steps"] = np.array(int(np.ravel(reg.n_iter_)[0]))
        print(key, "steps", int(np.ravel(reg.n_iter_)[0]), "nonzero", np.count_nonzero(out[key + "_coef"]))
    # the reference's --algorithm ridge: Ridge(alpha, fit_intercept=False)
    for name, alpha in (("water2b", 1e-3), ("ch4b", 1e-3)):
        d = np.load(os.path.join(HERE, name, "ref.npz"))
        reg = linear_model.Ridge(alpha=alpha, fit_intercept=False)
        reg.fit(d["A"], d["b"])
        out[f"{name}_ridge_{alpha:.0e}_coef"] = np.asarray(reg.coef_).ravel()
    np.savez_compressed(os.path.join(HERE, "lars", "sklearn_lassolars.npz"), **out)


if __name__ == "__main__":
    main()
