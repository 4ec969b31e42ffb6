"""DLARS restatement on the normal equations -- TEST INFRASTRUCTURE ONLY (the checker
of the device cg_dlars; nothing in the product imports it).

The reference's DLARS solver (contrib/dlars/src/dlars.C, `chimes_lsq.py --algorithm
dlars | dlasso`, src/chimes_lsq.py:714-790) walks the LARS path of Efron, Hastie,
Johnstone and Tibshirani (Ann. Stat. 32, 407-499, 2004) over the unnormalised A:

* correlations c = A^T (b - mu), C = max |c_j| (DLARS::correlation, :1484-1518);
* the first index with ||c_j| - C| < 1e-6 enters when no step named one
  (update_active_set, :1896-1955);
* signed active Gram G_A = s s^T * G[A, A], A_A = (1^T G_A^-1 1)^-1/2,
  w_A = A_A G_A^-1 1, a = A^T u_A = sum_k w_k s_k G[:, A_k] (build_u_A, :1829-1883,
  chol_backsub :1332-1417);
* step gamma = min over inactive j of the positive (C -+ c_j) / (A_A -+ a_j)
  (update_step_gamma, :1957-1997); the lasso variant also stops where an active
  coefficient reaches zero, min over gamma_i = -beta_i / (s_i w_i) > 1e-12
  (update_lasso_gamma, :1999-2017), and drops that variable before the next step;
* the objective 0.5 ||b - A beta||^2 / n + lambda ||beta||_1 is evaluated at every
  vertex (objective_func, :1476-1482); the driver (:376-420) stops at the first
  vertex whose objective exceeds the previous one's by more than 1e-10 and reports
  that vertex (its `last_beta` holds the coefficients of the step just taken).

Here ||b - A beta||^2 = b^T b - beta^T h - beta^T c with c = h - G beta, so only the
normal equations (G, h, b^T b, n) are needed.
"""
import numpy as np


def dlars(G, h, btb, n, lam, lasso, max_iter=10000000, max_norm=1.0e50):
    """Returns (beta, iterations, stop) for DLARS `--algorithm lars` (lasso False)
    or `lasso` (lasso True) with `--lambda lam`, `--normalize n`, `--iterations
    max_iter` and `--max_norm max_norm` (the driver stops once the L1 norm of the
    coefficients after a step exceeds it and keeps the vertex before that step,
    contrib/dlars/src/dlars.C:376-381)."""
    G = np.asarray(G, dtype=np.float64)
    h = np.asarray(h, dtype=np.float64)
    p = G.shape[0]
    beta = np.zeros(p)
    c = h.copy()
    active = []
    add_prop = -1
    remove_prop = -1
    drop = False
    last_beta = beta.copy()
    last_obj = 1.0e50
    it = 0
    stop = "iterations"
    while it + 1 <= max_iter:
        if len(active) >= p:
            stop = "no more iterations"
            break
        obj = 0.5 * (btb - beta @ h - beta @ c) / n + lam * np.abs(beta).sum()
        C = np.abs(c).max()
        if drop:
            active.pop(remove_prop)
        elif add_prop >= 0:
            active.append(add_prop)
        else:
            for j in range(p):
                if abs(abs(c[j]) - C) < 1e-6 and j not in active:
                    active.append(j)
                    break
        A = np.array(active)
        s = np.where(c[A] < 0, -1.0, 1.0)
        GA = G[np.ix_(A, A)] * np.outer(s, s)
        L = np.linalg.cholesky(GA)
        gi = np.linalg.solve(L.T, np.linalg.solve(L, np.ones(len(A))))
        AA = 1.0 / np.sqrt(gi.sum())
        w = AA * gi
        a = G[:, A] @ (w * s)
        gamma = 1.0e20
        add_prop = -1
        if len(A) < p:
            inact = np.ones(p, bool)
            inact[A] = False
            for j in np.nonzero(inact)[0]:
                c1 = (C - c[j]) / (AA - a[j])
                c2 = (C + c[j]) / (AA + a[j])
                if 0.0 < c1 < gamma:
                    gamma, add_prop = c1, j
                if 0.0 < c2 < gamma:
                    gamma, add_prop = c2, j
        else:
            gamma = C / AA
        gamma_lasso = 1.0e20
        remove_prop = -1
        if lasso:
            for i in range(len(A)):
                if abs(w[i]) > 1.0e-40:
                    gi_ = -beta[A[i]] / (s[i] * w[i])
                    if 1.0e-12 < gi_ < gamma_lasso:
                        gamma_lasso, remove_prop = gi_, i
        drop = lasso and gamma > gamma_lasso
        g = gamma_lasso if drop else gamma
        beta[A] += w * s * g
        if drop:
            beta[A[remove_prop]] = 0.0
        c = c - g * a
        it += 1
        if np.abs(beta).sum() > max_norm:
            stop = "max norm"
            break
        if obj > last_obj + 1.0e-10:
            stop = "objective increased"
            break
        last_beta = beta.copy()
        last_obj = obj
    return last_beta, it, stop


def dlars_normalized(G, h, colsum, bsum, btb, n, lam, lasso, max_iter=10000000, max_norm=1.0e50):
    """DLARS with --normalize=y (Matrix::normalize / Vector::normalize,
    contrib/dlars/src/Matrix.h:614-660, Vector.h:140-150; print_unscaled
    dlars.C:2073-2097): columns centred and scaled to unit norm, b centred;
    returns the unscaled coefficients (beta / scale), iterations, stop reason."""
    G = np.asarray(G, dtype=np.float64)
    mu = np.asarray(colsum, dtype=np.float64) / n
    ybar = bsum / n
    sig = np.sqrt(np.diag(G) - n * mu * mu)
    if np.any(~(sig > 0.0)):
        raise ValueError("a column of A is constant: its normalisation scale is 0")
    Gc = (G - n * np.outer(mu, mu)) / np.outer(sig, sig)
    hc = (np.asarray(h) - ybar * np.asarray(colsum)) / sig
    beta, it, stop = dlars(Gc, hc, btb - n * ybar * ybar, n, lam, lasso, max_iter, max_norm)
    return beta / sig, it, stop
