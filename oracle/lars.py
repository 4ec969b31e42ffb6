"""LARS with the lasso modification on the normal equations -- TEST INFRASTRUCTURE ONLY.

A plain numpy restatement used by tests/ as the checker of the device LARS
(cg_lars).  The reference's `--algorithm lassolars` calls scikit-learn's
`linear_model.LassoLars(alpha, fit_intercept=False, fit_path=False,
max_iter=100000)` (src/chimes_lsq.py:248-263); its DLARS code
(contrib/dlars/src/dlars.C:471-2221, Cholesky updates in solve_G_A :1101-1329)
implements the same published algorithm: Efron, Hastie, Johnstone and Tibshirani,
"Least angle regression", Ann. Statist. 32 (2004), sections 2-3.  The lasso
solution minimises  (1 / 2n) ||y - X w||^2 + alpha ||w||_1  (n = rows of X).

Written from the paper on G = X^T X and h = X^T y:
  correlations c = h - G w; C = max |c_j|; the active set moves along the
  equiangular direction w_A = A_A G_AA^-1 s_A (A_A = (s_A^T G_AA^-1 s_A)^-1/2);
  the step ends when an inactive correlation reaches the active ones, or (lasso)
  when an active coefficient crosses zero (that variable leaves, and no variable
  enters on the next step); the path stops exactly at C / n = alpha.
The factor of G_AA is kept by rank-1 additions and Givens-rotation deletions.
"""
import numpy as np


def _chol_add(L, g_col, g_jj):
    """Append one variable to the lower Cholesky factor L of G_AA."""
    k = L.shape[0]
    if k == 0:
        return np.array([[np.sqrt(g_jj)]])
    l = np.linalg.solve(L, g_col) if k < 64 else _fwd(L, g_col)
    d2 = g_jj - l @ l
    if not d2 > 1e-13 * g_jj:   # dependent on the active set
        return None
    Ln = np.zeros((k + 1, k + 1))
    Ln[:k, :k] = L
    Ln[k, :k] = l
    Ln[k, k] = np.sqrt(d2)
    return Ln


def _fwd(L, b):
    x = np.zeros_like(b)
    for i in range(len(b)):
        x[i] = (b[i] - L[i, :i] @ x[:i]) / L[i, i]
    return x


def _chol_delete(L, k):
    """Factor of G_AA without variable k: drop row k, restore the lower
    triangle with Givens rotations on neighbouring columns."""
    n = L.shape[0]
    M = np.delete(L, k, axis=0)            # (n-1) x n, rows >= k have one extra entry
    for j in range(k, n - 1):
        a, b = M[j, j], M[j, j + 1]
        r = np.hypot(a, b)
        cs, sn = a / r, b / r
        cj, cj1 = M[j:, j].copy(), M[j:, j + 1].copy()
        M[j:, j] = cs * cj + sn * cj1
        M[j:, j + 1] = -sn * cj + cs * cj1
    return M[:, : n - 1]


def _solve(L, s):
    y = np.linalg.solve(L, s) if L.shape[0] < 64 else _fwd(L, s)
    return np.linalg.solve(L.T, y)


def lars_lasso(G, h, n_samples, alpha, max_iter=100000, tiny=0.0):
    """Coefficients of the lasso at penalty alpha, and the number of steps."""
    G = np.asarray(G, dtype=np.float64)
    h = np.asarray(h, dtype=np.float64)
    p = h.size
    beta = np.zeros(p)
    c = h.copy()
    active = []
    is_active = np.zeros(p, dtype=bool)
    L = np.zeros((0, 0))
    drop = False
    just_dropped = -1
    C = np.abs(c).max() if p else 0.0
    steps = 0
    target = n_samples * alpha
    while steps < max_iter:
        if C <= target:
            break
        if not drop:
            cand = np.where(~is_active, np.abs(c), -1.0)
            j = int(np.argmax(cand))
            if cand[j] < 0:
                break
            Ln = _chol_add(L, G[np.array(active, dtype=int), j], G[j, j])
            if Ln is None:           # collinear with the active set: leave it out
                is_active[j] = True   # never reconsidered
                continue
            L = Ln
            active.append(j)
            is_active[j] = True
            C = max(C, abs(c[j]))
        drop = False
        idx = np.array(active, dtype=int)
        s = np.sign(c[idx])
        w = _solve(L, s)
        AA = 1.0 / np.sqrt(s @ w)
        w *= AA
        a = G[:, idx] @ w
        gamma = C / AA                # all correlations reach zero
        inact = ~is_active
        if inact.any():
            ci, ai = c[inact], a[inact]
            with np.errstate(divide="ignore", invalid="ignore"):
                g1 = (C - ci) / (AA - ai)
                g2 = (C + ci) / (AA + ai)
            if just_dropped >= 0:
                # the variable that just left sits at c = +-C: its same-sign root is the
                # current point; only the opposite-sign crossing is a new event
                kk = int(np.searchsorted(np.flatnonzero(inact), just_dropped))
                if c[just_dropped] > 0:
                    g1[kk] = np.inf
                else:
                    g2[kk] = np.inf
            cand = np.concatenate([g1, g2])
            cand = cand[np.isfinite(cand) & (cand > tiny)]
            if cand.size:
                gamma = min(gamma, cand.min())
        just_dropped = -1
        # lasso: the first active coefficient to cross zero
        with np.errstate(divide="ignore", invalid="ignore"):
            z = -beta[idx] / w
        zpos = np.where(z > tiny, z, np.inf)
        kz = int(np.argmin(zpos)) if zpos.size else -1
        if kz >= 0 and zpos[kz] < gamma:
            gamma = zpos[kz]
            drop = True
        # stop exactly at alpha
        if C - gamma * AA < target:
            gamma = (C - target) / AA
            drop = False
            beta[idx] += gamma * w
            steps += 1
            break
        beta[idx] += gamma * w
        c -= gamma * a
        C -= gamma * AA
        steps += 1
        if drop:
            k = kz
            beta[active[k]] = 0.0
            is_active[active[k]] = False
            just_dropped = active[k]
            L = _chol_delete(L, k)
            del active[k]
    return beta, steps
