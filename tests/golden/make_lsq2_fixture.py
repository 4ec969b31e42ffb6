"""Normal equations of the reference's lsq2 case and its solvers' published answers.

lsq2 (test_suite-lsq/lsq2: 33 frames of 96-atom water, FITCOUL with two charge
constraints, 2B10 / 3B6 / 4B2, 9,506 x 419 A) is the case the reference's own
suite uses for its solvers.  This script runs the reference's chimes_lsq
(oracle/_ref) on it, forms G = A^T A (upper triangle), h = A^T b and b^T b, and
reads the coefficients of the reference's committed outputs
params.ridge.1.0e-03.txt, params.lassolars.1.0e-04.txt, params.dlars.1.0e-04.txt
params.dlasso.1.0e-04.txt and params.dlasso.norm.txt (chimes_lsq.py --algorithm
ridge / lassolars / dlars / dlasso, the last with --normalize) with this
package's params.txt reader; A^T 1 and the sum of b serve the normalisation.

Run where the reference sources are present:
    sh oracle/build_ref.sh && python tests/golden/make_lsq2_fixture.py
"""
import importlib
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
cg = importlib.import_module("chimes_lsq-myllfork_gb300")
REF = os.path.join(ROOT, "oracle", "_ref", "chimes_lsq")
CASE = os.path.join(os.environ.get("CHIMES_REF_DIR", "/root/reference"), "test_suite-lsq", "lsq2")


def main():
    out = os.path.join(HERE, "lsq2")
    os.makedirs(out, exist_ok=True)
    with tempfile.TemporaryDirectory() as tmp:
        for f in ("fm_setup.in", "input.xyzf"):
            shutil.copy(os.path.join(CASE, f), tmp)
        subprocess.run([REF, "fm_setup.in"], cwd=tmp, check=True, stdout=subprocess.DEVNULL)
        A = np.loadtxt(os.path.join(tmp, "A.txt"))
        b = np.loadtxt(os.path.join(tmp, "b.txt"))
        m = cg.Model(os.path.join(tmp, "fm_setup.in"))
    G = A.T @ A
    iu = np.triu_indices(G.shape[0])
    gold = {}
    for key, name in (("x_ridge_1e-3", "params.ridge.1.0e-03.txt"), ("x_lassolars_1e-4", "params.lassolars.1.0e-04.txt"),
                      ("x_dlars_1e-4", "params.dlars.1.0e-04.txt"), ("x_dlasso_1e-4", "params.dlasso.1.0e-04.txt"),
                      ("x_dlasso_norm_1e-4", "params.dlasso.norm.txt")):
        gold[key] = m.params_read(open(os.path.join(CASE, "correct_output", name)).read())
    np.savez_compressed(os.path.join(out, "normal.npz"), G_upper=G[iu], h=A.T @ b, btb=float(b @ b),
                        colsum=A.sum(axis=0), bsum=float(b.sum()), nrows=A.shape[0], ncols=A.shape[1], **gold)
    print("lsq2", A.shape, {k: float(np.abs(v).max()) for k, v in gold.items()})


if __name__ == "__main__":
    main()
