"""Golden vectors of the reference's DLARS solver on its own 64 x 32 test problem
(contrib/dlars/tests: X.64.32.txt, Y.64.32.txt and the committed outputs in
correct_output/), for the device DLARS options --max_norm, --lambda and --iterations.

    CHIMES_REF_DIR=/path/to/reference python tests/golden/make_dlars64_fixture.py

Writes tests/golden/dlars64/dlars64.npz: the inputs X (64 x 32) and y, and per case the
final coefficients the reference printed ("Final values: Beta:", the normalised
problem's coefficients, --normalize=y), its stop message and iteration count.
"""
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(os.environ.get("CHIMES_REF_DIR", "/root/reference"), "contrib", "dlars", "tests")

# name -> (output file, lasso, lambda, max_norm, iterations): the Makefile's
# lars / lasso / stopping targets on X.64.32 (all with --normalize=y)
CASES = {
    "lars": ("dlars.64.32.txt", 0, 0.0, 1e50, 10000000),
    "lasso": ("dlasso.64.32.txt", 1, 0.0, 1e50, 10000000),
    "maxnorm": ("dlasso.64.32.mn.txt", 1, 0.0, 20.0, 10000000),
    "lambda": ("dlasso.64.32.lam.txt", 1, 5.0e-3, 1e50, 10000000),
    "iters": ("dlasso.64.32.its.txt", 1, 0.0, 1e50, 10),
}


def final_beta(text, nprops):
    tail = text[text.rindex("Final values:"):]
    block = tail[tail.index("[") + 1: tail.index("]")]
    beta = np.zeros(nprops)
    for line in block.strip().splitlines():
        k, v = line.split()
        beta[int(k)] = float(v)
    return beta


def main():
    nprops, ndata = map(int, open(os.path.join(REF, "X.64.32.dim")).read().split())
    X = np.loadtxt(os.path.join(REF, "X.64.32.txt")).reshape(ndata, nprops)
    y = np.loadtxt(os.path.join(REF, "Y.64.32.txt"))
    out = {"X": X, "y": y}
    for name, (fn, lasso, lam, mn, its) in CASES.items():
        text = open(os.path.join(REF, "correct_output", fn)).read()
        out[name + "_beta"] = final_beta(text, nprops)
        out[name + "_params"] = np.array([lasso, lam, mn, its], dtype=np.float64)
        out[name + "_iterations"] = np.array(len(re.findall(r"^Finished iteration \d+", text, re.M)))
        stop = re.findall(r"^Stopping: (.*)$", text, re.M)
        out[name + "_stop"] = np.array(stop[-1] if stop else "iterations")
    os.makedirs(os.path.join(HERE, "dlars64"), exist_ok=True)
    np.savez_compressed(os.path.join(HERE, "dlars64", "dlars64.npz"), **out)
    print({k: (v.shape if v.ndim else v) for k, v in out.items()})


if __name__ == "__main__":
    main()
