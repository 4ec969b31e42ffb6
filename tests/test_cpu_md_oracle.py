"""The oracle's MD force (ZCalc / Cheby::Force_all restated) pinned against the
reference: its own chimes_md outputs on the committed MD fixtures (made by
tests/golden/make_md_fixtures.py) and, where the reference checkout is present,
the verify-lsq-forces goldens of its MD test suite.

Tolerances: forces 1e-10 of the largest component (the goldens carry 15
significant digits); per-atom energy 5e-8 and pressure 5e-9 GPa relative (the
printed digits of run_md.out)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, REFERENCE

GPA = 6.9476955   # src/functions.h:45
MD_FIXTURES = ["md_water3b", "md_ch4b"]


def load_md(name):
    d = np.load(os.path.join(GOLDEN, name, "md_ref.npz"))
    return os.path.join(GOLDEN, name, "fm_setup.in"), {k: d[k] for k in d.files}


def table_row(d, S, K):
    """Vtot/N and P (GPa) of run_md.out from the force scalars and kinetic energy."""
    n = len(d["types"])
    V = abs(np.linalg.det(d["cell"].reshape(3, 3)))
    return S[0] / n, (S[1] + 2.0 * K / (3.0 * V)) * GPA


@pytest.mark.parametrize("name", MD_FIXTURES)
def test_oracle_md_force_matches_reference_chimes_md(oracle, name):
    fm, d = load_md(name)
    n = len(d["types"])
    F, S = oracle.md_force(fm, [n], d["types"], d["xyz"], d["cell"][None], d["x"], offsets=True, nthreads=4)
    G = d["forces"][0]
    assert np.abs(F - G).max() <= 1e-10 * np.abs(G).max()
    m = d["masses"][d["types"]]
    K = 0.5 * (m[:, None] * d["v"] ** 2).sum()
    vn, p = table_row(d, S[0], K)
    assert abs(vn - d["table"][0, 3]) <= 5e-8 * max(1.0, abs(vn))
    assert abs(p - d["table"][0, 6]) <= 5e-9 * max(1.0, abs(p))


def test_oracle_md_force_is_minus_energy_gradient(oracle):
    fm, d = load_md("md_ch4b")
    n = len(d["types"])
    args = ([n], d["types"])
    F, _ = oracle.md_force(fm, *args, d["xyz"], d["cell"][None], d["x"], nthreads=4)
    h = 1e-5
    for a, c in [(0, 0), (7, 1), (23, 2)]:
        xp, xm = d["xyz"].copy(), d["xyz"].copy()
        xp[a, c] += h
        xm[a, c] -= h
        _, Sp = oracle.md_force(fm, *args, xp, d["cell"][None], d["x"], nthreads=4)
        _, Sm = oracle.md_force(fm, *args, xm, d["cell"][None], d["x"], nthreads=4)
        fd = -(Sp[0, 0] - Sm[0, 0]) / (2 * h)
        assert abs(fd - F[a, c]) <= 1e-5 * max(1.0, abs(F[a, c]))


# ---------------------------------------------------------------- reference MD suite
VERIFY = ["special3b", "special4b", "stress-and-ener-2b1", "stress-and-ener-4b", "stress-and-ener-4b2"]
REF_MD = os.path.join(REFERENCE, "test_suite-md")
needs_ref = pytest.mark.skipif(not os.path.isdir(REF_MD), reason="reference test suite not present")


def _header_types(cg, model):
    lines = model.params_header().splitlines()
    i = next(k for k, ln in enumerate(lines) if ln.startswith("# TYPEIDX #"))
    n = int(next(ln for ln in lines if ln.startswith("ATOM TYPES:")).split()[2])
    return [lines[i + 1 + k].split()[1] for k in range(n)]


def _read_xyz(path, names):
    L = open(path).read().split("\n")
    n = int(L[0].split()[0])
    t = L[1].split()
    if t[0] == "NON_ORTHO":
        cell = [float(v) for v in t[1:10]]
    else:
        a, b, c = (float(v) for v in t[:3])
        cell = [a, 0, 0, 0, b, 0, 0, 0, c]
    types, xyz = [], []
    for k in range(n):
        w = L[2 + k].split()
        types.append(names.index(w[0]))
        xyz.append([float(v) for v in w[1:4]])
    return n, np.array(types), np.array(xyz), np.array(cell)


@needs_ref
@pytest.mark.parametrize("case", VERIFY)
def test_oracle_md_force_matches_reference_suite(cg, oracle, case):
    """verify-lsq-forces-<case>: the suite's chimes_md forces (forceout.txt) for the
    LSQ case's fitted coefficients (test_suite_params.txt) on input.xyzf."""
    lsq = os.path.join(REFERENCE, "test_suite-lsq", case)
    md = os.path.join(REF_MD, "verify-lsq-forces-" + case)
    fm = os.path.join(lsq, "fm_setup.in")
    model = cg.Model(fm)
    x = np.array([float(ln.split()[1]) for ln in open(os.path.join(lsq, "correct_output", "test_suite_params.txt"))
                  if ln.strip()])
    runin = open(os.path.join(md, "run_md.in")).read().split("# CRDFILE #")[1].splitlines()[1:]
    crd = [ln for ln in runin if ln.strip()][0].split()[0]
    n, types, xyz, cell = _read_xyz(os.path.join(md, crd), _header_types(cg, model))
    F, _ = oracle.md_force(fm, [n], types, xyz, cell[None], x, nthreads=4)
    G = np.loadtxt(os.path.join(md, "correct_output", "forceout.txt")).reshape(-1, 3)
    assert np.abs(F - G).max() <= 1e-10 * np.abs(G).max()
