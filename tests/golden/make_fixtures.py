"""Generate the golden fixtures of tests/golden/ with the reference's own chimes_lsq.

Run in a container where the reference sources are available:
    python oracle/build_ref.sh && python tests/golden/make_fixtures.py
Each fixture directory holds the seeded synthetic inputs (fm_setup.in, traj.xyzf)
and ref.npz with the reference's A matrix and b vector (read back from its
A.txt / b.txt, written with %.16e, so the round trip is exact); a FITCOUL fixture's
A ends with the charge-constraint rows, as the reference writes them.
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
synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
REF = os.path.join(ROOT, "oracle", "_ref", "chimes_lsq")
REF_DIR = os.environ.get("CHIMES_REF_DIR", "/root/reference")
REF_PY = os.path.join(REF_DIR, "src", "chimes_lsq.py")   # the reference's solver script (read in place)

# name -> (workload, overrides, nframes, seed)
FIXTURES = {
    # 2-body water, forces only (the water-2b basis)
    "water2b": ("water-2b", {}, 2, 11),
    # 2B16 + 3B8 water with full stress and energy rows (the water-3b basis), 32 molecules
    "water3b": ("water-3b", dict(nmol=32, L=9.86), 1, 12),
    # C/H triclinic with 2B8 / 3B4 / 4B3, stress and energy rows
    "ch4b": ("chno-4b", dict(natoms=40, order=(8, 4, 3), triclinic=False, density=0.1, species2=True), 2, 13),
    # small cubic cell (extent below the cut-off): unordered neighbour convention, PERM_SCALE 1/n!
    "small4b": ("chno-4b", dict(natoms=12, order=(6, 3, 2), triclinic=False, density=0.1, species2=True,
                                fitstrs=None, fitener=True), 1, 14),
    # 32 water molecules with the Ewald charge columns and charge constraints (FITCOUL)
    "watercoul": ("water-2b", dict(nmol=32, L=9.86, order=(8, 4, 0), smax=(5.0, 4.0, None), fitcoul=True,
                                   disp=0.1), 2, 15),
    # two trajectory files of different sizes behind TRJFILE MULTI, label flags on the second
    "multifile": ("multi", {}, 3, 16),
    # SKPFRMS 2 over 5 frames (frames 0, 2, 4 kept) with stress rows for the first 3
    # trajectory frames only (FITSTRS FIRSTALL 3): the cut-off counts trajectory frames
    "skipframes": ("water-3b", dict(nmol=24, L=8.96, order=(8, 4, 0), fitstrs="FIRSTALL 3", fitener=True), 5, 18),
    # HIERARC: the O-H 2-body block and the H energy offset left out of A
    "hierarc": ("water-3b", dict(nmol=24, L=8.96, order=(8, 4, 0), fitstrs="ALL", fitener=True), 2, 19),
}

# The input branches of the remaining fm_setup.in options, each a C/H 4-body system
# (or water for the inverse-r transform) with one option changed; the cut-off
# blocks use the reference's syntax (src/input.C:690-874, 1207-1282, src/Fcut.C:40-65).
CH4B = dict(order=(6, 3, 2), triclinic=False, density=0.1, species2=True)
FIXTURES.update({
    # TERSOFF smooth cut-off with offset 0.5, a cell wide enough for the ordered lists
    "tersoff": ("chno-4b", dict(CH4B, natoms=120), 1, 21),
    # inverse-r Chebyshev transform (water, 2-body + 3-body)
    "invr": ("water-3b", dict(nmol=24, L=8.96, order=(8, 4, 0), fitstrs="ALL", fitener=True), 1, 22),
    # no transform (x = r)
    "notrans": ("chno-4b", dict(CH4B, natoms=60), 1, 23),
    # per-cluster-type S_MAXIM and S_MINIM of 3- and 4-body types (SPECIAL ... SPECIFIC)
    "specific": ("chno-4b", dict(CH4B, natoms=120), 1, 24),
    # 3- and 4-body cluster types left out of A (EXCLUDE 3B / 4B INTERACTION)
    "exclude": ("chno-4b", dict(CH4B, natoms=60), 1, 25),
    # below-s_min variants of the 3/4-body basis (CHEBYFIX), with inner cut-offs raised
    # to 1.3 A so that pairs at 0.9-1.3 A fall below them
    "chebyfix_zero": ("chno-4b", dict(CH4B, natoms=60), 1, 26),
    "chebyfix_const": ("chno-4b", dict(CH4B, natoms=60), 1, 27),
    "chebyfix_smooth": ("chno-4b", dict(CH4B, natoms=60), 1, 28),
})
RAISE_SMIN = "\nSPECIAL 3B S_MINIM: ALL 1.3\n\nSPECIAL 4B S_MINIM: ALL 1.3\n"
PATCH = {   # name -> [(old, new), ...] applied to the generated fm_setup.in
    "tersoff": [("\tCUBIC", "\tTERSOFF 0.5")],
    "invr": [("\tMORSE", "\tINVRSE_R")],
    "notrans": [("\tMORSE", "\tNONE")],
    "specific": [("SPECIAL 3B S_MAXIM: ALL 4.0",
                  "SPECIAL 3B S_MAXIM: SPECIFIC 2\nCCCCCC CC CC CC 4.2 4.2 4.2\nCCCHCH CC CH CH 3.9 3.6 3.6\n\n"
                  "SPECIAL 3B S_MINIM: SPECIFIC 1\nCHCHHH CH CH HH 1.1 1.1 1.2"),
                 ("SPECIAL 4B S_MAXIM: ALL 3.5",
                  "SPECIAL 4B S_MAXIM: SPECIFIC 2\nCCCCCCCCCCCC CC CC CC CC CC CC 3.6 3.6 3.6 3.6 3.6 3.6\n"
                  "CCCCCHCCCHCH CC CC CH CC CH CH 3.4 3.4 3.1 3.4 3.1 3.1")],
    "exclude": [("# ENDFILE #", "EXCLUDE 3B INTERACTION: 1\nC C H\n\nEXCLUDE 4B INTERACTION: 2\nC C C H\n"
                                "H H H H\n\n# ENDFILE #")],
    "chebyfix_zero": [("# PAIRTYP #", "# CHEBYFIX #\n\tZERO_DERIV\n# PAIRTYP #"),
                      ("# FCUTTYP #", RAISE_SMIN + "\n# FCUTTYP #")],
    "chebyfix_const": [("# PAIRTYP #", "# CHEBYFIX #\n\tCONSTANT_DERIV\n# PAIRTYP #"),
                       ("# FCUTTYP #", RAISE_SMIN + "\n# FCUTTYP #")],
    "chebyfix_smooth": [("# PAIRTYP #", "# CHEBYFIX #\n\tSMOOTH 0.02\n# PAIRTYP #"),
                        ("# FCUTTYP #", RAISE_SMIN + "\n# FCUTTYP #")],
}

SKIP = {"skipframes": 2}
HIER = {"hierarc": ("EXCLUDE 1B INTERACTION: 1\nH\n\nEXCLUDE 2B INTERACTION: 1\nO H\n")}


def make_multifile(d):
    """Two trajectory files (32 and 24 water molecules) behind a MULTI list, with
    label flags on the second file: TRJFILE MULTI traj_list.dat."""
    with tempfile.TemporaryDirectory() as t1, tempfile.TemporaryDirectory() as t2:
        synth.make_workload("water-3b", t1, nframes=2, seed=16, nmol=32, L=9.86, order=(8, 4, 0), fitstrs="ALL",
                            fitener=True)
        synth.make_workload("water-3b", t2, nframes=1, seed=17, nmol=24, L=8.96, order=(8, 4, 0), fitstrs="ALL",
                            fitener=True)
        shutil.copy(os.path.join(t1, "traj.xyzf"), os.path.join(d, "part_a.xyzf"))
        shutil.copy(os.path.join(t2, "traj.xyzf"), os.path.join(d, "part_b.xyzf"))
        fm = open(os.path.join(t1, "fm_setup.in")).read()
    fm = fm.replace("# TRJFILE #\n\ttraj.xyzf", "# TRJFILE #\n\tMULTI traj_list.dat")
    fm = fm.replace("# NFRAMES #\n\t2", "# NFRAMES #\n\t3")
    open(os.path.join(d, "fm_setup.in"), "w").write(fm)
    open(os.path.join(d, "traj_list.dat"), "w").write("2\n2 part_a.xyzf\n1 part_b.xyzf 300.0 fa_ sb_ eb_\n")
    return ["part_a.xyzf", "part_b.xyzf", "traj_list.dat"]


def make(name):
    wl, over, nframes, seed = FIXTURES[name]
    d = os.path.join(HERE, name)
    os.makedirs(d, exist_ok=True)
    inputs = ["traj.xyzf"]
    if wl == "multi":
        inputs = make_multifile(d)
    else:
        synth.make_workload(wl, d, nframes=nframes, seed=seed, **over)
    if name in SKIP:
        fm = open(os.path.join(d, "fm_setup.in")).read()
        key = f"# NFRAMES #\n\t{nframes}\n"
        assert key in fm
        fm = fm.replace(key, key + f"# SKPFRMS #\n\t{SKIP[name]}\n")
        open(os.path.join(d, "fm_setup.in"), "w").write(fm)
    if name in PATCH:
        fm = open(os.path.join(d, "fm_setup.in")).read()
        for a, b in PATCH[name]:
            assert a in fm, (name, a)
            fm = fm.replace(a, b, 1)
        open(os.path.join(d, "fm_setup.in"), "w").write(fm)
    if name in HIER:
        fm = open(os.path.join(d, "fm_setup.in")).read()
        key = f"# NFRAMES #\n\t{nframes}\n"
        assert key in fm and "# ENDFILE #" in fm
        fm = fm.replace(key, key + "# HIERARC #\n\ttrue\n")
        fm = fm.replace("# ENDFILE #", HIER[name] + "\n# ENDFILE #")
        open(os.path.join(d, "fm_setup.in"), "w").write(fm)
    with tempfile.TemporaryDirectory() as tmp:
        shutil.copy(os.path.join(d, "fm_setup.in"), tmp)
        for f in inputs:
            shutil.copy(os.path.join(d, f), tmp)
        subprocess.run([REF, "fm_setup.in"], cwd=tmp, check=True, stdout=subprocess.DEVNULL)
        A = np.loadtxt(os.path.join(tmp, "A.txt"), ndmin=2)
        b = np.loadtxt(os.path.join(tmp, "b.txt"))
        for f in ("params.header", "ff_groups.map"):
            shutil.copy(os.path.join(tmp, f), os.path.join(d, f))
        if wl == "multi":   # the labels file carries the per-file flags
            shutil.copy(os.path.join(tmp, "b-labeled.txt"), os.path.join(d, "b-labeled.txt"))
        if name in HIER:   # the reference's solver script on that A: params.txt with the exclusions
            out = subprocess.run([sys.executable, REF_PY, "--test_suite", "true"], cwd=tmp, check=True,
                                 capture_output=True, text=True).stdout
            open(os.path.join(d, "params.txt"), "w").write(out)
            shutil.copy(os.path.join(tmp, "test_suite_params.txt"), os.path.join(d, "test_suite_params.txt"))
    np.savez_compressed(os.path.join(d, "ref.npz"), A=A, b=b)
    print(name, A.shape)


if __name__ == "__main__":
    for n in (sys.argv[1:] or FIXTURES):
        make(n)
