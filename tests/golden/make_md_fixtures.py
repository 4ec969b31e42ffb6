"""Generate the MD fixtures of tests/golden/md_*/ with the reference's own chimes_md.

Run in a container where the reference sources are available:
    oracle/build_ref.sh && python tests/golden/make_md_fixtures.py
Per fixture: a seeded synthetic trajectory is fitted (numpy least squares on the
oracle's A, only to obtain a physically shaped coefficient vector x), params.txt is
written by the library's writer, and the reference chimes_md runs NVE from the
first frame with seeded 300 K velocities.  md_ref.npz keeps the configuration, x,
the velocities, the reference's forces of every step (forceout.txt, 15 digits) and
its per-step table (Ktot/N, Vtot/N, Etot/N, T, P from run_md.out).  md_nvt.npz (the
4-body fixture) keeps the same from CONSRNT NVT-MTK HOOVER 10 (plus Econs/N) and
NVT-BEREND 50 runs of 20 steps on the same inputs.
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
cg = importlib.import_module("chimes_lsq-myllfork_gb300")
from oracle import oracle  # noqa: E402

REF_MD = os.path.join(ROOT, "oracle", "_ref", "chimes_md")
KB = 0.0019872067   # kcal/mol/K (src/functions.h:43)

# name -> (workload, overrides, fit frames, seed, NVE steps)
MD_FIXTURES = {
    "md_water3b": ("water-3b", dict(nmol=32, L=9.86), 3, 31, 10),
    "md_ch4b": ("chno-4b", dict(natoms=40, order=(8, 4, 3), triclinic=False, density=0.1, species2=True), 8, 32, 10),
}

RUN_MD = """# RNDSEED #
	12357
# TEMPERA #
	300.0
# CMPRFRC #
	false
# TIMESTP #
	{dt}
# N_MDSTP #
	{steps}
# NLAYERS #
	1
# USENEIG #
	true
# PRMFILE #
	params.txt
# CRDFILE #
	input.xyzf
# VELINIT #
	READ
# CONSRNT #
	NVE
# PRSCALC #
	ANALYTICAL
# WRPCRDS #
	false
# FRQDFTB #
	1000
# FRQENER #
	1
# PRNTFRC #
	true 1
# ENDFILE #
"""


def header_types(model):
    lines = model.params_header().splitlines()
    i = next(k for k, ln in enumerate(lines) if ln.startswith("# TYPEIDX #"))
    n = int(next(ln for ln in lines if ln.startswith("ATOM TYPES:")).split()[2])
    rows = [lines[i + 1 + k].split() for k in range(n)]
    return [r[1] for r in rows], np.array([float(r[3]) for r in rows])


def read_first_frame(path, names):
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
    return n, np.array(types, dtype=np.int32), np.array(xyz), np.array(cell)


def make(name):
    wl, over, nfit, seed, steps = MD_FIXTURES[name]
    d = os.path.join(HERE, name)
    os.makedirs(d, exist_ok=True)
    fm = synth.make_workload(wl, d, nframes=nfit, seed=seed, **over)
    model = cg.Model(fm)
    A, b = oracle.assemble(fm, nthreads=8)
    lam = 1e-8 * np.abs(A).max() ** 2
    x = np.linalg.solve(A.T @ A + lam * np.eye(A.shape[1]), A.T @ b)
    names, masses = header_types(model)
    n, types, xyz, cell = read_first_frame(os.path.join(d, "traj.xyzf"), names)
    rng = np.random.default_rng(seed)
    tfs = 48.888   # internal time unit in fs (src/functions.h:44)
    v = rng.standard_normal((n, 3)) * np.sqrt(KB * 300.0 / masses[types])[:, None]
    v -= (masses[types][:, None] * v).sum(0) / masses[types].sum()
    dt = 0.2
    with tempfile.TemporaryDirectory() as tmp:
        open(os.path.join(tmp, "params.txt"), "w").write(model.params_txt(x, "! synthetic fit for MD fixtures\n!\n"))
        with open(os.path.join(tmp, "input.xyzf"), "w") as f:
            f.write(f"{n}\n")
            if cell[1] == 0 and cell[2] == 0 and cell[3] == 0 and cell[5] == 0 and cell[6] == 0 and cell[7] == 0:
                f.write(f"{cell[0]:.10f} {cell[4]:.10f} {cell[8]:.10f}\n")
            else:
                f.write("NON_ORTHO " + " ".join(f"{c:.10f}" for c in cell) + "\n")
            for k in range(n):
                f.write(f"{names[types[k]]} {xyz[k, 0]:.10f} {xyz[k, 1]:.10f} {xyz[k, 2]:.10f} "
                        f"{v[k, 0]:.16e} {v[k, 1]:.16e} {v[k, 2]:.16e}\n")
        open(os.path.join(tmp, "run_md.in"), "w").write(RUN_MD.format(dt=dt, steps=steps))
        p = subprocess.run([REF_MD, "run_md.in"], cwd=tmp, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"chimes_md failed for {name}:\n{p.stdout[-2000:]}")
        # read the positions / velocities back exactly as chimes_md parsed them
        _, _, xyz_in, _ = read_first_frame(os.path.join(tmp, "input.xyzf"), names)
        Fall = np.loadtxt(os.path.join(tmp, "forceout.txt")).reshape(-1, n, 3)
        table = []
        out = p.stdout.split("Ktot/N", 1)[1].split("END SIMULATION", 1)[0]
        for ln in out.splitlines():
            w = ln.split()
            if len(w) == 7 and w[0].isdigit():   # Step Time Ktot/N Vtot/N Etot/N T P (NVE)
                table.append([float(t) for t in w])
    vin = np.array([[float(t) for t in f"{v[k, 0]:.16e} {v[k, 1]:.16e} {v[k, 2]:.16e}".split()] for k in range(n)])
    np.savez_compressed(os.path.join(d, "md_ref.npz"), x=x, types=types, xyz=xyz_in, cell=cell, v=vin,
                        masses=masses, dt=dt, steps=steps, forces=Fall, table=np.array(table))
    os.remove(os.path.join(d, "traj.xyzf"))   # the fixture keeps its first frame in md_ref.npz
    print(name, "atoms", n, "cols", x.size, "force blocks", Fall.shape[0], "table rows", len(table))


def make_coul(name="md_watercoul", steps=10, seed=33):
    """Ewald MD: the FITCOUL water model (2B8 + 3B4 + charge products) with the
    short-range coefficients fitted on the watercoul fixture's reference A and
    consistent charges q_O = -0.82, q_H = +0.41 (products in Stillinger units, as
    chimes_lsq.py writes them); chimes_md runs NVE from the fixture's first frame."""
    src = os.path.join(HERE, "watercoul")
    d = os.path.join(HERE, name)
    os.makedirs(d, exist_ok=True)
    fm = open(os.path.join(src, "fm_setup.in")).read()
    open(os.path.join(d, "fm_setup.in"), "w").write(fm)
    model = cg.Model(os.path.join(d, "fm_setup.in"))
    ref = np.load(os.path.join(src, "ref.npz"))
    A, b = ref["A"], ref["b"]
    x = np.linalg.solve(A.T @ A + 1e-6 * np.abs(A).max() ** 2 * np.eye(A.shape[1]), A.T @ b)
    names, masses = header_types(model)
    ke = 332.0637157615209
    q = {"O": -0.82, "H": 0.41}
    ncoul, _ = model.charge_columns()
    hdr = model.params_header().splitlines()
    k = next(i for i, ln in enumerate(hdr) if ln.startswith("ATOM PAIRS:"))
    short = model.ncols - ncoul
    for p_ in range(ncoul):   # pair rows of the header: index, atom1, atom2
        w = hdr[k + 3 + p_].split()
        x[short + p_] = q[w[1]] * q[w[2]] * ke
    n, types, xyz, cell = read_first_frame(os.path.join(src, "traj.xyzf"), names)
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((n, 3)) * np.sqrt(KB * 300.0 / masses[types])[:, None]
    v -= (masses[types][:, None] * v).sum(0) / masses[types].sum()
    dt = 0.2
    with tempfile.TemporaryDirectory() as tmp:
        open(os.path.join(tmp, "params.txt"), "w").write(model.params_txt(x, "! synthetic fit for MD fixtures\n!\n"))
        with open(os.path.join(tmp, "input.xyzf"), "w") as f:
            f.write(f"{n}\n{cell[0]:.10f} {cell[4]:.10f} {cell[8]:.10f}\n")
            for j in range(n):
                f.write(f"{names[types[j]]} {xyz[j, 0]:.10f} {xyz[j, 1]:.10f} {xyz[j, 2]:.10f} "
                        f"{v[j, 0]:.16e} {v[j, 1]:.16e} {v[j, 2]:.16e}\n")
        open(os.path.join(tmp, "run_md.in"), "w").write(RUN_MD.format(dt=dt, steps=steps))
        p = subprocess.run([REF_MD, "run_md.in"], cwd=tmp, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"chimes_md failed for {name}:\n{p.stdout[-2000:]}")
        _, _, xyz_in, _ = read_first_frame(os.path.join(tmp, "input.xyzf"), names)
        Fall = np.loadtxt(os.path.join(tmp, "forceout.txt")).reshape(-1, n, 3)
        table = []
        out = p.stdout.split("Ktot/N", 1)[1].split("END SIMULATION", 1)[0]
        for ln in out.splitlines():
            w = ln.split()
            if len(w) == 7 and w[0].isdigit():
                table.append([float(t) for t in w])
    vin = np.array([[float(t) for t in f"{v[j, 0]:.16e} {v[j, 1]:.16e} {v[j, 2]:.16e}".split()] for j in range(n)])
    np.savez_compressed(os.path.join(d, "md_ref.npz"), x=x, types=types, xyz=xyz_in, cell=cell, v=vin,
                        masses=masses, dt=dt, steps=steps, forces=Fall, table=np.array(table))
    print(name, n, "atoms", Fall.shape, len(table))


def write_inputs(tmp, model, names, d, consrnt, steps):
    n = len(d["types"])
    cell, xyz, v, types = d["cell"], d["xyz"], d["v"], d["types"]
    open(os.path.join(tmp, "params.txt"), "w").write(model.params_txt(d["x"], "! synthetic fit for MD fixtures\n!\n"))
    with open(os.path.join(tmp, "input.xyzf"), "w") as f:
        f.write(f"{n}\n{cell[0]:.10f} {cell[4]:.10f} {cell[8]:.10f}\n")
        for k in range(n):
            f.write(f"{names[types[k]]} {xyz[k, 0]:.10f} {xyz[k, 1]:.10f} {xyz[k, 2]:.10f} "
                    f"{v[k, 0]:.16e} {v[k, 1]:.16e} {v[k, 2]:.16e}\n")
    open(os.path.join(tmp, "run_md.in"), "w").write(RUN_MD.format(dt=float(d["dt"]), steps=steps).replace("NVE", consrnt))


def make_nvt(name="md_ch4b", steps=20):
    d = np.load(os.path.join(HERE, name, "md_ref.npz"))
    model = cg.Model(os.path.join(HERE, name, "fm_setup.in"))
    names, _ = header_types(model)
    n = len(d["types"])
    out = {}
    for key, consrnt, ncol in (("mtk", "NVT-MTK HOOVER 10", 8), ("berend", "NVT-BEREND 50", 7)):
        with tempfile.TemporaryDirectory() as tmp:
            write_inputs(tmp, model, names, d, consrnt, steps)
            p = subprocess.run([REF_MD, "run_md.in"], cwd=tmp, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                               text=True)
            if p.returncode != 0:
                raise RuntimeError(f"chimes_md failed ({consrnt}):\n{p.stdout[-2000:]}")
            table = []
            body = p.stdout.split("Ktot/N", 1)[1].split("END SIMULATION", 1)[0]
            for ln in body.splitlines():
                w = ln.split()
                if len(w) == ncol and w[0].isdigit():
                    table.append([float(t) for t in w])
            out[f"table_{key}"] = np.array(table)
            out[f"forces_{key}"] = np.loadtxt(os.path.join(tmp, "forceout.txt")).reshape(-1, n, 3)
    np.savez_compressed(os.path.join(HERE, name, "md_nvt.npz"), steps=steps, tau_mtk=10.0, tau_berend=50.0,
                        temperature=300.0, **out)
    print(name, "nvt", {k: v.shape for k, v in out.items()})


def make_npt(name="md_ch4b", steps=20, pressure=1.0):
    """CONSRNT NPT-BEREND 50 100, NPT-BEREND-ANISO 50 100 and NPT-MTK HOOVER 10 100 at
    PRESSUR 1 GPa: the reference's per-step table (step, time, K/N, V/N, E/N, T, P,
    volume) and forces."""
    d = np.load(os.path.join(HERE, name, "md_ref.npz"))
    model = cg.Model(os.path.join(HERE, name, "fm_setup.in"))
    names, _ = header_types(model)
    n = len(d["types"])
    out = {}
    for key, consrnt in (("berend", "NPT-BEREND 50 100"), ("aniso", "NPT-BEREND-ANISO 50 100"),
                         ("mtk", "NPT-MTK HOOVER 10 100")):
        with tempfile.TemporaryDirectory() as tmp:
            write_inputs(tmp, model, names, d, consrnt, steps)
            run = open(os.path.join(tmp, "run_md.in")).read()
            run = run.replace("# TEMPERA #\n\t300.0\n", f"# TEMPERA #\n\t300.0\n# PRESSUR #\n\t{pressure}\n")
            open(os.path.join(tmp, "run_md.in"), "w").write(run)
            p = subprocess.run([REF_MD, "run_md.in"], cwd=tmp, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                               text=True)
            if p.returncode != 0:
                raise RuntimeError(f"chimes_md failed ({consrnt}):\n{p.stdout[-2000:]}")
            table = []
            body = p.stdout.split("Ktot/N", 1)[1].split("END SIMULATION", 1)[0]
            for ln in body.splitlines():
                w = ln.split()
                if len(w) == 8 and w[0].isdigit():
                    table.append([float(t) for t in w])
            out[f"table_{key}"] = np.array(table)
            out[f"forces_{key}"] = np.loadtxt(os.path.join(tmp, "forceout.txt")).reshape(-1, n, 3)
    np.savez_compressed(os.path.join(HERE, name, "md_npt.npz"), steps=steps, tau=10.0, tau_berend=50.0,
                        tau_baro=100.0, temperature=300.0, pressure=pressure, **out)
    print(name, "npt", {k: v.shape for k, v in out.items()})


def make_traj(name="md_ch4b", steps=6):
    """The reference's MD output files for a 6-step NVE run with FRQDFTB 1 and FRQRSTR 3:
    traj.gen / traj.xyz / traj.lammpstrj (TRAJEXT GEN, XYZ, LAMMPSTRJ), output.xyz,
    restart.xyzv (after step 6) and restart.bak (after step 3); and an NVT-MTK HOOVER 10
    run's restart.bak with its per-step table, to resume from."""
    d = np.load(os.path.join(HERE, name, "md_ref.npz"))
    model = cg.Model(os.path.join(HERE, name, "fm_setup.in"))
    names, _ = header_types(model)
    out = os.path.join(HERE, name, "traj")
    os.makedirs(out, exist_ok=True)
    tables = {}
    for ext, consrnt in (("GEN", "NVE"), ("XYZ", "NVE"), ("LAMMPSTRJ", "NVE"), ("GEN", "NVT-MTK HOOVER 10")):
        with tempfile.TemporaryDirectory() as tmp:
            write_inputs(tmp, model, names, d, consrnt, steps)
            run = open(os.path.join(tmp, "run_md.in")).read()
            run = run.replace("# FRQDFTB #\n\t1000\n", f"# FRQDFTB #\n\t1\n# TRAJEXT #\n\t{ext}\n# FRQRSTR #\n\t3\n")
            open(os.path.join(tmp, "run_md.in"), "w").write(run)
            p = subprocess.run([REF_MD, "run_md.in"], cwd=tmp, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                               text=True)
            if p.returncode != 0:
                raise RuntimeError(f"chimes_md failed ({ext}, {consrnt}):\n{p.stdout[-2000:]}")
            if consrnt == "NVE":
                shutil.copy(os.path.join(tmp, "traj." + ext.lower()), out)
                if ext == "GEN":
                    for f in ("output.xyz", "restart.xyzv", "restart.bak"):
                        shutil.copy(os.path.join(tmp, f), out)
            else:
                shutil.copy(os.path.join(tmp, "restart.bak"), os.path.join(out, "nvt_restart.bak"))
                table = []
                body = p.stdout.split("Ktot/N", 1)[1].split("END SIMULATION", 1)[0]
                for ln in body.splitlines():
                    w = ln.split()
                    if len(w) == 8 and w[0].isdigit():
                        table.append([float(t) for t in w])
                tables["table_nvt"] = np.array(table)
    np.savez_compressed(os.path.join(out, "tables.npz"), steps=steps, tau=10.0, temperature=300.0, **tables)
    print(name, "traj", sorted(os.listdir(out)))


def make_scale(name="md_ch4b", steps=8, freq=3):
    """CONSRNT NVT-SCALE 3 for 8 steps: the reference's per-step table."""
    d = np.load(os.path.join(HERE, name, "md_ref.npz"))
    model = cg.Model(os.path.join(HERE, name, "fm_setup.in"))
    names, _ = header_types(model)
    with tempfile.TemporaryDirectory() as tmp:
        write_inputs(tmp, model, names, d, f"NVT-SCALE {freq}", steps)
        p = subprocess.run([REF_MD, "run_md.in"], cwd=tmp, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"chimes_md failed (NVT-SCALE):\n{p.stdout[-2000:]}")
        table = []
        body = p.stdout.split("Ktot/N", 1)[1].split("END SIMULATION", 1)[0]
        for ln in body.splitlines():
            w = ln.split()
            if len(w) == 7 and w[0].isdigit():
                table.append([float(t) for t in w])
    out = os.path.join(HERE, name, "traj")
    os.makedirs(out, exist_ok=True)
    np.savez_compressed(os.path.join(out, "nvt_scale.npz"), steps=steps, freq=freq, temperature=300.0,
                        table=np.array(table))
    print(name, "nvt-scale", np.array(table).shape)


def make_velgen(name="md_ch4b", steps=2, seed=4321):
    """VELINIT GEN with RNDSEED 4321 and PRNTVEL every step: the reference's
    velocout.txt, whose first block holds the generated velocities after the
    centre-of-mass correction."""
    d = np.load(os.path.join(HERE, name, "md_ref.npz"))
    model = cg.Model(os.path.join(HERE, name, "fm_setup.in"))
    names, _ = header_types(model)
    with tempfile.TemporaryDirectory() as tmp:
        write_inputs(tmp, model, names, d, "NVE", steps)
        run = open(os.path.join(tmp, "run_md.in")).read()
        run = run.replace("# VELINIT #\n\tREAD\n", "# VELINIT #\n\tGEN\n# PRNTVEL #\n\ttrue 1\n")
        run = run.replace("# RNDSEED #\n\t12357\n", f"# RNDSEED #\n\t{seed}\n")
        assert "GEN" in run and str(seed) in run
        open(os.path.join(tmp, "run_md.in"), "w").write(run)
        p = subprocess.run([REF_MD, "run_md.in"], cwd=tmp, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"chimes_md failed (VELINIT GEN):\n{p.stdout[-2000:]}")
        out = os.path.join(HERE, name, "traj")
        shutil.copy(os.path.join(tmp, "velocout.txt"), os.path.join(out, "velgen_velocout.txt"))
    print(name, "velgen")


def make_numpress(name="md_ch4b", steps=6):
    """A 6-step NVE run with PRSCALC NUMERICAL: the reference's per-step table, whose P
    column is the finite-difference pressure plus the kinetic term."""
    d = np.load(os.path.join(HERE, name, "md_ref.npz"))
    model = cg.Model(os.path.join(HERE, name, "fm_setup.in"))
    names, _ = header_types(model)
    with tempfile.TemporaryDirectory() as tmp:
        write_inputs(tmp, model, names, d, "NVE", steps)
        run = open(os.path.join(tmp, "run_md.in")).read()
        run = run.replace("# PRSCALC #\n\tANALYTICAL\n", "# PRSCALC #\n\tNUMERICAL\n")
        assert "NUMERICAL" in run
        open(os.path.join(tmp, "run_md.in"), "w").write(run)
        p = subprocess.run([REF_MD, "run_md.in"], cwd=tmp, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"chimes_md failed (numerical pressure):\n{p.stdout[-2000:]}")
        table = []
        body = p.stdout.split("Ktot/N", 1)[1].split("END SIMULATION", 1)[0]
        for ln in body.splitlines():
            w = ln.split()
            if len(w) == 7 and w[0].isdigit():
                table.append([float(t) for t in w])
    out = os.path.join(HERE, name, "traj")
    os.makedirs(out, exist_ok=True)
    np.savez_compressed(os.path.join(out, "numpress.npz"), steps=steps, table=np.array(table))
    print(name, "numpress", np.array(table).shape)


if __name__ == "__main__":
    for nm in (sys.argv[1:] or list(MD_FIXTURES) + ["nvt", "npt", "traj", "numpress", "scale", "velgen", "md_watercoul"]):
        if nm == "traj":
            make_traj()
        elif nm == "numpress":
            make_numpress()
        elif nm == "scale":
            make_scale()
        elif nm == "velgen":
            make_velgen()
        elif nm == "npt":
            make_npt()
        elif nm == "nvt":
            make_nvt()
        elif nm == "md_watercoul":
            make_coul()
        else:
            make(nm)
