"""Seeded synthetic trajectories and fm_setup.in files for the benchmark workloads.

No public dataset is named for this path, so the workloads are generated:

* ``water``: rigid H2O (O-H 0.96 A, HOH 104.5 deg) at random positions and
  orientations with a minimum O-O distance of 2.5 A, optionally with Gaussian
  displacements; labels from a Lennard-Jones O-O term (eps 0.0067 eV,
  sigma 3.16 A) plus a harmonic intramolecular O-H term (22 eV/A^2).
* ``chno``: C/H/N/O atoms placed uniformly with a 0.9 A minimum separation in a
  triclinic or cubic cell; labels from a Morse pair term plus an Axilrod-Teller
  triple-dipole term.

Files follow the reference's formats: .xyzf (count line, box line with optional
stress and energy, ``type x y z fx fy fz`` with forces in Hartree/Bohr;
src/ClassDefs.C:2411-2683) and fm_setup.in (src/input.C).
"""
import os

import numpy as np

EV = 23.0605                                  # kcal/mol per eV
FCONV = 627.50960803 * 1.889725989            # file forces (Hartree/Bohr) -> kcal/mol/A
GPA = 6.9476955                               # kcal/mol/A^3 -> GPa factor used by the reference


def _pairs(x, cell, cut):
    """Unordered pairs (i<j) under the minimum-image convention with |d| < cut,
    d = image(x_j) - x_i.  Valid while cut is below half the cell's widths."""
    inv = np.linalg.inv(cell)
    f = x @ inv
    df = f[None, :, :] - f[:, None, :]
    df -= np.round(df)
    d = df @ cell
    r = np.linalg.norm(d, axis=2)
    ii, jj = np.nonzero(np.triu(r < cut, k=1))
    return ii, jj, d[ii, jj]


def _rot(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                     [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                     [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def water_frame(rng, nmol, L, disp_sigma=0.0, min_oo=2.5):
    cell = np.diag([L, L, L])
    centers = []
    tries = 0
    while len(centers) < nmol:
        tries += 1
        if tries > 200000:
            raise RuntimeError("could not place water molecules")
        c = rng.uniform(0, L, size=3)
        if centers:
            d = np.array(centers) - c
            d -= L * np.round(d / L)
            if np.min(np.linalg.norm(d, axis=1)) < min_oo:
                continue
        centers.append(c)
    half = np.deg2rad(104.5 / 2)
    body = 0.96 * np.array([[np.sin(half), 0.0, np.cos(half)], [-np.sin(half), 0.0, np.cos(half)]])
    xyz, types, mol = [], [], []
    for k, c in enumerate(centers):
        R = _rot(rng)
        xyz.append(c); types.append(0); mol.append(k)
        for h in body:
            xyz.append(c + R @ h); types.append(1); mol.append(k)
    xyz = np.array(xyz)
    if disp_sigma > 0:
        xyz = xyz + rng.normal(scale=disp_sigma, size=xyz.shape)
    return xyz % L, np.array(types, dtype=np.int32), cell, np.array(mol)


def water_labels(xyz, types, cell, mol):
    """Energy (kcal/mol), forces (kcal/mol/A), stress (kcal/mol/A^3, xx yy zz xy xz yz)."""
    eps, sig, k, r0 = 0.0067 * EV, 3.16, 22.0 * EV, 0.96
    i, j, d = _pairs(xyz, cell, 6.0)
    r = np.linalg.norm(d, axis=1)
    E = 0.0
    dEdr = np.zeros_like(r)
    oo = (types[i] == 0) & (types[j] == 0)
    sr6 = (sig / r[oo]) ** 6
    E += np.sum(4 * eps * (sr6 * sr6 - sr6))
    dEdr[oo] += 4 * eps * (-12 * sr6 * sr6 + 6 * sr6) / r[oo]
    oh = (mol[i] == mol[j]) & (types[i] != types[j]) & (r < 1.5)
    E += np.sum(0.5 * k * (r[oh] - r0) ** 2)
    dEdr[oh] += k * (r[oh] - r0)
    return _finish(xyz, cell, i, j, d, r, dEdr, E)


def _finish(xyz, cell, i, j, d, r, dEdr, E):
    F = np.zeros_like(xyz)
    u = d / r[:, None]
    g = dEdr[:, None] * u            # dE/dx_j
    np.add.at(F, j, -g)
    np.add.at(F, i, g)
    V = abs(np.linalg.det(cell))
    w = -(dEdr / r)[:, None, None] * d[:, :, None] * d[:, None, :]
    W = w.sum(axis=0) / V
    stress = np.array([W[0, 0], W[1, 1], W[2, 2], W[0, 1], W[0, 2], W[1, 2]])
    return E, F, stress


def chno_frame(rng, natoms, cell, min_sep=0.9, ntypes=4):
    inv = np.linalg.inv(cell)
    pts = np.empty((natoms, 3))
    n = 0
    tries = 0
    while n < natoms:
        tries += 1
        if tries > 500000:
            raise RuntimeError("could not place atoms")
        p = rng.uniform(0, 1, size=3) @ cell
        if n:
            d = pts[:n] - p
            f = d @ inv
            f -= np.round(f)
            if np.min(np.linalg.norm(f @ cell, axis=1)) < min_sep:
                continue
        pts[n] = p
        n += 1
    types = rng.integers(0, ntypes, size=natoms).astype(np.int32)
    return pts, types


def triclinic_cell(rng, lo=12.0, hi=16.0, alo=80.0, ahi=100.0):
    a, b, c = rng.uniform(lo, hi, size=3)
    al, be, ga = np.deg2rad(rng.uniform(alo, ahi, size=3))
    ax = np.array([a, 0, 0])
    bx = np.array([b * np.cos(ga), b * np.sin(ga), 0])
    cx_ = c * np.cos(be)
    cy = c * (np.cos(al) - np.cos(be) * np.cos(ga)) / np.sin(ga)
    cz = np.sqrt(c * c - cx_ * cx_ - cy * cy)
    return np.array([ax, bx, [cx_, cy, cz]])


def chno_labels(xyz, types, cell):
    """Morse pair + Axilrod-Teller triple-dipole, cut smoothly at 5.0 / 4.0 A."""
    De = np.array([0.10, 0.05, 0.08, 0.09]) * EV
    ii, jj, d = _pairs(xyz, cell, 5.0)
    r = np.linalg.norm(d, axis=1)
    D = np.sqrt(De[types[ii]] * De[types[jj]])
    a, re, rc = 1.6, 1.5, 5.0
    ex = np.exp(-a * (r - re))
    sw = (1 - r / rc) ** 2
    dsw = -2 * (1 - r / rc) / rc
    e = D * (1 - ex) ** 2 - D
    de = 2 * D * (1 - ex) * a * ex
    E = np.sum(e * sw)
    dEdr = de * sw + e * dsw
    E_at, F_at, W_at = _axilrod_teller(xyz, cell, ii, jj, d, r)
    E2, F2, S2 = _finish(xyz, cell, ii, jj, d, r, dEdr, E)
    return E2 + E_at, F2 + F_at, S2 + W_at


def _axilrod_teller(xyz, cell, ii, jj, d, r, nu=50.0, rc=4.0):
    """E = nu (1 + 3 cos g1 cos g2 cos g3) / (r12 r13 r23)^3 * prod (1 - r/rc)^2,
    summed over triangles with all sides below rc; forces and virial by autograd."""
    import torch
    n = len(xyz)
    sel = r < rc
    ii, jj, d = ii[sel], jj[sel], d[sel]
    # directed edges with image vectors, then triangles (a<b<c) from a's neighbours
    src = np.concatenate([ii, jj])
    dst = np.concatenate([jj, ii])
    vec = np.concatenate([d, -d])
    order = np.argsort(src, kind="stable")
    src, dst, vec = src[order], dst[order], vec[order]
    starts = np.searchsorted(src, np.arange(n + 1))
    A_, B_, C_, V1, V2 = [], [], [], [], []
    for a in range(n):
        s0, s1 = starts[a], starts[a + 1]
        nb, nv = dst[s0:s1], vec[s0:s1]
        m = nb > a
        nb, nv = nb[m], nv[m]
        if len(nb) < 2:
            continue
        p, q = np.triu_indices(len(nb), k=1)
        keep = nb[p] < nb[q]
        p, q = p[keep], q[keep]
        A_.append(np.full(len(p), a)); B_.append(nb[p]); C_.append(nb[q]); V1.append(nv[p]); V2.append(nv[q])
    if not A_:
        return 0.0, np.zeros_like(xyz), np.zeros(6)
    A_, B_, C_ = np.concatenate(A_), np.concatenate(B_), np.concatenate(C_)
    V1, V2 = np.concatenate(V1), np.concatenate(V2)
    x0 = torch.zeros((len(A_), 3), dtype=torch.float64, requires_grad=True)
    x1 = torch.tensor(V1, requires_grad=True)
    x2 = torch.tensor(V2, requires_grad=True)
    a1, a2, a3 = x1 - x0, x2 - x0, x2 - x1
    l1, l2, l3 = a1.norm(dim=1), a2.norm(dim=1), a3.norm(dim=1)
    c1 = (a1 * a2).sum(1) / (l1 * l2)
    c2 = -(a1 * a3).sum(1) / (l1 * l3)
    c3 = (a2 * a3).sum(1) / (l2 * l3)
    fc = (1 - l1 / rc).clamp(min=0) ** 2 * (1 - l2 / rc).clamp(min=0) ** 2 * (1 - l3 / rc).clamp(min=0) ** 2
    e = nu * (1 + 3 * c1 * c2 * c3) / (l1 * l2 * l3) ** 3 * fc
    E = e.sum()
    E.backward()
    g0, g1, g2 = x0.grad.numpy(), x1.grad.numpy(), x2.grad.numpy()
    F = np.zeros_like(xyz)
    np.add.at(F, A_, -g0)
    np.add.at(F, B_, -g1)
    np.add.at(F, C_, -g2)
    Wt = -(np.einsum("ka,kb->ab", V1, g1) + np.einsum("ka,kb->ab", V2, g2))
    V = abs(np.linalg.det(cell))
    W = (Wt + Wt.T) / 2 / V
    return float(E.detach()), F, np.array([W[0, 0], W[1, 1], W[2, 2], W[0, 1], W[0, 2], W[1, 2]])


# ---------------------------------------------------------------- writers
def write_xyzf(path, frames, species):
    """frames: list of dicts with xyz, types, cell (3x3 rows), forces (kcal/mol/A),
    optional stress (kcal/mol/A^3: xx yy zz xy xz yz) and energy (kcal/mol)."""
    with open(path, "w") as f:
        for fr in frames:
            cell = fr["cell"]
            f.write(f"{len(fr['xyz'])}\n")
            ortho = np.allclose(cell - np.diag(np.diag(cell)), 0.0)
            if ortho:
                box = " ".join(f"{v:.10f}" for v in np.diag(cell))
            else:
                box = "NON_ORTHO " + " ".join(f"{v:.10f}" for v in cell.reshape(-1))
            extra = ""
            if fr.get("stress") is not None:
                extra += " " + " ".join(f"{v * GPA:.10e}" for v in fr["stress"])
            if fr.get("energy") is not None:
                extra += f" {fr['energy']:.10e}"
            f.write(box + extra + "\n")
            for t, x, F in zip(fr["types"], fr["xyz"], fr["forces"]):
                Ff = F / FCONV
                f.write(f"{species[t]} {x[0]:.10f} {x[1]:.10f} {x[2]:.10f} {Ff[0]:.10e} {Ff[1]:.10e} {Ff[2]:.10e}\n")


def write_fm_setup(path, xyzf_name, nframes, species, masses, order2, order3, order4, smin, smax2, lam,
                   smax3=None, smax4=None, fitstrs=None, fitener=False, nlayers=1, fitcoul=False, charges=None):
    """fitcoul: fit the Ewald charge products (FITCOUL true, charge signs instead of
    charges, npairs-1 CHARGE CONSTRAINTS lines tying the products together)."""
    lines = ["####### CONTROL VARIABLES #######", "", "# TRJFILE #", f"\t{xyzf_name}", "# WRAPTRJ #", "\ttrue",
             "# NFRAMES #", f"\t{nframes}", "# NLAYERS #", f"\t{nlayers}", "# FITCOUL #",
             "\ttrue" if fitcoul else "\tfalse"]
    if fitstrs:
        lines += ["# FITSTRS #", f"\t{fitstrs}"]
    if fitener:
        lines += ["# FITENER #", "\ttrue"]
    lines += ["# PAIRTYP #", f"\tCHEBYSHEV {order2} {order3} {order4}", "# CHBTYPE #", "\tMORSE", "",
              "####### TOPOLOGY VARIABLES #######", "", "# NATMTYP # ", f"\t{len(species)}", "",
              "# TYPEIDX #\t# ATM_TYP #\t# ATMCHRG #\t# ATMMASS #"]
    for k, (s, m) in enumerate(zip(species, masses)):   # charges: fixed charges (Ewald subtraction)
        chg = ("-" if k == 0 else "+") if fitcoul else (f"{charges[k]}" if charges else "0.0")
        lines.append(f"{k + 1}\t\t{s}\t\t{chg}\t\t{m}")
    lines += ["", "# PAIRIDX #\t# ATM_TY1 #\t# ATM_TY1 #\t# S_MINIM #\t# S_MAXIM #\t# S_DELTA #\t# MORSE_LAMBDA #"]
    k = 1
    n = len(species)
    pairs = [(i, i) for i in range(n)] + [(i, j) for i in range(n) for j in range(i + 1, n)]
    for a, b in pairs:
        lines.append(f"{k}\t\t{species[a]}\t\t{species[b]}\t\t{smin}\t\t{smax2}\t\t0.01\t\t{lam}")
        k += 1
    if fitcoul:   # npairs-1 constraints: names, one weight per pair, force
        names = [species[a] + species[b] for a, b in pairs]
        lines.append("CHARGE CONSTRAINTS:")
        for c in range(len(pairs) - 1):
            w = [10000.0 * (1 + ((c + i) % 3)) * (-1 if (c + i) % 2 else 1) for i in range(len(pairs))]
            lines.append("\t".join(names + [f"{v:.1f}" for v in w] + ["0.0"]))
    if order3 and smax3 is not None:
        lines += ["", f"SPECIAL 3B S_MAXIM: ALL {smax3}"]
    if order4 and smax4 is not None:
        lines += ["", f"SPECIAL 4B S_MAXIM: ALL {smax4}"]
    lines += ["", "# FCUTTYP #", "\tCUBIC", "", "# ENDFILE #", ""]
    with open(path, "w") as f:
        f.write("\n".join(lines))


# ---------------------------------------------------------------- workloads
WORKLOADS = {
    # water-2b: plain 2-body, forces only (64 molecules, 10 frames)
    "water-2b": dict(kind="water", nmol=64, L=12.42, nframes=10, disp=0.0, order=(12, 0, 0), smin=0.8,
                     smax=(5.0, None, None), lam=1.4, fitstrs=None, fitener=False),
    # water-3b: 2B 16 @ 5.0, 3B 8 @ 4.0, forces + energy + full stress (128 molecules, 200 frames)
    "water-3b": dict(kind="water", nmol=128, L=15.65, nframes=200, disp=0.1, order=(16, 8, 0), smin=0.8,
                     smax=(5.0, 4.0, None), lam=1.4, fitstrs="ALL", fitener=True),
    # chno-4b: C/H/N/O triclinic, 2B 16 / 3B 8 / 4B 4 at 5.0 / 4.0 / 3.5 (256 atoms)
    "chno-4b": dict(kind="chno", natoms=256, nframes=1000, order=(16, 8, 4), smin=0.8, smax=(5.0, 4.0, 3.5),
                    lam=1.4, fitstrs="ALL", fitener=True, triclinic=True),
}


def _chno_labels_many(args):
    return [chno_labels(*a) for a in args]


def _labels_parallel(jobs, workers):
    """chno_labels of every (xyz, types, cell) job, in a pool of `workers` fresh
    interpreters (spawn: safe beside an initialised CUDA context); same values as
    the serial loop, since each frame's labels depend on that frame alone."""
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    chunks = [jobs[i::workers] for i in range(workers)]
    with ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
        parts = list(ex.map(_chno_labels_many, chunks))
    out = [None] * len(jobs)
    for i, part in enumerate(parts):
        out[i::workers] = part
    return out


def make_workload(name, outdir, nframes=None, seed=1234, labels=True, workers=1, **over):
    """Write <outdir>/fm_setup.in and <outdir>/traj.xyzf; returns the fm_setup.in path.
    workers > 1 computes the C/H/N/O labels in that many processes."""
    cfg = dict(WORKLOADS[name])
    cfg.update(over)
    if nframes is not None:
        cfg["nframes"] = nframes
    os.makedirs(outdir, exist_ok=True)
    rng = np.random.default_rng(seed)
    frames = []
    if cfg["kind"] == "water":
        species, masses = ["O", "H"], [15.9994, 1.0079]
        for _ in range(cfg["nframes"]):
            xyz, types, cell, mol = water_frame(rng, cfg["nmol"], cfg["L"], cfg["disp"])
            if labels:
                E, F, S = water_labels(xyz, types, cell, mol)
            else:
                E, F, S = 0.0, np.zeros_like(xyz), np.zeros(6)
            frames.append(dict(xyz=xyz, types=types, cell=cell, forces=F,
                               stress=S if cfg["fitstrs"] else None, energy=E if cfg["fitener"] else None))
    else:
        species, masses = ["C", "H", "N", "O"], [12.011, 1.0079, 14.007, 15.9994]
        if cfg.get("species2"):
            species, masses = species[:2], masses[:2]
        sizes = cfg.get("sizes")
        geo = []
        for k in range(cfg["nframes"]):
            n = int(sizes[k]) if sizes is not None else cfg["natoms"]
            if cfg.get("triclinic", False):
                cell = triclinic_cell(rng)
            else:
                L = (n / cfg.get("density", 0.1)) ** (1.0 / 3.0)
                cell = np.diag([L, L, L])
            xyz, types = chno_frame(rng, n, cell, ntypes=len(species))
            geo.append((xyz, types, cell))
        if not labels:
            lab = [(0.0, np.zeros_like(g[0]), np.zeros(6)) for g in geo]
        elif workers > 1 and len(geo) > 1:
            lab = _labels_parallel(geo, min(workers, len(geo)))
        else:
            lab = [chno_labels(*g) for g in geo]
        for (xyz, types, cell), (E, F, S) in zip(geo, lab):
            frames.append(dict(xyz=xyz, types=types, cell=cell, forces=F,
                               stress=S if cfg["fitstrs"] else None, energy=E if cfg["fitener"] else None))
    write_xyzf(os.path.join(outdir, "traj.xyzf"), frames, species)
    o2, o3, o4 = cfg["order"]
    s2, s3, s4 = cfg["smax"]
    p = os.path.join(outdir, "fm_setup.in")
    write_fm_setup(p, "traj.xyzf", cfg["nframes"], species, masses, o2, o3, o4, cfg["smin"], s2, cfg["lam"],
                   smax3=s3, smax4=s4, fitstrs=cfg["fitstrs"], fitener=cfg["fitener"],
                   fitcoul=cfg.get("fitcoul", False), charges=cfg.get("charges"))
    return p


def frames_arrays(frames_xyzf_path, nframes, species):
    """Parse a synthetic .xyzf into arrays for Frames.from_arrays (cell rows a,b,c)."""
    nat, typ, xyz, frc, cell, st, en = [], [], [], [], [], [], []
    with open(frames_xyzf_path) as f:
        for _ in range(nframes):
            n = int(f.readline())
            tk = f.readline().split()
            if tk[0] == "NON_ORTHO":
                c = np.array(list(map(float, tk[1:10])))
                rest = tk[10:]
            else:
                c = np.diag(list(map(float, tk[0:3]))).reshape(-1)
                rest = tk[3:]
            cell.append(c)
            vals = list(map(float, rest))
            st.append(vals[:6] + [0.0] * max(0, 6 - len(vals[:6])))
            en.append(vals[-1] if vals else 0.0)
            nat.append(n)
            for _ in range(n):
                t = f.readline().split()
                typ.append(species.index(t[0]))
                xyz.append(list(map(float, t[1:4])))
                frc.append(list(map(float, t[4:7])))
    return (np.array(nat, np.int32), np.array(typ, np.int32), np.array(xyz), np.array(cell), np.array(frc),
            np.array(st), np.array(en))
