"""GPU MD force (cg_md_force*, cg_md_nve) against the oracle and the reference's
own chimes_md outputs (tests/golden/md_*/md_ref.npz).

Tolerances (FP64): forces within 1e-10 of the largest component, energy and
virial within 1e-10 relative.  FP32 contraction: forces within 2e-5 of the
largest component, energy within 2e-6 relative.  NVE against the reference's
10-step run: per-atom kinetic / potential energy to the printed 7 decimals
(5e-8), pressure to the printed 8 decimals, forces of every step within 1e-8.
"""
import importlib
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
GPA = 6.9476955
MD_FIXTURES = ["md_water3b", "md_ch4b"]


def load_md(name):
    d = np.load(os.path.join(GOLDEN, name, "md_ref.npz"))
    return os.path.join(GOLDEN, name, "fm_setup.in"), {k: d[k] for k in d.files}


def gpu_force(cg, fm, natoms, types, xyz, cell, x, precision=0, offsets=False):
    model = cg.Model(fm)
    sess = cg.Session(model, 0)
    sess.md_setup(x, precision=precision, energy_offsets=offsets)
    fr = cg.Frames.from_arrays(model, natoms, types, xyz, cell).independent()
    F, S = sess.md_force(fr)
    return F, S, sess


def close(a, b, rel):
    return np.abs(a - b).max() <= rel * max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("name", MD_FIXTURES)
def test_md_force_fp64_matches_reference_and_oracle(cg, oracle, name):
    fm, d = load_md(name)
    n = len(d["types"])
    F, S, sess = gpu_force(cg, fm, [n], d["types"], d["xyz"], d["cell"][None], d["x"], offsets=True)
    Fo, So = oracle.md_force(fm, [n], d["types"], d["xyz"], d["cell"][None], d["x"], offsets=True, nthreads=8)
    assert close(F, d["forces"][0], 1e-10)
    assert close(F, Fo, 1e-10)
    assert abs(S[0, 0] - So[0, 0]) <= 1e-10 * abs(So[0, 0])
    assert close(S[0, 1:], So[0, 1:], 1e-10)
    c = sess.md_last_counts()
    assert c["pairs"] > 0 and c["launches"] > 0


def _chno_batch(cg, tmp_path, sizes, triclinic, seed):
    synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
    fm = synth.make_workload("chno-4b", str(tmp_path), nframes=len(sizes), seed=seed, order=(8, 4, 3),
                             sizes=list(sizes), triclinic=triclinic, density=0.1)
    model = cg.Model(fm)
    nat, types, xyz, cell = synth.frames_arrays(os.path.join(str(tmp_path), "traj.xyzf"), len(sizes),
                                                ["C", "H", "N", "O"])[:4]
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(model.ncols) * 0.05
    return fm, model, (nat, types, xyz, cell), x


@pytest.mark.parametrize("triclinic", [False, True])
def test_md_force_batch_matches_oracle_and_each_alone(cg, oracle, tmp_path, triclinic):
    """Frames of different sizes in one batch: each result equals the oracle's and
    the same frame evaluated alone (atomics reorder sums: 1e-12 relative)."""
    sizes = [24, 60, 33] if not triclinic else [150, 90]
    fm, model, (nat, types, xyz, cell), x = _chno_batch(cg, tmp_path, sizes, triclinic, 71 + triclinic)
    F, S, _ = gpu_force(cg, fm, nat, types, xyz, cell, x)
    Fo, So = oracle.md_force(fm, nat, types, xyz, cell, x, nthreads=8)
    assert close(F, Fo, 1e-10)
    assert close(S, So, 1e-10)
    ofs = np.concatenate([[0], np.cumsum(nat)])
    for f in range(len(nat)):
        a, b = ofs[f], ofs[f + 1]
        F1, S1, _ = gpu_force(cg, fm, [nat[f]], types[a:b], xyz[a:b], cell[f:f + 1], x)
        assert close(F1, F[a:b], 1e-12)
        assert close(S1[0], S[f], 1e-12)


def test_md_force_small_cell_convention(cg, oracle):
    """Cell extent below the cut-off: unordered lists with PERM_SCALE 1/n!."""
    fm = os.path.join(GOLDEN, "small4b", "fm_setup.in")
    model = cg.Model(fm)
    synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
    nat, types, xyz, cell = synth.frames_arrays(os.path.join(GOLDEN, "small4b", "traj.xyzf"), 1, ["C", "H"])[:4]
    x = np.random.default_rng(5).standard_normal(model.ncols) * 0.05
    F, S, _ = gpu_force(cg, fm, nat, types, xyz, cell, x)
    Fo, So = oracle.md_force(fm, nat, types, xyz, cell, x, nthreads=4)
    assert close(F, Fo, 1e-10)
    assert close(S, So, 1e-10)


def test_md_force_equals_design_matrix_times_coefficients(cg):
    """The reference's verify-lsq-forces identity: MD forces = A x on the force rows
    (and energy / stress rows against the MD energy and virial) when no pair is
    inside s_min + 0.01 (the fit's 2-body rows skip r <= s_min)."""
    fm, d = load_md("md_ch4b")
    n = len(d["types"])
    model = cg.Model(fm)
    fr = cg.Frames.from_arrays(model, [n], d["types"], d["xyz"], d["cell"][None])
    sess = cg.Session(model, 0)
    A = sess.assemble(fr, cg.CG_FP64)
    sess.md_setup(d["x"], energy_offsets=True, penalty_scale=0.0)
    F, S = sess.md_force(fr)
    y = A @ d["x"]
    assert close(F.reshape(-1), y[:3 * n], 1e-10)
    rows = A.shape[0] - 3 * n
    if rows >= 12:   # 9 stress rows (xx xy xz yx yy yz zx zy zz) then 3 energy rows
        assert close(S[0, 2:11], y[3 * n:3 * n + 9], 1e-10)
        assert abs(y[-1] - S[0, 0]) <= 1e-10 * abs(S[0, 0])


@pytest.mark.parametrize("name", MD_FIXTURES)
def test_md_force_fp32_contraction_tolerance(cg, name):
    fm, d = load_md(name)
    n = len(d["types"])
    F64, S64, _ = gpu_force(cg, fm, [n], d["types"], d["xyz"], d["cell"][None], d["x"])
    F32, S32, _ = gpu_force(cg, fm, [n], d["types"], d["xyz"], d["cell"][None], d["x"], precision=1)
    err = np.abs(F32 - F64).max() / np.abs(F64).max()
    print(f"\n{name}: FP32-contraction force error {err:.3e} of max |F|", flush=True)
    assert err <= 2e-5
    assert abs(S32[0, 0] - S64[0, 0]) <= 2e-6 * abs(S64[0, 0])


@pytest.mark.parametrize("name", MD_FIXTURES)
def test_md_nve_matches_reference_run(cg, name):
    torch = pytest.importorskip("torch")
    fm, d = load_md(name)
    n = len(d["types"])
    steps = int(d["steps"]) - 1          # the reference prints steps 0..N_MDSTP-1
    model = cg.Model(fm)
    sess = cg.Session(model, 0)
    sess.md_setup(d["x"], energy_offsets=True)
    fr = cg.Frames.from_arrays(model, [n], d["types"], d["xyz"], d["cell"][None]).independent()
    F0, _ = sess.md_force(fr)
    dfr = sess.upload(fr)
    v = torch.from_numpy(d["v"].reshape(-1).copy()).cuda()
    Fd = torch.zeros(3 * n, dtype=torch.float64, device="cuda")
    So = torch.zeros((steps + 1, 11), dtype=torch.float64, device="cuda")
    ke = torch.zeros(steps + 1, dtype=torch.float64, device="cuda")
    sess.md_nve(dfr, d["masses"], float(d["dt"]), steps, v.data_ptr(), Fd.data_ptr(), So.data_ptr(), ke.data_ptr())
    torch.cuda.synchronize()
    So_h, ke_h = So.cpu().numpy(), ke.cpu().numpy()
    V = abs(np.linalg.det(d["cell"].reshape(3, 3)))
    tab = d["table"]
    assert close(F0, d["forces"][0], 1e-10)
    assert close(Fd.cpu().numpy().reshape(n, 3), d["forces"][steps], 1e-8)
    for s in range(steps + 1):
        kn = ke_h[s] / n
        vn = So_h[s, 0] / n
        p = (So_h[s, 1] + 2.0 * ke_h[s] / (3.0 * V)) * GPA
        assert abs(kn - tab[s, 2]) <= 5e-8 * max(1.0, abs(kn)) + 1e-12, (s, kn, tab[s, 2])
        assert abs(vn - tab[s, 3]) <= 5e-8 * max(1.0, abs(vn)) + 1e-12, (s, vn, tab[s, 3])
        assert abs(p - tab[s, 6]) <= 5e-9 * max(1.0, abs(p)) + 1e-12, (s, p, tab[s, 6])


def test_md_serving_results_same_alone_and_in_the_mix(cg, tmp_path):
    """Continuous batching: requests of different sizes arriving while others run
    give the same final positions as each request alone (one-at-a-time serving) and
    as the plain NVE call, within 1e-9 A after 6 steps (atomics reorder FP64 sums)."""
    torch = pytest.importorskip("torch")
    sizes = [40, 96, 64, 150, 33, 80]
    fm, model, (nat, types, xyz, cell), x = _chno_batch(cg, tmp_path, sizes, False, 91)
    x *= 0.02
    masses = np.array([12.011, 1.0079, 14.007, 15.9994])
    rng = np.random.default_rng(3)
    ofs = np.concatenate([[0], np.cumsum(nat)])
    reqs = []
    for k in range(len(sizes)):
        a, b = ofs[k], ofs[k + 1]
        v = rng.standard_normal((b - a, 3)) * 0.01
        reqs.append(dict(types=types[a:b], xyz=xyz[a:b], cell=cell[k], v=v, nsteps=6, arrival=0.0005 * k))
    sess = cg.Session(model, 0)
    sess.md_setup(x)
    mix, res, step_ms, nb = sess.md_serve(reqs, masses, dt_fs=0.2, max_batch_atoms=300, max_batch_frames=3)
    alone, res1, _, nb1 = sess.md_serve(reqs, masses, dt_fs=0.2, max_batch_frames=1)
    assert nb1 == 6 * len(sizes) and nb < nb1
    assert np.all(res["finished"] >= res["admitted"]) and np.all(step_ms > 0)
    for k, q in enumerate(reqs):
        assert np.abs(mix[k] - alone[k]).max() <= 1e-9
        # the plain NVE call on the same request
        fr = cg.Frames.from_arrays(model, [sizes[k]], q["types"], q["xyz"], q["cell"][None]).independent()
        dfr = sess.upload(fr)
        vd = torch.from_numpy(q["v"].reshape(-1).copy()).cuda()
        Fd = torch.zeros(3 * sizes[k], dtype=torch.float64, device="cuda")
        sess.md_nve(dfr, masses, 0.2, 5, vd.data_ptr(), Fd.data_ptr())
        torch.cuda.synchronize()
        pos = dfr.read_positions()
        assert np.abs(pos.reshape(-1, 3) - mix[k]).max() <= 1e-9


def test_md_skin_lists_match_per_step_enumeration(cg, tmp_path):
    """NVE with neighbour / cluster lists reused under a 0.5 A skin (rebuilt when an
    atom has moved 0.25 A) equals NVE that enumerates every step: same cluster sets,
    forces summed in another order (1e-9 A after 40 steps)."""
    torch = pytest.importorskip("torch")
    sizes = [64, 120]
    fm, model, (nat, types, xyz, cell), x = _chno_batch(cg, tmp_path, sizes, False, 55)
    x *= 0.02
    masses = np.array([12.011, 1.0079, 14.007, 15.9994])
    v0 = np.random.default_rng(8).standard_normal((int(sum(nat)), 3)) * 0.02
    out = []
    for skin_milli in (500, 0):
        sess = cg.Session(model, 0)
        sess.md_setup(x)
        sess.tune("md_skin_milli", skin_milli)
        fr = cg.Frames.from_arrays(model, nat, types, xyz, cell).independent()
        dfr = sess.upload(fr)
        v = torch.from_numpy(v0.reshape(-1).copy()).cuda()
        Fd = torch.zeros(3 * int(sum(nat)), dtype=torch.float64, device="cuda")
        sess.md_nve(dfr, masses, 0.5, 40, v.data_ptr(), Fd.data_ptr())
        torch.cuda.synchronize()
        out.append((dfr.read_positions(), Fd.cpu().numpy()))
    assert np.abs(out[0][0] - out[1][0]).max() <= 1e-9
    assert close(out[0][1], out[1][1], 1e-8)


@pytest.mark.parametrize("style", ["mtk", "berend"])
def test_md_nvt_matches_reference_run(cg, style):
    """CONSRNT NVT-MTK HOOVER 10 and NVT-BEREND 50 against the reference chimes_md on
    the 4-body fixture (tests/golden/md_ch4b/md_nvt.npz, 20 steps): per-step Ktot/N,
    Vtot/N and P to the printed digits, Econs/N for MTK (kinetic + potential + the
    thermostat's Q zeta^2 / 2 + N_DOF kB T s), and the last step's forces (1e-8)."""
    torch = pytest.importorskip("torch")
    fm, d = load_md("md_ch4b")
    t = np.load(os.path.join(GOLDEN, "md_ch4b", "md_nvt.npz"))
    tab = t[f"table_{style}"]
    n = len(d["types"])
    steps = int(t["steps"]) - 1
    model = cg.Model(fm)
    sess = cg.Session(model, 0)
    sess.md_setup(d["x"], energy_offsets=True)
    fr = cg.Frames.from_arrays(model, [n], d["types"], d["xyz"], d["cell"][None]).independent()
    dfr = sess.upload(fr)
    v = torch.from_numpy(d["v"].reshape(-1).copy()).cuda()
    Fd = torch.zeros(3 * n, dtype=torch.float64, device="cuda")
    So = torch.zeros((steps + 1, 11), dtype=torch.float64, device="cuda")
    ke = torch.zeros(steps + 1, dtype=torch.float64, device="cuda")
    cons = torch.zeros(steps + 1, dtype=torch.float64, device="cuda")
    st = cg.CG_NVT_MTK if style == "mtk" else cg.CG_NVT_BEREND
    tau = float(t["tau_mtk"] if style == "mtk" else t["tau_berend"])
    sess.md_nvt(dfr, d["masses"], float(d["dt"]), steps, st, float(t["temperature"]), tau, v.data_ptr(),
                Fd.data_ptr(), So.data_ptr(), ke.data_ptr(), cons.data_ptr())
    torch.cuda.synchronize()
    So_h, ke_h, c_h = So.cpu().numpy(), ke.cpu().numpy(), cons.cpu().numpy()
    V = abs(np.linalg.det(d["cell"].reshape(3, 3)))
    assert close(Fd.cpu().numpy().reshape(n, 3), t[f"forces_{style}"][steps], 1e-8)
    for s in range(steps + 1):
        kn, vn = ke_h[s] / n, So_h[s, 0] / n
        p = (So_h[s, 1] + 2.0 * ke_h[s] / (3.0 * V)) * GPA
        assert abs(kn - tab[s, 2]) <= 5e-8 * max(1.0, abs(kn)) + 1e-12, (s, kn, tab[s, 2])
        assert abs(vn - tab[s, 3]) <= 5e-8 * max(1.0, abs(vn)) + 1e-12, (s, vn, tab[s, 3])
        assert abs(p - tab[s, 6]) <= 5e-9 * max(1.0, abs(p)) + 1e-12, (s, p, tab[s, 6])
        if style == "mtk":
            en = (ke_h[s] + So_h[s, 0] + c_h[s]) / n
            assert abs(en - tab[s, 7]) <= 5e-8 * max(1.0, abs(en)) + 1e-12, (s, en, tab[s, 7])


def _md_coul_run(cg, steps):
    torch = pytest.importorskip("torch")
    fm, d = load_md("md_watercoul")
    n = len(d["types"])
    model = cg.Model(fm)
    sess = cg.Session(model, 0)
    sess.md_setup(d["x"])
    fr = cg.Frames.from_arrays(model, [n], d["types"], d["xyz"], d["cell"][None]).independent()
    F0, S0 = sess.md_force(fr)
    dfr = sess.upload(fr)
    v = torch.from_numpy(d["v"].reshape(-1).copy()).cuda()
    Fd = torch.zeros(3 * n, dtype=torch.float64, device="cuda")
    So = torch.zeros((steps + 1, 11), dtype=torch.float64, device="cuda")
    ke = torch.zeros(steps + 1, dtype=torch.float64, device="cuda")
    sess.md_nve(dfr, d["masses"], float(d["dt"]), steps, v.data_ptr(), Fd.data_ptr(), So.data_ptr(), ke.data_ptr())
    torch.cuda.synchronize()
    return d, n, F0, Fd.cpu().numpy().reshape(n, 3), So.cpu().numpy(), ke.cpu().numpy()


def test_md_coulomb_matches_reference_run(cg):
    """Ewald MD (charges from a FITCOUL fit's products, ZCalc_Ewald) against the
    reference chimes_md on 96 water atoms (tests/golden/md_watercoul): forces of step
    0 and of the last step (1e-10 / 1e-8 of max|F|), Ktot/N, Vtot/N and P of every
    step to the printed digits."""
    fm, dd = load_md("md_watercoul")
    steps = int(dd["steps"]) - 1
    d, n, F0, Fl, So_h, ke_h = _md_coul_run(cg, steps)
    assert close(F0, d["forces"][0], 1e-10)
    assert close(Fl, d["forces"][steps], 1e-8)
    V = abs(np.linalg.det(d["cell"].reshape(3, 3)))
    tab = d["table"]
    for s in range(steps + 1):
        kn, vn = ke_h[s] / n, So_h[s, 0] / n
        p = (So_h[s, 1] + 2.0 * ke_h[s] / (3.0 * V)) * GPA
        assert abs(kn - tab[s, 2]) <= 5e-8 * max(1.0, abs(kn)) + 1e-12, (s, kn, tab[s, 2])
        assert abs(vn - tab[s, 3]) <= 5e-8 * max(1.0, abs(vn)) + 1e-12, (s, vn, tab[s, 3])
        assert abs(p - tab[s, 6]) <= 5e-9 * max(1.0, abs(p)) + 1e-12, (s, p, tab[s, 6])


def test_fixed_charge_labels_lose_the_ewald_forces(cg, tmp_path):
    """Fixed charges (FITCOUL false, O -0.82 / H +0.41): cg_frames_subtract_coulomb
    removes from each force label the Ewald force that the MD force call (pinned on
    chimes_md by the Coulomb run above) gives the same frame with zero short-range
    coefficients.  (The reference chimes_lsq built here faults on this path: its
    ZCalc_Ewald writes PRESSURE_TENSORS_XYZ_ALL, which the LSQ frames never size.)"""
    import importlib
    synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
    fm = synth.make_workload("water-2b", str(tmp_path), nframes=2, seed=17, nmol=32, L=9.86, order=(8, 0, 0),
                             charges=[-0.82, 0.41], disp=0.1)
    model = cg.Model(fm)
    assert model.params_header().startswith("USECOUL: true")
    sess = cg.Session(model, 0)
    fr = cg.Frames.read(model)
    raw = fr.labels().copy()
    fr.subtract_coulomb(sess)
    got = fr.labels()
    sess.md_setup(np.zeros(model.ncols), penalty_scale=0.0)
    names = ["O", "H"]
    nat, types, xyz, cell = synth.frames_arrays(os.path.join(tmp_path, "traj.xyzf"), 2, names)[:4]
    r0 = 0
    a0 = 0
    for k in range(2):
        n = int(nat[k])
        one = cg.Frames.from_arrays(model, [n], types[a0:a0 + n], xyz[a0:a0 + n], cell[k:k + 1]).independent()
        F, _ = sess.md_force(one)
        expect = raw[r0:r0 + 3 * n] - F.reshape(-1)
        assert np.allclose(got[r0:r0 + 3 * n], expect, rtol=0, atol=1e-12 * np.abs(F).max())
        assert np.abs(F).max() > 1.0   # the charges do act
        r0 += 3 * n
        a0 += n


def test_hierarchical_md_force_equals_design_matrix(cg):
    """HIERARC fixture: with the reference solver's coefficients (zeros for the
    excluded O-H pair and H offset in its params.txt), the MD force read from that
    params.txt equals A x over the compacted columns, force and energy rows."""
    d = os.path.join(GOLDEN, "hierarc")
    model = cg.Model(os.path.join(d, "fm_setup.in"))
    x = model.params_read(open(os.path.join(d, "params.txt")).read())
    fr = cg.Frames.read(model)
    sess = cg.Session(model, 0)
    A = sess.assemble(fr, cg.CG_FP64)
    ref = np.load(os.path.join(d, "ref.npz"))
    colmax = np.abs(ref["A"]).max(axis=0)
    assert np.all(np.abs(A - ref["A"]) <= 1e-12 * np.abs(ref["A"]) + 1e-12 * colmax[None, :])
    sess.md_setup(x, energy_offsets=True, penalty_scale=0.0)
    y = A @ x
    natoms = 72   # 24 molecules; frame 0's rows: 216 force, 9 stress, 3 energy
    fr0 = cg.Frames.read(model, nframes=1).independent()
    F, S = sess.md_force(fr0)
    assert close(F.reshape(-1), y[:3 * natoms], 1e-10)
    assert abs(y[3 * natoms + 9] - S[0, 0]) <= 1e-10 * abs(S[0, 0])


@pytest.mark.parametrize("style", ["berend", "aniso", "mtk"])
def test_md_npt_matches_reference_run(cg, style):
    """CONSRNT NPT-BEREND 50 100, NPT-BEREND-ANISO 50 100 and NPT-MTK HOOVER 10 100 at
    1 GPa against the reference chimes_md on the 4-body fixture
    (tests/golden/md_ch4b/md_npt.npz, 20 steps): per-step Ktot/N, Vtot/N, P and the
    cell volume to the printed digits, and the last step's forces (1e-8)."""
    torch = pytest.importorskip("torch")
    fm, d = load_md("md_ch4b")
    t = np.load(os.path.join(GOLDEN, "md_ch4b", "md_npt.npz"))
    tab = t[f"table_{style}"]
    n = len(d["types"])
    steps = int(t["steps"]) - 1
    model = cg.Model(fm)
    sess = cg.Session(model, 0)
    sess.md_setup(d["x"], energy_offsets=True)
    fr = cg.Frames.from_arrays(model, [n], d["types"], d["xyz"], d["cell"][None]).independent()
    dfr = sess.upload(fr)
    v = torch.from_numpy(d["v"].reshape(-1).copy()).cuda()
    Fd = torch.zeros(3 * n, dtype=torch.float64, device="cuda")
    So = torch.zeros((steps + 1, 11), dtype=torch.float64, device="cuda")
    ke = torch.zeros(steps + 1, dtype=torch.float64, device="cuda")
    vol = torch.zeros(steps + 1, dtype=torch.float64, device="cuda")
    st = {"berend": cg.CG_NPT_BEREND, "aniso": cg.CG_NPT_BEREND_ANISO, "mtk": cg.CG_NPT_MTK}[style]
    tau = float(t["tau"] if style == "mtk" else t["tau_berend"])
    sess.md_npt(dfr, d["masses"], float(d["dt"]), steps, st, float(t["temperature"]), tau, float(t["pressure"]),
                float(t["tau_baro"]), v.data_ptr(), Fd.data_ptr(), So.data_ptr(), ke.data_ptr(), 0, vol.data_ptr())
    torch.cuda.synchronize()
    So_h, ke_h, V_h = So.cpu().numpy(), ke.cpu().numpy(), vol.cpu().numpy()
    assert close(Fd.cpu().numpy().reshape(n, 3), t[f"forces_{style}"][steps], 1e-8)
    for s in range(steps + 1):
        kn, vn = ke_h[s] / n, So_h[s, 0] / n
        p = (So_h[s, 1] + 2.0 * ke_h[s] / (3.0 * V_h[s])) * GPA
        assert abs(kn - tab[s, 2]) <= 5e-8 * max(1.0, abs(kn)) + 1e-12, (s, kn, tab[s, 2])
        assert abs(vn - tab[s, 3]) <= 5e-8 * max(1.0, abs(vn)) + 1e-12, (s, vn, tab[s, 3])
        assert abs(p - tab[s, 6]) <= 5e-9 * max(1.0, abs(p)) + 1e-12, (s, p, tab[s, 6])
        assert abs(V_h[s] - tab[s, 7]) <= 5e-8 * tab[s, 7], (s, V_h[s], tab[s, 7])


# ---------------------------------------------------------------- MD output files and restart
TRAJ = os.path.join(GOLDEN, "md_ch4b", "traj")
KB = 0.0019872067


def _nve_steps(cg, torch, nsteps):
    """The 4-body fixture run one NVE step per call: positions, velocities, forces and
    kinetic energy after each step (step 0 = the initial state)."""
    fm, d = load_md("md_ch4b")
    n = len(d["types"])
    model = cg.Model(fm)
    sess = cg.Session(model, 0)
    sess.md_setup(d["x"], energy_offsets=True)
    fr = cg.Frames.from_arrays(model, [n], d["types"], d["xyz"], d["cell"][None]).independent()
    dfr = sess.upload(fr)
    v = torch.from_numpy(d["v"].reshape(-1).copy()).cuda()
    Fd = torch.zeros(3 * n, dtype=torch.float64, device="cuda")
    ke = torch.zeros(2, dtype=torch.float64, device="cuda")
    states = []
    for s in range(nsteps + 1):
        sess.md_nve(dfr, d["masses"], float(d["dt"]), 0 if s == 0 else 1, v.data_ptr(), Fd.data_ptr(), 0,
                    ke.data_ptr())
        torch.cuda.synchronize()
        xs = dfr.read_positions()
        k = float(ke.cpu().numpy()[0 if s == 0 else 1])
        states.append(dict(xyz=xs.reshape(n, 3), v=v.cpu().numpy().reshape(n, 3), f=Fd.cpu().numpy().reshape(n, 3),
                           ke=k))
    return model, sess, d, n, states


def test_md_trajectory_files_match_reference(cg, tmp_path):
    """traj.gen / traj.xyz / traj.lammpstrj of a 6-step NVE run (FRQDFTB 1) written from
    the device run are byte-identical to the reference chimes_md's."""
    torch = pytest.importorskip("torch")
    model, sess, d, n, states = _nve_steps(cg, torch, 5)
    tfs = 48.888
    for fmt, name in ((cg.CG_TRAJ_GEN, "traj.gen"), (cg.CG_TRAJ_XYZ, "traj.xyz"),
                      (cg.CG_TRAJ_LAMMPSTRJ, "traj.lammpstrj")):
        out = tmp_path / name
        for s, st in enumerate(states):
            T = 2.0 * st["ke"] / ((3 * n - 3) * KB)
            model.md_write_traj(fmt, out, s, s, float(d["dt"]), T, d["types"], st["xyz"], st["v"], d["cell"])
        assert open(out).read() == open(os.path.join(TRAJ, name)).read(), name


def test_md_restart_written_and_resumed_like_reference(cg, tmp_path):
    """restart.xyzv after the 6-step NVE run matches the reference's numerically (step
    line, cell, positions, velocities, accelerations, N_DOF); and an NVT-MTK run resumed
    from the reference's restart file after its third step continues that run's table
    (Ktot/N, Vtot/N, Econs/N) to the printed digits."""
    torch = pytest.importorskip("torch")
    model, sess, d, n, states = _nve_steps(cg, torch, 5)
    last = states[-1]
    masses = np.asarray(d["masses"])[np.asarray(d["types"])]
    acc = last["f"] / masses[:, None]
    sess.md_write_restart(0, tmp_path / "restart.xyzv", d["types"], last["xyz"], last["v"], acc, d["cell"], 5,
                          float(model.md_read_restart(os.path.join(TRAJ, "restart.xyzv"), n)["padding"]))
    ours = model.md_read_restart(tmp_path / "restart.xyzv", n)
    ref = model.md_read_restart(os.path.join(TRAJ, "restart.xyzv"), n)
    assert ours["step"] == ref["step"] == 6
    assert np.array_equal(ours["types"], ref["types"]) and np.allclose(ours["cell"], ref["cell"], rtol=1e-14)
    for k in ("xyz", "v", "acc"):
        assert close(ours[k], ref[k], 1e-9), k
    assert ours["constraint"][26] == ref["constraint"][26]
    # resume an NVT-MTK run from the reference's restart file
    r = model.md_read_restart(os.path.join(TRAJ, "nvt_restart.bak"), n)
    tab = np.load(os.path.join(TRAJ, "tables.npz"))
    rows = tab["table_nvt"]
    fr = cg.Frames.from_arrays(model, [n], r["types"], r["xyz"], r["cell"][None]).independent()
    dfr = sess.upload(fr)
    v = torch.from_numpy(r["v"].reshape(-1).copy()).cuda()
    Fd = torch.zeros(3 * n, dtype=torch.float64, device="cuda")
    steps = len(rows) - r["step"]
    So = torch.zeros((steps + 1, 11), dtype=torch.float64, device="cuda")
    ke = torch.zeros(steps + 1, dtype=torch.float64, device="cuda")
    cons = torch.zeros(steps + 1, dtype=torch.float64, device="cuda")
    sess.md_resume(r["constraint"][None])
    sess.md_nvt(dfr, d["masses"], float(d["dt"]), steps, cg.CG_NVT_MTK, float(tab["temperature"]), float(tab["tau"]),
                v.data_ptr(), Fd.data_ptr(), So.data_ptr(), ke.data_ptr(), cons.data_ptr())
    torch.cuda.synchronize()
    So_h, ke_h, c_h = So.cpu().numpy(), ke.cpu().numpy(), cons.cpu().numpy()
    for s in range(steps + 1):
        row = rows[r["step"] - 1 + s]
        kn, vn, en = ke_h[s] / n, So_h[s, 0] / n, (ke_h[s] + So_h[s, 0] + c_h[s]) / n
        assert abs(kn - row[2]) <= 5e-8 * max(1.0, abs(kn)) + 1e-12, (s, kn, row[2])
        assert abs(vn - row[3]) <= 5e-8 * max(1.0, abs(vn)) + 1e-12, (s, vn, row[3])
        assert abs(en - row[7]) <= 5e-8 * max(1.0, abs(en)) + 1e-12, (s, en, row[7])


def test_md_numerical_pressure_and_stress(cg):
    """PRSCALC NUMERICAL: the finite-difference pressure of each step of a 6-step NVE
    run (all strained replicas of all steps in one batched force call) plus the kinetic
    term matches the reference chimes_md's printed P; the finite-difference stress
    tensor (STRSCALC NUMERICAL) agrees with the analytic virial tensor to the O(eps^2)
    truncation of the central difference."""
    torch = pytest.importorskip("torch")
    model, sess, d, n, states = _nve_steps(cg, torch, 5)
    tab = np.load(os.path.join(TRAJ, "numpress.npz"))["table"]
    k = len(states)
    fr = cg.Frames.from_arrays(model, [n] * k, np.tile(d["types"], k), np.concatenate([s["xyz"] for s in states]),
                               np.tile(d["cell"], (k, 1))).independent()
    P = sess.md_numerical_pressure(fr)
    V = abs(np.linalg.det(d["cell"].reshape(3, 3)))
    for s, st in enumerate(states):
        p = (P[s] + 2.0 * st["ke"] / (3.0 * V)) * GPA
        assert abs(p - tab[s, 6]) <= 2e-8 * max(1.0, abs(p)), (s, p, tab[s, 6])
    S = sess.md_numerical_stress(fr)
    F, So = sess.md_force(fr)
    for s in range(k):
        an = So[s, 2:11].reshape(3, 3)
        assert np.abs(S[s] - an).max() <= 1e-6 * np.abs(an).max(), (s, S[s], an)


def test_md_nvt_scale_matches_reference_run(cg):
    """CONSRNT NVT-SCALE 3 against the reference chimes_md (8 steps): per-step Ktot/N and
    Vtot/N to the printed digits across the rescalings after steps 3 and 6."""
    torch = pytest.importorskip("torch")
    fm, d = load_md("md_ch4b")
    t = np.load(os.path.join(TRAJ, "nvt_scale.npz"))
    tab = t["table"]
    n = len(d["types"])
    steps = int(t["steps"]) - 1
    model = cg.Model(fm)
    sess = cg.Session(model, 0)
    sess.md_setup(d["x"], energy_offsets=True)
    fr = cg.Frames.from_arrays(model, [n], d["types"], d["xyz"], d["cell"][None]).independent()
    dfr = sess.upload(fr)
    v = torch.from_numpy(d["v"].reshape(-1).copy()).cuda()
    Fd = torch.zeros(3 * n, dtype=torch.float64, device="cuda")
    So = torch.zeros((steps + 1, 11), dtype=torch.float64, device="cuda")
    ke = torch.zeros(steps + 1, dtype=torch.float64, device="cuda")
    sess.md_nvt(dfr, d["masses"], float(d["dt"]), steps, cg.CG_NVT_SCALE, float(t["temperature"]), float(t["freq"]),
                v.data_ptr(), Fd.data_ptr(), So.data_ptr(), ke.data_ptr())
    torch.cuda.synchronize()
    So_h, ke_h = So.cpu().numpy(), ke.cpu().numpy()
    for s in range(steps + 1):
        kn, vn = ke_h[s] / n, So_h[s, 0] / n
        assert abs(kn - tab[s, 2]) <= 5e-8 * max(1.0, abs(kn)) + 1e-12, (s, kn, tab[s, 2])
        assert abs(vn - tab[s, 3]) <= 5e-8 * max(1.0, abs(vn)) + 1e-12, (s, vn, tab[s, 3])
