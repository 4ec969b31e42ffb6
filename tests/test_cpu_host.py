"""CPU-only checks: the C ABI library loads and exports its header, the host
topology reproduces the reference's params.header / ff_groups.map, the labels
(b) and row layout match, and the CPU oracle reproduces the reference's A."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from conftest import FIXTURES, GOLDEN, REFERENCE, ROOT, fixture_dir, frame_part

HEADER = os.path.join(ROOT, "include", "chimes_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(cg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(cg):
    lib = cg.lib()
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    assert len(declared_symbols()) >= 20


@pytest.mark.parametrize("name", FIXTURES)
def test_header_and_map_match_reference(cg, name):
    d = fixture_dir(name)
    m = cg.Model(os.path.join(d, "fm_setup.in"))
    assert m.params_header() == open(os.path.join(d, "params.header")).read()
    assert m.ff_groups_map() == open(os.path.join(d, "ff_groups.map")).read()


@pytest.mark.parametrize("name", FIXTURES)
def test_labels_and_rows_match_reference(cg, name):
    d = fixture_dir(name)
    ref = np.load(os.path.join(d, "ref.npz"))
    m = cg.Model(os.path.join(d, "fm_setup.in"))
    fr = cg.Frames.read(m)
    A, b, Ac, bc = frame_part(m, ref)
    assert fr.nrows == A.shape[0]
    assert m.ncols == ref["A"].shape[1]
    assert np.array_equal(fr.labels(), b)
    Cc, cb = m.constraint_rows()   # FITCOUL charge-constraint rows (none otherwise)
    assert np.array_equal(Cc, Ac) and np.array_equal(cb, bc)


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_matches_reference_fixture(cg, oracle, name):
    d = fixture_dir(name)
    A, b = oracle.assemble(os.path.join(d, "fm_setup.in"), nthreads=4)
    ref = np.load(os.path.join(d, "ref.npz"))
    R, rb, _, _ = frame_part(cg.Model(os.path.join(d, "fm_setup.in")), ref)
    colmax = np.abs(R).max(axis=0)
    assert np.all(np.abs(A - R) <= 4e-16 * np.abs(R) + 1e-15 * colmax[None, :])
    assert np.array_equal(b, rb)


def test_model_errors_are_reported(cg, tmp_path):
    with pytest.raises(cg.ChimesError) as e:
        cg.Model(str(tmp_path / "missing.in"))
    assert e.value.code == 2
    # charge columns with stress / energy rows: the reference prints no charge
    # columns there, so the combination is refused
    src = open(os.path.join(fixture_dir("water3b"), "fm_setup.in")).read()
    bad = src.replace("# FITCOUL #\n\tfalse", "# FITCOUL #\n\ttrue")
    assert bad != src
    p = tmp_path / "fm_setup.in"
    p.write_text(bad)
    with pytest.raises(cg.ChimesError, match="FITCOUL"):
        cg.Model(str(p))


def test_column_counts_of_benchmark_workloads(cg, tmp_path):
    import importlib
    synth = importlib.import_module("chimes_lsq-myllfork_gb300.synth")
    expect = {"water-2b": 36, "water-3b": 820, "chno-4b": 51209}
    for name, ncol in expect.items():
        fm = synth.make_workload(name, str(tmp_path / name), nframes=1, labels=False)
        assert cg.Model(fm).ncols == ncol


# ---------------------------------------------------------------- reference test suite
REF_LSQ = os.path.join(REFERENCE, "test_suite-lsq")
needs_ref = pytest.mark.skipif(not os.path.isdir(REF_LSQ), reason="reference test suite not present")


@needs_ref
def test_oracle_matches_nonorth2_golden(oracle, tmp_path):
    """Complete golden A of the reference's triclinic nonorth2 case (8640 x 12)."""
    src = os.path.join(REF_LSQ, "nonorth2")
    shutil.copy(os.path.join(src, "fm_setup.in"), tmp_path)
    shutil.copy(os.path.join(src, "input.xyzf"), tmp_path)
    A, b = oracle.assemble(str(tmp_path / "fm_setup.in"), nthreads=4)
    G = np.loadtxt(os.path.join(src, "correct_output", "A.txt.aa"))
    gb = np.loadtxt(os.path.join(src, "correct_output", "b.txt"))
    assert A.shape == G.shape
    assert np.abs(A - G).max() < 1e-12
    assert np.allclose(b, gb, rtol=1e-15, atol=0)


@needs_ref
@pytest.mark.parametrize("case", ["special3b", "special4b", "test_4atoms", "test_4atoms.2", "fitstrs3b",
                                  "stress-and-ener-2b1"])
def test_headers_match_reference_suite(cg, case):
    d = os.path.join(REF_LSQ, case, "correct_output")
    m = cg.Model(os.path.join(REF_LSQ, case, "fm_setup.in"))
    assert m.params_header() == open(os.path.join(d, "params.header")).read()
    assert m.ff_groups_map() == open(os.path.join(d, "ff_groups.map")).read()


@needs_ref
@pytest.mark.parametrize("case", ["test_4atoms.2", "special4b"])
def test_oracle_matches_reference_suite_tail(oracle, tmp_path, case):
    """Golden A chunks of the reference suite are truncated; compare the last rows."""
    src = os.path.join(REF_LSQ, case)
    for f in os.listdir(src):
        if os.path.isfile(os.path.join(src, f)):
            shutil.copy(os.path.join(src, f), tmp_path)
    gold = os.path.join(src, "correct_output")
    chunks = sorted(f for f in os.listdir(gold) if f.startswith("A.txt"))
    if not chunks:
        pytest.skip("no golden A chunk")
    lines = open(os.path.join(gold, chunks[-1])).read().splitlines()
    rows = [ln for ln in lines[1:] if ln.strip()]   # first line of a chunk may be partial
    G = np.array([[float(v) for v in ln.split()] for ln in rows])
    A, b = oracle.assemble(str(tmp_path / "fm_setup.in"), nthreads=4)
    tail = A[-len(G):]
    assert tail.shape == G.shape
    scale = np.abs(G).max(axis=0) + 1e-300
    assert (np.abs(tail - G) / scale).max() < 1e-10
    gb = np.loadtxt(os.path.join(gold, "b.txt"))
    assert np.allclose(b, gb, rtol=1e-12, atol=1e-12)


PARAMS_CASES = ["fitstrs", "fitstrs3b", "h2o-invr", "nonorth2", "one-file-three-trajs", "special3b", "special4b",
                "stress-and-ener-2b1", "stress-and-ener-2b2", "stress-and-ener-2b3", "stress-and-ener-4b",
                "stress-and-ener-4b2", "test_4atoms", "test_4atoms.2"]


@needs_ref
@pytest.mark.parametrize("case", PARAMS_CASES)
def test_params_txt_matches_reference_suite(cg, case):
    """params.txt from the reference's fitted coefficients (test_suite_params.txt) and
    its "!" solver preamble is byte-identical to the reference's params.txt."""
    d = os.path.join(REF_LSQ, case, "correct_output")
    m = cg.Model(os.path.join(REF_LSQ, case, "fm_setup.in"))
    gold = open(os.path.join(d, "params.txt")).read()
    lines = gold.splitlines(True)
    k = 0
    while k < len(lines) and lines[k].startswith("!"):
        k += 1
    x = np.array([float(ln.split()[1]) for ln in open(os.path.join(d, "test_suite_params.txt")) if ln.strip()])
    assert x.size == m.ncols
    assert m.params_txt(x, "".join(lines[:k])) == gold


def test_params_txt_rejects_wrong_count(cg):
    m = cg.Model(os.path.join(GOLDEN, "water3b", "fm_setup.in"))
    with pytest.raises(cg.ChimesError):
        m.params_txt(np.zeros(m.ncols + 1))
    t = m.params_txt(np.arange(m.ncols, dtype=float))
    assert t.startswith(m.params_header().splitlines()[0]) and t.endswith("ENDFILE\n")


@needs_ref
@pytest.mark.parametrize("case", PARAMS_CASES)
def test_params_txt_reader_matches_reference_coefficients(cg, case):
    """params.txt -> coefficient vector equals the reference's test_suite_params.txt."""
    d = os.path.join(REF_LSQ, case, "correct_output")
    m = cg.Model(os.path.join(REF_LSQ, case, "fm_setup.in"))
    x = np.array([float(ln.split()[1]) for ln in open(os.path.join(d, "test_suite_params.txt")) if ln.strip()])
    assert np.array_equal(m.params_read(open(os.path.join(d, "params.txt")).read()), x)


@needs_ref
def test_lsq_text_files_match_reference_nonorth2(cg, tmp_path):
    """A.txt / b.txt / b-labeled.txt / natoms.txt / dim.txt byte-identical to the
    reference's for its own A values (the golden A.txt read back exactly)."""
    src = os.path.join(REF_LSQ, "nonorth2")
    for f in ("fm_setup.in", "input.xyzf"):
        shutil.copy(os.path.join(src, f), tmp_path)
    m = cg.Model(str(tmp_path / "fm_setup.in"))
    frames = cg.Frames.read(m)
    gold = os.path.join(src, "correct_output")
    A = np.loadtxt(os.path.join(gold, "A.txt.aa"))
    out = tmp_path / "out"
    out.mkdir()
    frames.write_lsq_files(A, out)
    for f in ("A.txt", "b.txt", "b-labeled.txt", "natoms.txt", "dim.txt"):
        ref = os.path.join(gold, "A.txt.aa" if f == "A.txt" else f)
        assert open(out / f).read() == open(ref).read(), f


# ---------------------------------------------------------------- FITCOUL (Ewald charge columns)
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "chimes_lsq")
needs_bin = pytest.mark.skipif(not os.path.isfile(REF_BIN), reason="reference binary not built here")
LSQ2_PARAMS = ["params.ridge.1.0e-03.txt", "params.lassolars.1.0e-04.txt", "params.dlars.1.0e-04.txt",
               "params.dlasso.1.0e-04.txt", "params.svd.1.0e-04.txt"]


@needs_ref
def test_lsq2_fitcoul_header_and_map(cg, tmp_path):
    """The reference's lsq2 case (FITCOUL, charge constraints, 2B10 / 3B6 / 4B2)."""
    src = os.path.join(REF_LSQ, "lsq2")
    m = cg.Model(os.path.join(src, "fm_setup.in"))
    assert m.charge_columns() == (3, 2)
    assert m.ncols == 419
    assert m.params_header() == open(os.path.join(src, "correct_output", "params.header")).read()


@needs_ref
@pytest.mark.parametrize("name", LSQ2_PARAMS)
def test_lsq2_params_txt_round_trip(cg, name):
    """The reference's lsq2 solver outputs (charge products "q_A x q_B" after each
    pair's coefficients): params.txt -> coefficients -> params.txt is byte-identical."""
    src = os.path.join(REF_LSQ, "lsq2")
    m = cg.Model(os.path.join(src, "fm_setup.in"))
    gold = open(os.path.join(src, "correct_output", name)).read()
    head = gold.index("USECOUL:")   # the solver's preamble ("!" lines, blank lines of the DLARS runs)
    pre = gold[:head]
    x = m.params_read(gold)
    assert m.params_txt(x, pre) == gold


@needs_ref
@needs_bin
def test_oracle_matches_reference_binary_lsq2(oracle, cg, tmp_path):
    """The oracle's Ewald restatement against the reference binary on the first two
    frames of lsq2 (real- and k-space charge columns, constraint rows, labels)."""
    src = os.path.join(REF_LSQ, "lsq2")
    shutil.copy(os.path.join(src, "input.xyzf"), tmp_path)
    fm = open(os.path.join(src, "fm_setup.in")).read()
    fm = re.sub(r"(# NFRAMES #[^\n]*\n\s*)33", r"\g<1>2", fm)
    (tmp_path / "fm_setup.in").write_text(fm)
    subprocess.run([REF_BIN, "fm_setup.in"], cwd=tmp_path, check=True, stdout=subprocess.DEVNULL)
    R = np.loadtxt(tmp_path / "A.txt")
    rb = np.loadtxt(tmp_path / "b.txt")
    A, b = oracle.assemble(str(tmp_path / "fm_setup.in"), nthreads=4)
    m = cg.Model(str(tmp_path / "fm_setup.in"))
    Cc, cb = m.constraint_rows()
    assert R.shape[0] == A.shape[0] + Cc.shape[0]
    colmax = np.abs(R).max(axis=0)
    assert np.all(np.abs(A - R[:A.shape[0]]) <= 1e-15 * np.abs(R[:A.shape[0]]) + 1e-15 * colmax[None, :])
    assert np.array_equal(Cc, R[A.shape[0]:]) and np.array_equal(cb, rb[A.shape[0]:])
    assert np.array_equal(b, rb[:A.shape[0]])


@needs_bin
def test_lsq_text_files_match_reference_fitcoul(cg, tmp_path):
    """A.txt (charge columns, constraint rows), b.txt, b-labeled.txt, natoms.txt and
    dim.txt byte-identical to the reference's on the FITCOUL fixture."""
    d = fixture_dir("watercoul")
    for f in ("fm_setup.in", "traj.xyzf"):
        shutil.copy(os.path.join(d, f), tmp_path)
    subprocess.run([REF_BIN, "fm_setup.in"], cwd=tmp_path, check=True, stdout=subprocess.DEVNULL)
    m = cg.Model(str(tmp_path / "fm_setup.in"))
    frames = cg.Frames.read(m)
    A = np.loadtxt(tmp_path / "A.txt")[: frames.nrows]
    out = tmp_path / "out"
    out.mkdir()
    frames.write_lsq_files(A, out)
    for f in ("A.txt", "b.txt", "b-labeled.txt", "natoms.txt", "dim.txt"):
        assert open(out / f).read() == open(tmp_path / f).read(), f


# ---------------------------------------------------------------- TRJFILE MULTI
def test_multifile_labels_carry_the_file_flags(cg, tmp_path):
    """b-labeled.txt of the two-file fixture (flags fa_ / sb_ / eb_ on the second
    file's force / stress / energy rows) byte-identical to the reference's."""
    d = fixture_dir("multifile")
    m = cg.Model(os.path.join(d, "fm_setup.in"))
    fr = cg.Frames.read(m)
    assert fr.nframes == 3
    A = np.zeros((fr.nrows, m.ncols))
    fr.write_lsq_files(A, tmp_path)
    assert open(tmp_path / "b-labeled.txt").read() == open(os.path.join(d, "b-labeled.txt")).read()


@needs_ref
def test_two_traj_files_match_reference_suite(cg, tmp_path):
    """The reference's two-traj-files case (TRJFILE MULTI, 64- and 128-atom files):
    labels, b.txt and b-labeled.txt as its golden output."""
    src = os.path.join(REF_LSQ, "two-traj-files")
    m = cg.Model(os.path.join(src, "fm_setup.in"))
    fr = cg.Frames.read(m)
    gold = os.path.join(src, "correct_output")
    assert np.array_equal(fr.labels(), np.loadtxt(os.path.join(gold, "b.txt")))
    A = np.zeros((fr.nrows, m.ncols))
    fr.write_lsq_files(A, tmp_path)
    for f in ("b.txt", "b-labeled.txt"):
        assert open(tmp_path / f).read() == open(os.path.join(gold, f)).read(), f
    assert m.params_header() == open(os.path.join(gold, "params.header")).read()


def test_rank_schedule_follows_the_reference(cg, tmp_path):
    """Frames of a SKPFRMS run on one rank: every n-th trajectory frame, each keeping
    its own index for the NSTRESS cut-off (skipframes fixture: frames 0, 2, 4 of 5)."""
    d = fixture_dir("skipframes")
    m = cg.Model(os.path.join(d, "fm_setup.in"))
    fr = cg.Frames.read(m)
    assert fr.nframes == 3
    # the same frames through the ranked reader on one rank
    fr1 = cg.Frames.read(m, nprocs=1)
    assert np.array_equal(fr1.labels(), fr.labels())
    # two ranks: rank 0 takes frames i with i % 2 == 0 and (i / 2) % 2 == 0 (0, 4),
    # rank 1 takes i with (i + 1) % 2 == 0 and ((i + 1) / 2) % 2 == 0 (3): b in rank order
    fr2 = cg.Frames.read(m, nprocs=2)
    assert fr2.nframes == 3
    ref = np.load(os.path.join(d, "ref.npz"))["b"]
    rows0 = 72 * 3 + 9 + 3
    assert np.array_equal(fr2.labels()[:rows0], ref[:rows0])


@needs_ref
@pytest.mark.parametrize("case", ["skip_frames", "tatb"])
def test_multi_rank_outputs_match_reference_suite(cg, tmp_path, case):
    """The reference suite's 36-rank runs (run_test_suite.sh NP=36): skip_frames
    (SKPFRMS 1, FITCOUL with charge constraints) and tatb (SPLITFI + SKPFRMS,
    NON_ORTHO cells, stress and energy rows).  b.txt, b-labeled.txt, natoms.txt and
    dim.txt / dim.%04d.txt byte-identical to its golden output, header too."""
    src = os.path.join(REF_LSQ, case)
    gold = os.path.join(src, "correct_output")
    run = tmp_path / "in"
    run.mkdir()
    # the golden output's own copy of the input (tatb's was made with a 4-body order of 2)
    shutil.copy(os.path.join(gold, "fm_setup.in"), run / "fm_setup.in")
    for f in os.listdir(src):
        if f.endswith(".xyzf"):
            shutil.copy(os.path.join(src, f), run / f)
    m = cg.Model(str(run / "fm_setup.in"))
    fr = cg.Frames.read(m, nprocs=36)
    fr.write_lsq_files(None, tmp_path)
    names = ["b.txt", "b-labeled.txt", "natoms.txt"]
    if case == "tatb":
        names += [f"dim.{r:04d}.txt" for r in range(36)]
        assert not os.path.exists(tmp_path / "dim.txt")
    else:
        names.append("dim.txt")
    for f in names:
        g = os.path.join(gold, f)
        if not os.path.exists(g):
            continue
        if case == "tatb" and f == "b.txt":
            # tatb's golden b.txt holds its stress labels as 0 (an older writer; its
            # b-labeled.txt and the current reference binary carry the values): the
            # other rows byte-identical, the stress rows as b-labeled.txt prints them
            lab = open(os.path.join(gold, "b-labeled.txt")).read().splitlines()
            ours = open(tmp_path / f).read().splitlines()
            theirs = open(g).read().splitlines()
            assert len(ours) == len(theirs) == len(lab)
            for o, t, lb in zip(ours, theirs, lab):
                if lb.startswith("s_"):
                    assert f"{float(o):g}" == lb.split()[1], lb
                else:
                    assert o == t
            continue
        assert open(tmp_path / f).read() == open(g).read(), f
    # these goldens predate the EXCLD1B / EXCLD2B header lines the current reference prints
    def strip(t):
        return "".join(ln for ln in t.splitlines(True) if not ln.startswith(("EXCLD1B:", "EXCLD2B:")))
    assert strip(m.params_header()) == strip(open(os.path.join(gold, "params.header")).read())
    assert m.ff_groups_map() == open(os.path.join(gold, "ff_groups.map")).read()


def test_split_files_hold_each_ranks_rows(cg, tmp_path):
    """SPLITFI: A.%04d.txt per rank with data and dim.%04d.txt "columns first last
    total"; their concatenation is the A.txt of the same run without SPLITFI."""
    d = fixture_dir("skipframes")
    src = open(os.path.join(d, "fm_setup.in")).read()
    key = "# SKPFRMS #\n\t2\n"
    assert key in src
    split_dir, whole_dir = tmp_path / "split", tmp_path / "whole"
    for out, extra in ((split_dir, "# SPLITFI #\n\ttrue\n"), (whole_dir, "")):
        out.mkdir()
        open(out / "fm_setup.in", "w").write(src.replace(key, key + extra))
        shutil.copy(os.path.join(d, "traj.xyzf"), out / "traj.xyzf")
    ms = cg.Model(str(split_dir / "fm_setup.in"))
    mw = cg.Model(str(whole_dir / "fm_setup.in"))
    fs, fw = cg.Frames.read(ms, nprocs=2), cg.Frames.read(mw, nprocs=2)
    assert fs.nframes == fw.nframes == 3   # rank 0: frames 0, 4; rank 1: frame 3
    A = np.random.default_rng(3).standard_normal((fs.nrows, ms.ncols))
    fs.write_lsq_files(A, split_dir)
    fw.write_lsq_files(A, whole_dir)
    assert not (split_dir / "A.txt").exists() and not (split_dir / "dim.txt").exists()
    joined = open(split_dir / "A.0000.txt").read() + open(split_dir / "A.0001.txt").read()
    assert joined == open(whole_dir / "A.txt").read()
    r0 = 2 * 72 * 3 + 9 + 3 + 3          # frame 0 (stress + energy) and frame 4 (energy)
    total = fs.nrows
    assert open(split_dir / "dim.0000.txt").read() == f"{ms.ncols} 0 {r0 - 1} {total}\n"
    assert open(split_dir / "dim.0001.txt").read() == f"{ms.ncols} {r0} {total - 1} {total}\n"
    assert open(whole_dir / "dim.txt").read() == f"{ms.ncols} {total}\n"
    for f in ("b.txt", "b-labeled.txt", "natoms.txt"):
        assert open(split_dir / f).read() == open(whole_dir / f).read()


def test_hierarchical_params_txt_matches_reference_script(cg):
    """HIERARC fixture (O-H 2-body block and the H energy offset excluded): params.txt
    from the reference solver script's coefficients is byte-identical to the one the
    script printed (zeros for the excluded pair and offset), and reads back to them."""
    d = fixture_dir("hierarc")
    m = cg.Model(os.path.join(d, "fm_setup.in"))
    cols = m.columns()
    ref = np.load(os.path.join(d, "ref.npz"))
    assert m.ncols == ref["A"].shape[1] == cols["n2b"] + cols["n3b"] + cols["n4b"] + cols["nener"]
    assert cols["n2b"] == 2 * 8 and cols["nener"] == 1
    gold = open(os.path.join(d, "params.txt")).read()
    lines = gold.splitlines(True)
    k = 0
    while k < len(lines) and lines[k].startswith("!"):
        k += 1
    x = np.array([float(ln.split()[1]) for ln in open(os.path.join(d, "test_suite_params.txt")) if ln.strip()])
    assert x.size == m.ncols
    assert m.params_txt(x, "".join(lines[:k])) == gold
    assert np.array_equal(m.params_read(gold), x)


# ---------------------------------------------------------------- MD output files
TRAJ = os.path.join(GOLDEN, "md_ch4b", "traj")


def test_md_restart_reader_and_output_xyz_match_reference(cg, tmp_path):
    """The reference's restart.xyzv after a 6-step NVE run read back; written as
    output.xyz it is byte-identical to the run's own output.xyz (same state)."""
    m = cg.Model(os.path.join(GOLDEN, "md_ch4b", "fm_setup.in"))
    r = m.md_read_restart(os.path.join(TRAJ, "restart.xyzv"), 40)
    assert r["step"] == 6 and r["cell"][0] == r["cell"][4] == r["cell"][8] > 7.0
    assert r["constraint"][26] == 117.0   # N_DOF = 3 * 40 - 3
    m.md_write_xyzv(tmp_path / "output.xyz", r["types"], r["xyz"], r["v"], r["cell"])
    assert open(tmp_path / "output.xyz").read() == open(os.path.join(TRAJ, "output.xyz")).read()
    with pytest.raises(cg.ChimesError):
        m.md_read_restart(os.path.join(TRAJ, "restart.xyzv"), 41)


def test_md_generated_velocities_match_reference(cg):
    """VELINIT GEN (RNDSEED 4321, 300 K) with the centre-of-mass correction: the
    velocities as the reference chimes_md printed them (velocout.txt, %13.6e) for the
    40-atom fixture."""
    d = np.load(os.path.join(GOLDEN, "md_ch4b", "md_ref.npz"))
    masses = np.asarray(d["masses"])[np.asarray(d["types"])]
    v = cg.md_velocities(masses, 300.0, 4321)
    lines = open(os.path.join(TRAJ, "velgen_velocout.txt")).read().splitlines()[:120]
    assert ["%13.6e" % x for x in v.reshape(-1)] == lines
    p = (masses[:, None] * v).sum(0)
    assert np.abs(p).max() <= 1e-12 * np.abs(masses[:, None] * v).sum()
    # read velocities keep their values apart from the centre-of-mass shift
    w = cg.md_velocities(masses, v=v + 0.25)
    assert np.allclose(w, v, rtol=0, atol=1e-12)
