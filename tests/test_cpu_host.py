"""CPU-only checks: the C ABI library loads and exports its header, the host
topology reproduces the reference's params.header / ff_groups.map, the labels
(b) and row layout match, and the CPU oracle reproduces the reference's A."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from conftest import FIXTURES, GOLDEN, REFERENCE, ROOT, fixture_dir

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
    assert fr.nrows == ref["A"].shape[0]
    assert m.ncols == ref["A"].shape[1]
    assert np.array_equal(fr.labels(), ref["b"])


@pytest.mark.parametrize("name", FIXTURES)
def test_oracle_matches_reference_fixture(oracle, name):
    d = fixture_dir(name)
    A, b = oracle.assemble(os.path.join(d, "fm_setup.in"), nthreads=4)
    ref = np.load(os.path.join(d, "ref.npz"))
    R = ref["A"]
    colmax = np.abs(R).max(axis=0)
    assert np.all(np.abs(A - R) <= 4e-16 * np.abs(R) + 1e-15 * colmax[None, :])
    assert np.array_equal(b, ref["b"])


def test_model_errors_are_reported(cg, tmp_path):
    with pytest.raises(cg.ChimesError) as e:
        cg.Model(str(tmp_path / "missing.in"))
    assert e.value.code == 2
    src = open(os.path.join(fixture_dir("water2b"), "fm_setup.in")).read()
    bad = src.replace("# FITCOUL #\n\tfalse", "# FITCOUL #\n\ttrue")
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
