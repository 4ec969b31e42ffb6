"""ctypes access to the CPU oracle (liboracle.so) -- test infrastructure only.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
checker / baseline; the chimes_gb300 library never calls it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_BIN = os.path.join(HERE, "_ref", "chimes_lsq")

_lib = None


def build():
    """Compile liboracle.so (and, when the reference sources exist, oracle/_ref)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    ref_src = os.environ.get("CHIMES_REF_DIR", "/root/reference")
    if os.path.isdir(os.path.join(ref_src, "src")) and not os.path.exists(REF_BIN):
        subprocess.run([os.path.join(HERE, "build_ref.sh")], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        L.oracle_sizes.restype = ctypes.c_int
        L.oracle_sizes.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int,
                                   ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int)]
        L.oracle_assemble.restype = ctypes.c_int
        L.oracle_assemble.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]
        L.oracle_md_force.restype = ctypes.c_int
        L.oracle_md_force.argtypes = [ctypes.c_char_p, ctypes.c_int] + [ctypes.c_void_p] * 5 + [
            ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_void_p,
            ctypes.c_void_p]
        L.oracle_last_error.restype = ctypes.c_char_p
        _lib = L
    return _lib


def _enc(p):
    return None if p is None else os.fspath(p).encode()


def sizes(fm_setup, xyzf=None, nframes=0):
    r, c = ctypes.c_int64(), ctypes.c_int()
    rc = lib().oracle_sizes(_enc(fm_setup), _enc(xyzf), int(nframes), ctypes.byref(r), ctypes.byref(c))
    if rc:
        raise RuntimeError(lib().oracle_last_error().decode())
    return r.value, c.value


def assemble(fm_setup, xyzf=None, nframes=0, first=0, count=0, nthreads=1):
    """(A, b) of frames [first, first+count) (count 0: to the end), float64."""
    if count <= 0:
        # rows of the requested frames only
        nall, ncols = sizes(fm_setup, xyzf, nframes)
        if first == 0:
            nrows = nall
        else:
            nrows = nall - sizes(fm_setup, xyzf, first)[0]
    else:
        nrows = sizes(fm_setup, xyzf, first + count)[0] - (sizes(fm_setup, xyzf, first)[0] if first else 0)
        ncols = sizes(fm_setup, xyzf, 1)[1]
    A = np.zeros((nrows, ncols), dtype=np.float64)
    b = np.zeros(nrows, dtype=np.float64)
    rc = lib().oracle_assemble(_enc(fm_setup), _enc(xyzf), int(nframes), int(first), int(count), int(nthreads),
                               ctypes.c_void_p(A.ctypes.data), ncols, ctypes.c_void_p(b.ctypes.data))
    if rc:
        raise RuntimeError(lib().oracle_last_error().decode())
    return A, b


def md_force(fm_setup, natoms, types, xyz, cell, x, offsets=False, pen_dist=0.01, pen_scale=1.0e4, nthreads=1):
    """MD forces [sum natoms, 3] and scalars [nframes, 11] of independent
    configurations (ZCalc restated; see chimes_oracle.cpp)."""
    natoms = np.ascontiguousarray(natoms, dtype=np.int32)
    types = np.ascontiguousarray(types, dtype=np.int32)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    cell = np.ascontiguousarray(cell, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    F = np.zeros((int(natoms.sum()), 3), dtype=np.float64)
    S = np.zeros((len(natoms), 11), dtype=np.float64)
    p = lambda a: ctypes.c_void_p(a.ctypes.data)
    rc = lib().oracle_md_force(_enc(fm_setup), len(natoms), p(natoms), p(types), p(xyz), p(cell), p(x), x.size,
                               1 if offsets else 0, float(pen_dist), float(pen_scale), int(nthreads), p(F), p(S))
    if rc:
        raise RuntimeError(lib().oracle_last_error().decode())
    return F, S


def run_reference(workdir):
    """Run the compiled reference chimes_lsq in workdir; returns (A, b) from A.txt / b.txt."""
    if not os.path.exists(REF_BIN):
        raise FileNotFoundError(REF_BIN)
    subprocess.run([REF_BIN, "fm_setup.in"], cwd=workdir, check=True, stdout=subprocess.DEVNULL,
                   stderr=subprocess.DEVNULL)
    A = np.loadtxt(os.path.join(workdir, "A.txt"), ndmin=2)
    b = np.loadtxt(os.path.join(workdir, "b.txt"))
    return A, b
