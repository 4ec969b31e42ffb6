"""Build the in-tree CUDA/C++ library (libchimes_gb300.so) for sm_103a.

Compiles every translation unit in parallel (nvcc for .cu, g++ for host .cpp)
and links one shared object under ``_lib/``.  Host code is compiled with
``-ffp-contract=off`` because the box set-up arithmetic has to round exactly like
the reference's.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libchimes_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CU_SOURCES = ["geom.cu", "assemble.cu", "ewald.cu", "session.cu", "gram.cu", "dense64.cu", "solve.cu", "md.cu", "md_host.cu", "lars.cu"]
CPP_SOURCES = ["model.cpp", "capi.cpp", "textio.cpp", "mdio.cpp"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build chimes_gb300")
    return cand


def _cuda_include():
    root = os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))
    return os.path.join(root, "include")


def _run(cmd):
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + p.stdout)
    return p.stdout


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    """Compile and link the library; returns its path."""
    os.makedirs(OUT, exist_ok=True)
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "chimes_gb300.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        if not os.path.exists(s):
            continue
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append([nvcc, ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xcompiler", "-ffp-contract=off", "-c", s, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I" + _cuda_include(),
                         "-c", s, "-o", o])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out.strip():
                    print(out)
    if force or jobs or not os.path.exists(LIB):
        _run([nvcc, ARCH, "-shared", "-o", LIB] + objs + ["-lcudart"])
    build_native_checks(force)
    return LIB


def build_native_checks(force=False):
    """The test programs that call the library through include/ alone: a C caller of
    chimes_gb300.h and a C++ caller of the ZCalc / ZCalc_Deriv drop-ins
    (tests/native/*), linked against the in-tree library."""
    root = os.path.dirname(HERE)
    inc = os.path.join(root, "include")
    src = os.path.join(root, "tests", "native")
    for name, comp, extra in (("capi_check.c", "gcc", ["-std=c11"]), ("zcalc_check.cpp", "g++", ["-std=c++17"])):
        s = os.path.join(src, name)
        if not os.path.exists(s):
            continue
        out = os.path.join(OUT, os.path.splitext(name)[0])
        deps = [s, LIB] + [os.path.join(inc, f) for f in os.listdir(inc)]
        if force or _stale(out, deps):
            _run([comp, "-O2"] + extra + ["-I" + inc, s, "-o", out, "-L" + OUT, "-lchimes_gb300",
                                          "-Wl,-rpath," + OUT])


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
