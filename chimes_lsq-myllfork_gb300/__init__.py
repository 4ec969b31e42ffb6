"""GB300 design-matrix path of ChIMES-lsq: Python mirror of the C ABI.

This package wraps ``libchimes_gb300.so`` (built in-tree by ``build.py``) with
ctypes.  The names follow the reference's operator surface:

* :class:`Model` parses ``fm_setup.in`` (INPUT::PARSE_INFILE_LSQ, src/input.C:172-225)
  and exposes the ``params.header`` / ``ff_groups.map`` text
  (print_param_header / print_map_file, src/chimes_lsq.C:562-716);
* :class:`Frames` reads ``.xyzf`` trajectories (FRAME::READ_XYZF,
  src/ClassDefs.C:2411-2683) or takes arrays;
* :class:`Session` assembles the A matrix on one GPU (the frame loop of
  src/chimes_lsq.C:292-328 calling ZCalc_Deriv, src/functions.C:755-804).

Errors from the library raise :class:`ChimesError` with the library's message.
There is no CPU fallback: without the compiled library every call fails.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libchimes_gb300.so")

CG_FP64 = 0
CG_FP32 = 1
CG_NVT_MTK, CG_NVT_BEREND, CG_NVT_SCALE = 1, 2, 6
CG_NPT_BEREND, CG_NPT_BEREND_ANISO, CG_NPT_MTK = 3, 4, 5
CG_TRAJ_GEN, CG_TRAJ_XYZ, CG_TRAJ_LAMMPSTRJ = 1, 2, 3
MD_ENERGY_OFFSETS = 1
MD_NSCALAR = 11   # energy, PRESSURE_XYZ/3V, virial tensor/V (3x3 row-major)

_lib = None


class ChimesError(RuntimeError):
    """A non-zero status from the C ABI."""

    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def build(verbose=False):
    """Compile the CUDA/C++ library in-tree (sm_103a)."""
    from importlib import util
    spec = util.spec_from_file_location("_chimes_gb300_build", os.path.join(_HERE, "build.py"))
    mod = util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(verbose=verbose)


def lib():
    """Load the compiled library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ChimesError(2, f"{LIB_PATH} is missing: run build() first (no CPU fallback exists)")
    L = ctypes.CDLL(LIB_PATH)
    vp, ip, i64p, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int64), ctypes.c_void_p
    pp = ctypes.POINTER(ctypes.c_void_p)
    sig = {
        "cg_model_load": (ctypes.c_int, [ctypes.c_char_p, pp]),
        "cg_model_free": (None, [vp]),
        "cg_model_columns": (ctypes.c_int, [vp, ip, ip, ip, ip, ip]),
        "cg_model_charge_columns": (ctypes.c_int, [vp, ip, ip]),
        "cg_model_constraint_rows": (ctypes.c_int, [vp, dp, ctypes.c_int64, dp]),
        "cg_model_sizes": (ctypes.c_int, [vp, ip, ip]),
        "cg_model_row_layout": (ctypes.c_int, [vp, ip, ip]),
        "cg_model_header_text": (ctypes.c_int, [vp, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
        "cg_model_map_text": (ctypes.c_int, [vp, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)]),
        "cg_model_params_text": (ctypes.c_int, [vp, dp, ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t,
                                                ctypes.POINTER(ctypes.c_size_t)]),
        "cg_frames_read": (ctypes.c_int, [vp, ctypes.c_char_p, ctypes.c_int, pp]),
        "cg_frames_read_ranks": (ctypes.c_int, [vp, ctypes.c_int, pp]),
        "cg_frames_create": (ctypes.c_int, [vp, ctypes.c_int, vp, vp, vp, vp, vp, vp, vp, ctypes.c_int, pp]),
        "cg_frames_free": (None, [vp]),
        "cg_frames_rows": (ctypes.c_int, [vp, i64p, i64p]),
        "cg_frames_labels": (ctypes.c_int, [vp, dp]),
        "cg_frames_count": (ctypes.c_int, [vp, ip]),
        "cg_frames_independent": (ctypes.c_int, [vp]),
        "cg_frames_slice": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_int, pp]),
        "cg_model_params_read": (ctypes.c_int, [vp, ctypes.c_char_p, dp, ctypes.c_int]),
        "cg_write_lsq_files": (ctypes.c_int, [vp, vp, dp, ctypes.c_int64, ctypes.c_char_p]),
        "cg_session_create": (ctypes.c_int, [vp, ctypes.c_int, pp]),
        "cg_session_free": (None, [vp]),
        "cg_session_stream": (ctypes.c_void_p, [vp]),
        "cg_assemble": (ctypes.c_int, [vp, vp, ctypes.c_int, vp, ctypes.c_int64]),
        "cg_frames_upload": (ctypes.c_int, [vp, vp, pp]),
        "cg_dframes_free": (None, [vp]),
        "cg_assemble_device": (ctypes.c_int, [vp, vp, ctypes.c_int, vp, ctypes.c_int64]),
        "cg_session_last_counts": (ctypes.c_int, [vp, i64p, i64p, i64p, i64p, i64p]),
        "cg_assemble_device_noalloc": (ctypes.c_int, [vp, vp, ctypes.c_int, vp, ctypes.c_int64]),
        "cg_session_last_launches": (ctypes.c_int, [vp, i64p]),
        "cg_session_profile": (ctypes.c_int, [vp, ctypes.c_int]),
        "cg_session_stage_times": (ctypes.c_int, [vp, vp, vp]),
        "cg_stage_name": (ctypes.c_char_p, [ctypes.c_int]),
        "cg_last_error": (ctypes.c_char_p, []),
        "cg_gram": (ctypes.c_int, [vp, ctypes.c_int, vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int, vp, ctypes.c_int,
                                   vp, vp]),
        "cg_gram_weighted": (ctypes.c_int, [vp, ctypes.c_int, vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int, vp, vp,
                                            ctypes.c_int, vp, vp]),
        "cg_gram_finish": (ctypes.c_int, [vp, vp, ctypes.c_int]),
        "cg_solve": (ctypes.c_int, [vp, vp, vp, ctypes.c_int, ctypes.c_double, vp, ctypes.c_int64, ctypes.c_int64, vp,
                                    ctypes.c_int, vp, vp]),
        "cg_assemble_stream": (ctypes.c_int, [vp, vp, ctypes.c_int, ctypes.c_int, vp, vp]),
        "cg_solve_streamed": (ctypes.c_int, [vp, vp, vp, ctypes.c_int, ctypes.c_double, ctypes.c_int, vp, vp, vp, vp,
                                             ctypes.c_int64, vp, vp, ctypes.c_int, ctypes.c_double, vp, vp]),
        "cg_cholesky": (ctypes.c_int, [vp, vp, ctypes.c_int, ctypes.c_double, vp, ctypes.POINTER(ctypes.c_double)]),
        "cg_cholesky_solve": (ctypes.c_int, [vp, vp, ctypes.c_int, vp, vp]),
        "cg_refine_streamed": (ctypes.c_int, [vp, vp, ctypes.c_int, ctypes.c_double, ctypes.c_int, vp, vp, vp, vp,
                                              ctypes.c_int64, vp, vp, ctypes.c_int, ctypes.c_double, vp, vp]),
        "cg_predict_streamed": (ctypes.c_int, [vp, ctypes.c_int, vp, vp, vp]),
        "cg_fp64_fma_rate": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_double)]),
        "cg_md_server_start": (ctypes.c_int, [vp, vp, ctypes.c_double, ctypes.c_double, ctypes.c_int64, ctypes.c_int,
                                              ctypes.POINTER(ctypes.c_void_p)]),
        "cg_md_server_submit": (ctypes.c_int, [vp, vp, ctypes.POINTER(ctypes.c_int64)]),
        "cg_md_server_poll": (ctypes.c_int, [vp, ctypes.c_int64, ctypes.c_int, vp, vp]),
        "cg_md_server_stop": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_int64)]),
        "cg_md_serve_memory": (ctypes.c_int, [vp, ctypes.c_int64, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                              ctypes.POINTER(ctypes.c_double)]),
        "cg_batch_fit_create": (ctypes.c_int, [vp, ctypes.c_int, vp, vp, ctypes.c_int, vp, ctypes.c_int64, vp, vp, pp]),
        "cg_batch_fit_launch": (ctypes.c_int, [vp, vp]),
        "cg_batch_fit_nodes": (ctypes.c_int, [vp, i64p]),
        "cg_batch_fit_free": (None, [vp]),
        "cg_session_tune": (ctypes.c_int, [vp, ctypes.c_char_p, ctypes.c_int]),
        "cg_lars": (ctypes.c_int, [vp, vp, vp, ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_int, vp, vp]),
        "cg_dlars": (ctypes.c_int, [vp, vp, vp, ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_int, vp, ctypes.c_double, ctypes.c_int, vp, vp]),
        "cg_dlars_ex": (ctypes.c_int, [vp, vp, vp, ctypes.c_int, ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_int, vp, ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                       ctypes.c_char_p, ctypes.c_char_p, vp, vp]),
        "cg_md_setup": (ctypes.c_int, [vp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                       ctypes.c_double]),
        "cg_md_force": (ctypes.c_int, [vp, vp, dp, dp]),
        "cg_md_force_device": (ctypes.c_int, [vp, vp, vp, vp]),
        "cg_md_nve": (ctypes.c_int, [vp, vp, dp, ctypes.c_double, ctypes.c_int, vp, vp, vp, vp]),
        "cg_frames_subtract_coulomb": (ctypes.c_int, [vp, vp]),
        "cg_md_nvt": (ctypes.c_int, [vp, vp, dp, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_double, vp, vp, vp, vp, vp]),
        "cg_md_npt": (ctypes.c_int, [vp, vp, dp, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_double, ctypes.c_double, vp, vp, vp, vp, vp, vp]),
        "cg_md_write_traj": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int, vp, vp, vp,
                                            vp]),
        "cg_md_write_xyzv": (ctypes.c_int, [vp, ctypes.c_char_p, ctypes.c_int, vp, vp, vp, vp, ctypes.c_int]),
        "cg_md_write_restart": (ctypes.c_int, [vp, ctypes.c_int, ctypes.c_char_p, ctypes.c_int, vp, vp, vp, vp, vp,
                                               ctypes.c_int, ctypes.c_double, vp, ctypes.c_int]),
        "cg_md_read_restart": (ctypes.c_int, [vp, ctypes.c_char_p, ctypes.c_int, vp, vp, vp, vp, vp,
                                              ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double), vp, vp]),
        "cg_md_resume": (ctypes.c_int, [vp, ctypes.c_int, vp]),
        "cg_md_numerical": (ctypes.c_int, [vp, vp, ctypes.c_int, vp]),
        "cg_md_velocities": (ctypes.c_int, [ctypes.c_int, vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, vp]),
        "cg_dframes_positions": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_void_p), i64p]),
        "cg_dframes_read_positions": (ctypes.c_int, [vp, dp]),
        "cg_md_last_counts": (ctypes.c_int, [vp, i64p, i64p, i64p, i64p]),
        "cg_md_serve": (ctypes.c_int, [vp, ctypes.c_int, vp, dp, ctypes.c_double, ctypes.c_double, ctypes.c_int64,
                                       ctypes.c_int, vp, vp, i64p]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


ROWS_SINK = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
                             ctypes.c_int64)


class MdRequest(ctypes.Structure):
    _fields_ = [("natoms", ctypes.c_int), ("nsteps", ctypes.c_int), ("arrival", ctypes.c_double),
                ("types", ctypes.c_void_p), ("xyz", ctypes.c_void_p), ("cell", ctypes.c_void_p),
                ("v", ctypes.c_void_p), ("xyz_out", ctypes.c_void_p)]


class MdResult(ctypes.Structure):
    _fields_ = [("admitted", ctypes.c_double), ("finished", ctypes.c_double), ("step_ms_sum", ctypes.c_double),
                ("step_ms_max", ctypes.c_double), ("reserved_bytes", ctypes.c_double)]


def _check(rc):
    if rc != 0:
        raise ChimesError(rc, lib().cg_last_error().decode(errors="replace"))


def _ptr(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def md_velocities(mass, temperature=0.0, seed=12357, v=None):
    """Initial velocities ([natoms, 3], internal units): drawn as `# VELINIT # GEN` does
    when v is None, else v as read; the centre-of-mass velocity removed (cg_md_velocities)."""
    m = np.ascontiguousarray(mass, dtype=np.float64)
    out = np.zeros((len(m), 3)) if v is None else np.array(v, dtype=np.float64).reshape(len(m), 3)
    _check(lib().cg_md_velocities(len(m), _ptr(m), 1 if v is None else 0, int(seed), float(temperature), _ptr(out)))
    return out


class Model:
    """Parsed fm_setup.in with its pair / cluster topology."""

    def __init__(self, fm_setup_path):
        h = ctypes.c_void_p()
        _check(lib().cg_model_load(os.fspath(fm_setup_path).encode(), ctypes.byref(h)))
        self._h = h
        self.path = os.fspath(fm_setup_path)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.cg_model_free(self._h)
            self._h = None

    def columns(self):
        """dict with n2b, n3b, n4b, nener, ntotal (A columns)."""
        v = [ctypes.c_int() for _ in range(5)]
        _check(lib().cg_model_columns(self._h, *[ctypes.byref(x) for x in v]))
        return dict(zip(["n2b", "n3b", "n4b", "nener", "ntotal"], [x.value for x in v]))

    @property
    def ncols(self):
        return self.columns()["ntotal"]

    def charge_columns(self):
        """(ncoul, nconstraints): FITCOUL charge columns and charge-constraint rows."""
        a, b = ctypes.c_int(), ctypes.c_int()
        _check(lib().cg_model_charge_columns(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def constraint_rows(self):
        """(A rows, b) of the charge constraints that follow the last frame of a fit."""
        _, n = self.charge_columns()
        A = np.zeros((n, self.ncols), dtype=np.float64)
        b = np.zeros(n, dtype=np.float64)
        if n:
            _check(lib().cg_model_constraint_rows(self._h, _ptr(A), A.shape[1], _ptr(b)))
        return A, b

    def sizes(self):
        nf, nt = ctypes.c_int(), ctypes.c_int()
        _check(lib().cg_model_sizes(self._h, ctypes.byref(nf), ctypes.byref(nt)))
        return nf.value, nt.value

    def _text(self, fn):
        need = ctypes.c_size_t()
        _check(fn(self._h, None, 0, ctypes.byref(need)))
        buf = ctypes.create_string_buffer(need.value + 1)
        _check(fn(self._h, buf, need.value + 1, ctypes.byref(need)))
        return buf.raw[: need.value].decode()

    def params_header(self):
        return self._text(lib().cg_model_header_text)

    def ff_groups_map(self):
        return self._text(lib().cg_model_map_text)

    def md_write_traj(self, fmt, path, frame_index, step, dt_fs, temperature, types, xyz, v, cell, wrap=False):
        """One trajectory frame (cg_md_write_traj; fmt CG_TRAJ_GEN / _XYZ / _LAMMPSTRJ)."""
        t = np.ascontiguousarray(types, dtype=np.int32)
        x = np.ascontiguousarray(xyz, dtype=np.float64)
        vv = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
        c = np.ascontiguousarray(cell, dtype=np.float64).reshape(9)
        _check(lib().cg_md_write_traj(self._h, int(fmt), os.fspath(path).encode(), int(frame_index), int(step),
                                      float(dt_fs), float(temperature), int(bool(wrap)), len(t), _ptr(t), _ptr(x),
                                      _ptr(vv), _ptr(c)))

    def md_write_xyzv(self, path, types, xyz, v, cell, wrap=False):
        """output.xyz of a run (cg_md_write_xyzv)."""
        t = np.ascontiguousarray(types, dtype=np.int32)
        x = np.ascontiguousarray(xyz, dtype=np.float64)
        vv = np.ascontiguousarray(v, dtype=np.float64)
        c = np.ascontiguousarray(cell, dtype=np.float64).reshape(9)
        _check(lib().cg_md_write_xyzv(self._h, os.fspath(path).encode(), len(t), _ptr(t), _ptr(x), _ptr(vv), _ptr(c),
                                      int(bool(wrap))))

    def md_read_restart(self, path, natoms):
        """restart.xyzv -> dict(types, xyz, v, acc, cell, step, padding, constraint[29], avg[7])."""
        n = int(natoms)
        t = np.zeros(n, dtype=np.int32)
        x, v, a = (np.zeros((n, 3)) for _ in range(3))
        c, c29, avg = np.zeros(9), np.zeros(29), np.zeros(7)
        step, pad = ctypes.c_int(), ctypes.c_double()
        _check(lib().cg_md_read_restart(self._h, os.fspath(path).encode(), n, _ptr(t), _ptr(x), _ptr(v), _ptr(a),
                                        _ptr(c), ctypes.byref(step), ctypes.byref(pad), _ptr(c29), _ptr(avg)))
        return dict(types=t, xyz=x, v=v, acc=a, cell=c, step=step.value, padding=pad.value, constraint=c29, avg=avg)

    def params_read(self, text):
        """Coefficient vector of a params.txt text written for this model."""
        x = np.zeros(self.ncols, dtype=np.float64)
        _check(lib().cg_model_params_read(self._h, text.encode(), _ptr(x), x.size))
        return x

    def params_txt(self, x, preamble=""):
        """params.txt text for the fitted coefficients x (one per A column)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        pre = preamble.encode()
        fn = lib().cg_model_params_text
        need = ctypes.c_size_t()
        _check(fn(self._h, _ptr(x), x.size, pre, None, 0, ctypes.byref(need)))
        buf = ctypes.create_string_buffer(need.value + 1)
        _check(fn(self._h, _ptr(x), x.size, pre, buf, need.value + 1, ctypes.byref(need)))
        return buf.raw[: need.value].decode()


class Frames:
    """A batch of frames (one A-matrix row block each)."""

    def __init__(self, handle, model):
        self._h = handle
        self.model = model

    @classmethod
    def read(cls, model, xyzf_path=None, nframes=0, nprocs=None):
        """The model's trajectory (or nframes of xyzf_path).  nprocs: the frames and
        output order of `chimes_lsq` run on that many ranks (SKPFRMS, SPLITFI)."""
        h = ctypes.c_void_p()
        if nprocs is not None:
            if xyzf_path is not None or nframes:
                raise ValueError("nprocs reads the model's own trajectory")
            _check(lib().cg_frames_read_ranks(model._h, int(nprocs), ctypes.byref(h)))
            return cls(h, model)
        p = None if xyzf_path is None else os.fspath(xyzf_path).encode()
        _check(lib().cg_frames_read(model._h, p, int(nframes), ctypes.byref(h)))
        return cls(h, model)

    @classmethod
    def from_arrays(cls, model, natoms, types, xyz, cell, forces=None, stress=None, energy=None, first_index=0):
        """natoms[F]; types[sum N] (TYPEIDX order); xyz[sum N,3] (A); cell[F,9]
        (ax ay az bx by bz cx cy cz); forces[sum N,3] (Hartree/Bohr); stress[F,6]
        (xx yy zz xy xz yz, GPa); energy[F]."""
        natoms = np.ascontiguousarray(natoms, dtype=np.int32)
        types = np.ascontiguousarray(types, dtype=np.int32)
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        cell = np.ascontiguousarray(cell, dtype=np.float64)
        forces = None if forces is None else np.ascontiguousarray(forces, dtype=np.float64)
        stress = None if stress is None else np.ascontiguousarray(stress, dtype=np.float64)
        energy = None if energy is None else np.ascontiguousarray(energy, dtype=np.float64)
        h = ctypes.c_void_p()
        _check(lib().cg_frames_create(model._h, len(natoms), _ptr(natoms), _ptr(types), _ptr(xyz), _ptr(forces),
                                      _ptr(cell), _ptr(stress), _ptr(energy), int(first_index), ctypes.byref(h)))
        return cls(h, model)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.cg_frames_free(self._h)
            self._h = None

    def slice(self, first, count):
        """Frames [first, first + count) as a new batch."""
        h = ctypes.c_void_p()
        _check(lib().cg_frames_slice(self._h, int(first), int(count), ctypes.byref(h)))
        return Frames(h, self.model)

    def subtract_coulomb(self, session):
        """Fixed charges: subtract the Ewald forces from the force labels (in place)."""
        _check(lib().cg_frames_subtract_coulomb(session._h, self._h))
        return self

    def write_lsq_files(self, A, directory):
        """A.txt / b.txt / b-labeled.txt / natoms.txt / dim.txt for these frames (A: host
        FP64; None writes all but the A files).  SPLITFI models: A.%04d.txt / dim.%04d.txt."""
        lda = 0
        if A is not None:
            A = np.ascontiguousarray(A, dtype=np.float64)
            lda = A.shape[1]
        _check(lib().cg_write_lsq_files(self.model._h, self._h, _ptr(A), lda, os.fspath(directory).encode()))

    def independent(self):
        """Each frame decides the small-cell convention alone (MD systems)."""
        _check(lib().cg_frames_independent(self._h))
        return self

    def rows(self):
        r, a = ctypes.c_int64(), ctypes.c_int64()
        _check(lib().cg_frames_rows(self._h, ctypes.byref(r), ctypes.byref(a)))
        return r.value, a.value

    @property
    def nrows(self):
        return self.rows()[0]

    @property
    def natoms_total(self):
        return self.rows()[1]

    @property
    def nframes(self):
        n = ctypes.c_int()
        _check(lib().cg_frames_count(self._h, ctypes.byref(n)))
        return n.value

    def labels(self):
        b = np.empty(self.nrows, dtype=np.float64)
        _check(lib().cg_frames_labels(self._h, _ptr(b)))
        return b


class DeviceFrames:
    """Frames resident on the GPU of a session."""

    def __init__(self, handle, nrows):
        self._h = handle
        self.nrows = nrows

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.cg_dframes_free(self._h)
            self._h = None

    def read_positions(self):
        """Current positions (host copy, [natoms, 3])."""
        _, n = self.positions_ptr()
        x = np.empty((n, 3), dtype=np.float64)
        _check(lib().cg_dframes_read_positions(self._h, _ptr(x)))
        return x

    def positions_ptr(self):
        """(device pointer to the 3*natoms positions, natoms)."""
        p, n = ctypes.c_void_p(), ctypes.c_int64()
        _check(lib().cg_dframes_positions(self._h, ctypes.byref(p), ctypes.byref(n)))
        return p.value, n.value


class BatchFit:
    """A batched fit captured as one CUDA graph (cg_batch_fit_*)."""

    def __init__(self, handle, session, keep):
        self._h = handle
        self.session = session
        self._keep = keep

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.cg_batch_fit_free(self._h)
            self._h = None

    def launch(self):
        _check(lib().cg_batch_fit_launch(self.session._h, self._h))

    @property
    def nodes(self):
        v = ctypes.c_int64()
        _check(lib().cg_batch_fit_nodes(self._h, ctypes.byref(v)))
        return v.value


CG_PENDING = 5


class MdServer:
    """cg_md_server_*: a library thread runs the serving loop; submit() queues a
    request (its arrays are copied), poll() returns None while it waits or runs, else
    (final xyz [n,3], result record)."""

    _RESULT = [("admitted", "f8"), ("finished", "f8"), ("step_ms_sum", "f8"), ("step_ms_max", "f8"),
               ("reserved_bytes", "f8")]

    def __init__(self, session, masses, dt_fs, hbm_budget, max_batch_atoms, max_batch_frames):
        self._session = session   # kept alive while the server runs
        m = np.ascontiguousarray(masses, dtype=np.float64)
        h = ctypes.c_void_p()
        _check(lib().cg_md_server_start(session._h, _ptr(m), float(dt_fs), float(hbm_budget), int(max_batch_atoms),
                                        int(max_batch_frames), ctypes.byref(h)))
        self._h = h
        self._natoms = {}

    def submit(self, types, xyz, cell, v, nsteps):
        t = np.ascontiguousarray(types, dtype=np.int32)
        x = np.ascontiguousarray(xyz, dtype=np.float64)
        c = np.ascontiguousarray(cell, dtype=np.float64).reshape(9)
        vv = np.ascontiguousarray(v, dtype=np.float64)
        req = MdRequest(len(t), int(nsteps), 0.0, t.ctypes.data, x.ctypes.data, c.ctypes.data, vv.ctypes.data, None)
        tk = ctypes.c_int64()
        _check(lib().cg_md_server_submit(self._h, ctypes.byref(req), ctypes.byref(tk)))
        self._natoms[tk.value] = len(t)
        return tk.value

    def poll(self, ticket, wait=False):
        out = np.zeros((self._natoms[ticket], 3))
        res = MdResult()
        rc = lib().cg_md_server_poll(self._h, int(ticket), 1 if wait else 0, ctypes.byref(res), _ptr(out))
        if rc == CG_PENDING:
            return None
        _check(rc)
        r = np.array([(res.admitted, res.finished, res.step_ms_sum, res.step_ms_max, res.reserved_bytes)],
                     dtype=self._RESULT)[0]
        return out, r

    def stop(self):
        """Finishes every queued and running request; returns the batched steps run."""
        if self._h is None:
            return 0
        nb = ctypes.c_int64()
        h, self._h = self._h, None
        _check(lib().cg_md_server_stop(h, ctypes.byref(nb)))
        return nb.value

    def __del__(self):
        if getattr(self, "_h", None) is not None:
            lib().cg_md_server_stop(self._h, None)
            self._h = None


class Session:
    """One GPU (device ordinal) with a CUDA stream, bound to a model."""

    def __init__(self, model, device=0):
        h = ctypes.c_void_p()
        _check(lib().cg_session_create(model._h, int(device), ctypes.byref(h)))
        self._h = h
        self.model = model

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.cg_session_free(self._h)
            self._h = None

    @property
    def stream(self):
        """cudaStream_t of the session as an integer."""
        return lib().cg_session_stream(self._h) or 0

    def assemble(self, frames, precision=CG_FP64, out=None):
        """A matrix of the frames in host memory (float64 or float32)."""
        nrows = frames.nrows
        ncols = self.model.ncols
        dt = np.float64 if precision == CG_FP64 else np.float32
        if out is None:
            out = np.empty((nrows, ncols), dtype=dt)
        assert out.dtype == dt and out.flags.c_contiguous and out.shape[0] == nrows
        _check(lib().cg_assemble(self._h, frames._h, int(precision), _ptr(out), out.shape[1]))
        return out

    def assemble_stream(self, frames, precision, sink, block_frames=0):
        """cg_assemble_stream: sink(first_row, A_block) is called with each row block
        (a numpy view of pinned host memory, valid during the call); a truthy return
        stops the assembly."""
        ncols = self.model.ncols
        dt = np.float64 if precision == CG_FP64 else np.float32
        err = []

        def cb(user, first, nrows, ptr, lda):
            try:
                buf = (ctypes.c_char * (int(nrows) * int(lda) * np.dtype(dt).itemsize)).from_address(ptr)
                view = np.frombuffer(buf, dtype=dt).reshape(int(nrows), int(lda))[:, :ncols]
                return 1 if sink(int(first), view) else 0
            except Exception as e:   # noqa: BLE001  (reported after the call)
                err.append(e)
                return 1
        cfn = ROWS_SINK(cb)
        rc = lib().cg_assemble_stream(self._h, frames._h, int(precision), int(block_frames),
                                      ctypes.cast(cfn, ctypes.c_void_p), None)
        if err:
            raise err[0]
        _check(rc)

    def upload(self, frames):
        h = ctypes.c_void_p()
        _check(lib().cg_frames_upload(self._h, frames._h, ctypes.byref(h)))
        return DeviceFrames(h, frames.nrows)

    def assemble_device(self, dframes, precision, a_device_ptr, lda):
        """Assemble into a device buffer (asynchronous on the session stream)."""
        _check(lib().cg_assemble_device(self._h, dframes._h, int(precision), ctypes.c_void_p(int(a_device_ptr)),
                                        int(lda)))

    NSTAGES = 18

    def profile(self, enable=True):
        """Turn per-stage CUDA-event timing on/off (clears the totals)."""
        _check(lib().cg_session_profile(self._h, 1 if enable else 0))

    def stage_times(self):
        """{stage: (total_ms, calls)} accumulated since profile() was called."""
        ms = np.zeros(self.NSTAGES, dtype=np.float64)
        calls = np.zeros(self.NSTAGES, dtype=np.int64)
        _check(lib().cg_session_stage_times(self._h, _ptr(ms), _ptr(calls)))
        return {lib().cg_stage_name(k).decode(): (float(ms[k]), int(calls[k])) for k in range(self.NSTAGES)}

    def last_launches(self):
        v = ctypes.c_int64()
        _check(lib().cg_session_last_launches(self._h, ctypes.byref(v)))
        return v.value

    def assemble_device_noalloc(self, dframes, precision, a_device_ptr, lda):
        """Allocation-free variant of assemble_device (work buffers from a fixed
        device array inside the library; see include/chimes_gb300.h)."""
        _check(lib().cg_assemble_device_noalloc(self._h, dframes._h, int(precision),
                                                ctypes.c_void_p(int(a_device_ptr)), int(lda)))

    # ---------------------------------------------------------------- normal equations
    def gram(self, a_precision, a_ptr, lda, nrows, ncols, b_ptr, mode, g_ptr, h_ptr, w_ptr=0):
        """Accumulate G += A^T A (upper triangle), h += A^T b on the device (cg_gram);
        with w_ptr (device row weights) the weighted rows w A, w b (cg_gram_weighted)."""
        if w_ptr:
            _check(lib().cg_gram_weighted(self._h, int(a_precision), ctypes.c_void_p(int(a_ptr)),
                                          ctypes.c_int64(int(lda)), ctypes.c_int64(int(nrows)), int(ncols),
                                          ctypes.c_void_p(int(b_ptr)), ctypes.c_void_p(int(w_ptr)), int(mode),
                                          ctypes.c_void_p(int(g_ptr)), ctypes.c_void_p(int(h_ptr))))
            return
        _check(lib().cg_gram(self._h, int(a_precision), ctypes.c_void_p(int(a_ptr)), ctypes.c_int64(int(lda)),
                             ctypes.c_int64(int(nrows)), int(ncols), ctypes.c_void_p(int(b_ptr)), int(mode),
                             ctypes.c_void_p(int(g_ptr)), ctypes.c_void_p(int(h_ptr))))

    def gram_finish(self, g_ptr, ncols):
        _check(lib().cg_gram_finish(self._h, ctypes.c_void_p(int(g_ptr)), int(ncols)))

    def solve(self, g_ptr, h_ptr, ncols, ridge, a_ptr, lda, nrows, b_ptr, iters, x_ptr):
        """Ridge least squares (cg_solve); returns (||b - A x||, ||A^T r - ridge x||, ridge used)."""
        info = (ctypes.c_double * 3)()
        _check(lib().cg_solve(self._h, ctypes.c_void_p(int(g_ptr)), ctypes.c_void_p(int(h_ptr)), int(ncols),
                              ctypes.c_double(ridge), ctypes.c_void_p(int(a_ptr) or None), ctypes.c_int64(int(lda)),
                              ctypes.c_int64(int(nrows)), ctypes.c_void_p(int(b_ptr) or None), int(iters),
                              ctypes.c_void_p(int(x_ptr)), info))
        return info[0], info[1], info[2]

    def solve_streamed(self, g_ptr, h_ptr, ncols, ridge, dframes, label_ptrs, x_ptr, weight_ptrs=None, extra=None,
                       max_iters=50, tol=1e-12):
        """The mixed form's ridge solve without a stored FP64 A (cg_solve_streamed):
        FP64 Cholesky of G + ridge I, then CG passes that assemble every uploaded
        block again in FP64.  extra: (A_ptr, nrows, b_ptr, w_ptr or 0) of rows outside
        the frames (device).  Returns dict(iters, rel_update, rnorm0, rnorm, ridge)."""
        n = len(dframes)
        blocks = (ctypes.c_void_p * max(n, 1))(*[d._h.value if isinstance(d._h, ctypes.c_void_p) else d._h
                                                 for d in dframes])
        labels = (ctypes.c_void_p * max(n, 1))(*[int(p) for p in label_ptrs])
        weights = None
        if weight_ptrs is not None:
            weights = ctypes.cast((ctypes.c_void_p * max(n, 1))(*[int(p) for p in weight_ptrs]), ctypes.c_void_p)
        ea, er, eb, ew = extra if extra is not None else (0, 0, 0, 0)
        info = (ctypes.c_double * 5)()
        _check(lib().cg_solve_streamed(self._h, ctypes.c_void_p(int(g_ptr)), ctypes.c_void_p(int(h_ptr)), int(ncols),
                                       ctypes.c_double(ridge), n, ctypes.cast(blocks, ctypes.c_void_p),
                                       ctypes.cast(labels, ctypes.c_void_p), weights,
                                       ctypes.c_void_p(int(ea) or None), ctypes.c_int64(int(er)),
                                       ctypes.c_void_p(int(eb) or None), ctypes.c_void_p(int(ew) or None),
                                       int(max_iters), ctypes.c_double(tol), ctypes.c_void_p(int(x_ptr)), info))
        return {"iters": int(info[0]), "rel_update": info[1], "rnorm0": info[2], "rnorm": info[3], "ridge": info[4]}

    @staticmethod
    def _blocks(dframes, ptrs=None):
        n = len(dframes)
        b = (ctypes.c_void_p * max(n, 1))(*[d._h.value if isinstance(d._h, ctypes.c_void_p) else d._h
                                            for d in dframes])
        return b

    def cholesky(self, g_ptr, ncols, ridge, l_ptr):
        """cg_cholesky: L <- factor of G + r I; returns r."""
        r = ctypes.c_double()
        _check(lib().cg_cholesky(self._h, ctypes.c_void_p(int(g_ptr)), int(ncols), ctypes.c_double(ridge),
                                 ctypes.c_void_p(int(l_ptr)), ctypes.byref(r)))
        return r.value

    def cholesky_solve(self, l_ptr, ncols, h_ptr, x_ptr):
        _check(lib().cg_cholesky_solve(self._h, ctypes.c_void_p(int(l_ptr)), int(ncols), ctypes.c_void_p(int(h_ptr)),
                                       ctypes.c_void_p(int(x_ptr))))

    def refine_streamed(self, l_ptr, ncols, ridge, dframes, label_ptrs, x_ptr, max_iters=50, tol=1e-12):
        """cg_refine_streamed from the x at x_ptr; returns dict(iters, rel_update, rnorm0, rnorm)."""
        n = len(dframes)
        blocks = self._blocks(dframes)
        labels = (ctypes.c_void_p * max(n, 1))(*[int(p) for p in label_ptrs])
        info = (ctypes.c_double * 4)()
        _check(lib().cg_refine_streamed(self._h, ctypes.c_void_p(int(l_ptr)), int(ncols), ctypes.c_double(ridge), n,
                                        ctypes.cast(blocks, ctypes.c_void_p), ctypes.cast(labels, ctypes.c_void_p),
                                        None, None, ctypes.c_int64(0), None, None, int(max_iters),
                                        ctypes.c_double(tol), ctypes.c_void_p(int(x_ptr)), info))
        return {"iters": int(info[0]), "rel_update": info[1], "rnorm0": info[2], "rnorm": info[3]}

    def predict_streamed(self, dframes, x_ptr, y_ptr):
        """cg_predict_streamed: y = A x over the blocks' rows (device pointers)."""
        blocks = self._blocks(dframes)
        _check(lib().cg_predict_streamed(self._h, len(dframes), ctypes.cast(blocks, ctypes.c_void_p),
                                         ctypes.c_void_p(int(x_ptr)), ctypes.c_void_p(int(y_ptr))))

    def fp64_fma_rate(self):
        """Measured FP64 FMA rate of the session's GPU (TFLOP/s)."""
        v = ctypes.c_double()
        _check(lib().cg_fp64_fma_rate(self._h, ctypes.byref(v)))
        return v.value

    def tune(self, key, value):
        _check(lib().cg_session_tune(self._h, key.encode(), int(value)))

    def batch_fit(self, dframes, label_ptrs, a_precision, a_ptr, lda, g_ptr, h_ptr):
        """Capture the blocks' assembly + tensor-core Gram as one CUDA graph."""
        n = len(dframes)
        blocks = (ctypes.c_void_p * n)(*[d._h.value if isinstance(d._h, ctypes.c_void_p) else d._h for d in dframes])
        labels = (ctypes.c_void_p * n)(*[int(p) for p in label_ptrs])
        h = ctypes.c_void_p()
        _check(lib().cg_batch_fit_create(self._h, n, ctypes.cast(blocks, ctypes.c_void_p),
                                         ctypes.cast(labels, ctypes.c_void_p), int(a_precision),
                                         ctypes.c_void_p(int(a_ptr)), int(lda), ctypes.c_void_p(int(g_ptr)),
                                         ctypes.c_void_p(int(h_ptr)), ctypes.byref(h)))
        return BatchFit(h, self, (dframes, blocks, labels))

    def lars(self, g_ptr, h_ptr, ncols, nsamples, alpha, x_ptr, max_iter=100000):
        """LARS-lasso on the normal equations (cg_lars); returns (steps, active, final C/n)."""
        info = (ctypes.c_double * 3)()
        _check(lib().cg_lars(self._h, ctypes.c_void_p(int(g_ptr)), ctypes.c_void_p(int(h_ptr)), int(ncols),
                             int(nsamples), float(alpha), int(max_iter), ctypes.c_void_p(int(x_ptr)), info))
        return int(info[0]), int(info[1]), info[2]

    def dlars(self, g_ptr, h_ptr, ncols, nsamples, btb, lam, lasso, x_ptr, max_iter=10000000, colsum_ptr=0,
              bsum=0.0, max_norm=0.0, restart_in=None, restart_out=None):
        """The reference's DLARS (lars / lasso) on the normal equations (cg_dlars_ex);
        colsum_ptr (device A^T 1) and bsum select --normalize=y; max_iter, max_norm,
        restart_in / restart_out as its --iterations, --max_norm, --restart.  Returns
        (iterations, active, objective of the last vertex)."""
        info = (ctypes.c_double * 3)()
        enc = lambda p: os.fspath(p).encode() if p else None
        _check(lib().cg_dlars_ex(self._h, ctypes.c_void_p(int(g_ptr)), ctypes.c_void_p(int(h_ptr)), int(ncols),
                                 int(nsamples), float(btb), float(lam), 1 if lasso else 0,
                                 ctypes.c_void_p(int(colsum_ptr) or None), float(bsum), int(max_iter),
                                 float(max_norm), enc(restart_in), enc(restart_out), ctypes.c_void_p(int(x_ptr)),
                                 info))
        return int(info[0]), int(info[1]), info[2]

    # ---------------------------------------------------------------- MD force
    def md_setup(self, x, precision=CG_FP64, energy_offsets=False, penalty_dist=0.01, penalty_scale=1.0e4):
        """Coefficients x (one per A column) for the MD force (cg_md_setup)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        _check(lib().cg_md_setup(self._h, _ptr(x), x.size, int(precision), MD_ENERGY_OFFSETS if energy_offsets else 0,
                                 float(penalty_dist), float(penalty_scale)))

    def md_force(self, frames):
        """(forces [natoms_total, 3], scalars [nframes, 11]) of host frames."""
        nat = frames.natoms_total
        F = np.zeros((nat, 3), dtype=np.float64)
        S = np.zeros((frames.nframes, MD_NSCALAR), dtype=np.float64)
        _check(lib().cg_md_force(self._h, frames._h, _ptr(F), _ptr(S)))
        return F, S

    def md_force_device(self, dframes, forces_ptr, scalars_ptr):
        _check(lib().cg_md_force_device(self._h, dframes._h, ctypes.c_void_p(int(forces_ptr)),
                                        ctypes.c_void_p(int(scalars_ptr))))

    def md_nve(self, dframes, masses, dt_fs, nsteps, v_ptr, forces_ptr, scalars_ptr=0, ke_ptr=0):
        """nsteps NVE steps of uploaded frames (device buffers, see cg_md_nve)."""
        m = np.ascontiguousarray(masses, dtype=np.float64)
        _check(lib().cg_md_nve(self._h, dframes._h, _ptr(m), float(dt_fs), int(nsteps), ctypes.c_void_p(int(v_ptr)),
                               ctypes.c_void_p(int(forces_ptr)), ctypes.c_void_p(int(scalars_ptr) or None),
                               ctypes.c_void_p(int(ke_ptr) or None)))

    def md_nvt(self, dframes, masses, dt_fs, nsteps, style, temperature, tau_fs, v_ptr, forces_ptr, scalars_ptr=0,
               ke_ptr=0, cons_ptr=0):
        """nsteps thermostatted steps (cg_md_nvt; style CG_NVT_MTK or CG_NVT_BEREND)."""
        m = np.ascontiguousarray(masses, dtype=np.float64)
        _check(lib().cg_md_nvt(self._h, dframes._h, _ptr(m), float(dt_fs), int(nsteps), int(style), float(temperature),
                               float(tau_fs), ctypes.c_void_p(int(v_ptr)), ctypes.c_void_p(int(forces_ptr)),
                               ctypes.c_void_p(int(scalars_ptr) or None), ctypes.c_void_p(int(ke_ptr) or None),
                               ctypes.c_void_p(int(cons_ptr) or None)))

    def md_npt(self, dframes, masses, dt_fs, nsteps, style, temperature, tau_fs, pressure_gpa, tau_baro_fs, v_ptr,
               forces_ptr, scalars_ptr=0, ke_ptr=0, cons_ptr=0, vol_ptr=0):
        """nsteps NPT steps (cg_md_npt; style CG_NPT_BEREND, CG_NPT_BEREND_ANISO or CG_NPT_MTK)."""
        m = np.ascontiguousarray(masses, dtype=np.float64)
        opt = [ctypes.c_void_p(int(p) or None) for p in (scalars_ptr, ke_ptr, cons_ptr, vol_ptr)]
        _check(lib().cg_md_npt(self._h, dframes._h, _ptr(m), float(dt_fs), int(nsteps), int(style), float(temperature),
                               float(tau_fs), float(pressure_gpa), float(tau_baro_fs), ctypes.c_void_p(int(v_ptr)),
                               ctypes.c_void_p(int(forces_ptr)), *opt))

    def md_write_restart(self, frame, path, types, xyz, v, acc, cell, step, rcut_padding, avg7=None, wrap=False):
        """restart.xyzv of one frame after the last MD run (cg_md_write_restart)."""
        t = np.ascontiguousarray(types, dtype=np.int32)
        x, vv, a = (np.ascontiguousarray(z, dtype=np.float64) for z in (xyz, v, acc))
        c = np.ascontiguousarray(cell, dtype=np.float64).reshape(9)
        av = None if avg7 is None else np.ascontiguousarray(avg7, dtype=np.float64)
        _check(lib().cg_md_write_restart(self._h, int(frame), os.fspath(path).encode(), len(t), _ptr(t), _ptr(x),
                                         _ptr(vv), _ptr(a), _ptr(c), int(step), float(rcut_padding), _ptr(av),
                                         int(bool(wrap))))

    def md_numerical_pressure(self, frames):
        """-dU/dV of each frame (cg_md_numerical what=0), kcal/mol/A^3."""
        out = np.zeros(frames.nframes)
        _check(lib().cg_md_numerical(self._h, frames._h, 0, _ptr(out)))
        return out

    def md_numerical_stress(self, frames):
        """Finite-difference stress tensor of each frame ([nframes, 3, 3], cg_md_numerical what=1)."""
        out = np.zeros((frames.nframes, 3, 3))
        _check(lib().cg_md_numerical(self._h, frames._h, 1, _ptr(out)))
        return out

    def md_resume(self, constraint29):
        """The next md_nvt / md_npt starts from these CONSTRAINT values ([nframes, 29])."""
        c = np.ascontiguousarray(constraint29, dtype=np.float64).reshape(-1, 29)
        _check(lib().cg_md_resume(self._h, c.shape[0], _ptr(c)))

    def md_serve(self, requests, masses, dt_fs=0.2, hbm_budget=150e9, max_batch_atoms=1 << 16,
                 max_batch_frames=1024, want_step_ms=True):
        """Continuous-batching NVE serving (cg_md_serve).  requests: list of dicts with
        types, xyz [n,3], cell [9], v [n,3], nsteps, arrival (s).  Returns (final xyz
        list, results structured array, step_ms [nreq, max nsteps] or None, batched steps)."""
        keep = []
        arr = (MdRequest * len(requests))()
        outs = []
        for k, q in enumerate(requests):
            t = np.ascontiguousarray(q["types"], dtype=np.int32)
            x = np.ascontiguousarray(q["xyz"], dtype=np.float64)
            c = np.ascontiguousarray(q["cell"], dtype=np.float64).reshape(9)
            v = np.ascontiguousarray(q["v"], dtype=np.float64)
            o = np.zeros_like(x)
            keep += [t, x, c, v]
            outs.append(o)
            arr[k] = MdRequest(len(t), int(q["nsteps"]), float(q.get("arrival", 0.0)), t.ctypes.data, x.ctypes.data,
                               c.ctypes.data, v.ctypes.data, o.ctypes.data)
        res = (MdResult * len(requests))()
        smax = max([int(q["nsteps"]) for q in requests] + [1])
        step_ms = np.zeros((len(requests), smax)) if want_step_ms else None
        nb = ctypes.c_int64()
        m = np.ascontiguousarray(masses, dtype=np.float64)
        _check(lib().cg_md_serve(self._h, len(requests), ctypes.cast(arr, ctypes.c_void_p), _ptr(m), float(dt_fs),
                                 float(hbm_budget), int(max_batch_atoms), int(max_batch_frames),
                                 ctypes.cast(res, ctypes.c_void_p), _ptr(step_ms), ctypes.byref(nb)))
        r = np.array([(x.admitted, x.finished, x.step_ms_sum, x.step_ms_max, x.reserved_bytes) for x in res],
                     dtype=[("admitted", "f8"), ("finished", "f8"), ("step_ms_sum", "f8"), ("step_ms_max", "f8"),
                            ("reserved_bytes", "f8")])
        return outs, r, step_ms, nb.value

    def md_serve_memory(self, max_batch_atoms=1 << 16, max_batch_frames=1024):
        """(arena bytes, reserved bytes per atom) of md_serve for these capacities."""
        a, p = ctypes.c_double(), ctypes.c_double()
        _check(lib().cg_md_serve_memory(self._h, int(max_batch_atoms), int(max_batch_frames), ctypes.byref(a),
                                        ctypes.byref(p)))
        return a.value, p.value

    def md_server(self, masses, dt_fs=0.2, hbm_budget=150e9, max_batch_atoms=1 << 16, max_batch_frames=1024):
        """Live continuous-batching server on this session (cg_md_server_start): submit
        requests from any thread while it runs, poll their results, stop() at the end.
        The session belongs to the server until stop()."""
        return MdServer(self, masses, dt_fs, hbm_budget, max_batch_atoms, max_batch_frames)

    def md_last_counts(self):
        v = [ctypes.c_int64() for _ in range(4)]
        _check(lib().cg_md_last_counts(self._h, *[ctypes.byref(x) for x in v]))
        return dict(zip(["pairs", "triplets", "quads", "launches"], [x.value for x in v]))

    def last_counts(self):
        v = [ctypes.c_int64() for _ in range(5)]
        _check(lib().cg_session_last_counts(self._h, *[ctypes.byref(x) for x in v]))
        return dict(zip(["pairs", "triplets", "quads", "evals3", "evals4"], [x.value for x in v]))
