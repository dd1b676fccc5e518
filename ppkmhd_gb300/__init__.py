"""ppkmhd_gb300: GB300-native MUSCL-Hancock + HLLD + CT MHD step.

Python view of the C ABI in ``include/ppkmhd_gb300.h`` (library
``ppkmhd_gb300/lib/libppkmhd_gb300.so``, built by ``ppkmhd_gb300.build``).
The compute path is the CUDA library only: if it is missing, importing the
binding raises, and creating a solver without a GPU returns the library's
MHD_ERR_NO_DEVICE as an exception.  There is no CPU fallback.

Typical use, mirroring ppkMHD's driver (src/main.cpp)::

    from ppkmhd_gb300 import MHDSolver
    s = MHDSolver.from_ini(open("orszag_tang_2d.ini").read())
    s.init_problem()
    s.run(100)
    U = s.get_state()           # numpy [var][(k)][j][i], ghosts included
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libppkmhd_gb300.so")

MHD_OK = 0
MHD_ERR_INVALID_ARG = -1
MHD_ERR_CUDA = -2
MHD_ERR_NO_DEVICE = -3
MHD_ERR_NUMERIC = -4
MHD_ERR_PARSE = -5
MHD_ERR_TOO_LARGE = -6
MHD_FINISHED = 1  # mhd_step_noalloc: t >= tEnd, nothing computed
MHD_ENSEMBLE_GRAPHS, MHD_ENSEMBLE_PERSISTENT, MHD_ENSEMBLE_FUSED = 0, 1, 2

MHD_RIEMANN_APPROX, MHD_RIEMANN_LLF, MHD_RIEMANN_HLL, MHD_RIEMANN_HLLC, MHD_RIEMANN_HLLD = range(5)
MHD_SOLVER_MHD_MUSCL, MHD_SOLVER_HYDRO_MUSCL = 0, 1
MHD_FORM_STAGES, MHD_FORM_FUSED, MHD_FORM_TIMED = 0, 1, 2
MHD_BC_REFLECTING, MHD_BC_OUTFLOW, MHD_BC_PERIODIC = 1, 2, 3
MHD_FP64, MHD_FP32 = 64, 32
MHD_FP_FAST, MHD_FP_EXACT = 0, 1
MHD_LAYOUT_LEFT, MHD_LAYOUT_RIGHT = 0, 1
MHD_PROBLEM_ORSZAG_TANG = 0
(MHD_PROBLEM_BLAST, MHD_PROBLEM_IMPLODE, MHD_PROBLEM_KELVIN_HELMHOLTZ, MHD_PROBLEM_ROTOR,
 MHD_PROBLEM_FIELD_LOOP, MHD_PROBLEM_WAVE) = range(1, 7)
# hydro solver problems
(MHD_PROBLEM_GRESHO_VORTEX, MHD_PROBLEM_FOUR_QUADRANT, MHD_PROBLEM_ISENTROPIC_VORTEX,
 MHD_PROBLEM_RAYLEIGH_TAYLOR, MHD_PROBLEM_RISING_BUBBLE) = range(7, 12)
MHD_MLP_PARAMS = 7832
MHD_MLP_FEATURES = 40
MHD_SAMPLE_FLOATS = 24
MHD_MLP_TRAIN, MHD_MLP_CHECK = 0, 1
MHD_MLP_WAIT_POLLS = 1 << 20
MHD_MLP_FORWARD_TILES = 0
MHD_MLP_FORWARD_PERSISTENT = 1


class MHDParams(ctypes.Structure):
    """Mirror of ``mhd_params`` (include/ppkmhd_gb300.h)."""

    _fields_ = [
        ("dim", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("ghost", ctypes.c_int),
        ("xmin", ctypes.c_double), ("xmax", ctypes.c_double), ("ymin", ctypes.c_double),
        ("ymax", ctypes.c_double), ("zmin", ctypes.c_double), ("zmax", ctypes.c_double),
        ("gamma0", ctypes.c_double), ("cfl", ctypes.c_double), ("slope_type", ctypes.c_double),
        ("smallr", ctypes.c_double), ("smallc", ctypes.c_double),
        ("riemann", ctypes.c_int), ("implementation_version", ctypes.c_int),
        ("boundary", ctypes.c_int * 6),
        ("tEnd", ctypes.c_double), ("tCurrent", ctypes.c_double), ("nStepmax", ctypes.c_int),
        ("problem", ctypes.c_int), ("ot_kt", ctypes.c_double),
        ("precision", ctypes.c_int), ("fp_mode", ctypes.c_int), ("device", ctypes.c_int),
        ("problem_real", ctypes.c_double * 24), ("problem_int", ctypes.c_int * 4),
        ("solver", ctypes.c_int), ("gravity", ctypes.c_int),
        ("gravity_field", ctypes.c_double * 3),
    ]

    @property
    def nvar(self) -> int:
        """Variables of the state arrays: 8 (MHD) or dim + 2 (hydro)."""
        return self.dim + 2 if self.solver == MHD_SOLVER_HYDRO_MUSCL else 8

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_}
        for f in ("boundary", "problem_real", "problem_int", "gravity_field"):
            d[f] = list(getattr(self, f))
        return d


class MHDError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


# Every entry point of include/ppkmhd_gb300.h with its ctypes signature.
_vp = ctypes.c_void_p
_ip = ctypes.POINTER(ctypes.c_int)
_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_i64p = ctypes.POINTER(ctypes.c_int64)
SIGNATURES = {
    "mhd_params_default": (ctypes.c_int, [ctypes.POINTER(MHDParams)]),
    "mhd_write_vtk": (ctypes.c_int, [ctypes.c_char_p, _vp, ctypes.c_int, ctypes.c_char_p,
                                     ctypes.c_size_t]),
    "mhd_params_from_ini": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(MHDParams),
                                           ctypes.c_char_p, ctypes.c_size_t]),
    "mhd_create": (ctypes.c_int, [ctypes.POINTER(MHDParams), ctypes.POINTER(_vp)]),
    "mhd_destroy": (ctypes.c_int, [_vp]),
    "mhd_init_problem": (ctypes.c_int, [_vp]),
    "mhd_initial_state": (ctypes.c_int, [ctypes.POINTER(MHDParams), _vp]),
    "mhd_set_state": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int]),
    "mhd_get_state": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int]),
    "mhd_step": (ctypes.c_int, [_vp]),
    "mhd_compute_dt": (ctypes.c_int, [_vp, _dp]),
    "mhd_step_dt": (ctypes.c_int, [_vp, ctypes.c_double]),
    "mhd_run": (ctypes.c_int, [_vp, ctypes.c_int, _ip]),
    "mhd_step_host": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, ctypes.c_int]),
    "mhd_set_host_slabs": (ctypes.c_int, [_vp, ctypes.c_int]),
    "mhd_set_fused": (ctypes.c_int, [_vp, ctypes.c_int]),
    "mhd_get_fused": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int)]),
    "mhd_time": (ctypes.c_int, [_vp, _dp, _dp, _ip]),
    "mhd_diagnostics": (ctypes.c_int, [_vp, _dp, _dp, _dp]),
    "mhd_run_timed": (ctypes.c_int, [_vp, ctypes.c_int, _fp]),
    "mhd_profile_step": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_char_p), _fp, ctypes.c_int,
                                        _ip]),
    "mhd_cell_counts": (ctypes.c_int, [_vp, _i64p, _i64p]),
    "mhd_sizes": (ctypes.c_int, [_vp, _ip]),
    "mhd_launches_per_step": (ctypes.c_int, [_vp, _ip]),
    "mhd_last_error": (ctypes.c_char_p, [_vp]),
    "mhd_version": (ctypes.c_char_p, []),
    "mhd_step_noalloc": (ctypes.c_int, [ctypes.POINTER(MHDParams), _vp, _vp, ctypes.c_double,
                                        _dp, _vp]),
    "mhd_ensemble_create": (ctypes.c_int, [ctypes.POINTER(MHDParams), ctypes.c_int,
                                           ctypes.POINTER(_vp)]),
    "mhd_ensemble_destroy": (ctypes.c_int, [_vp]),
    "mhd_ensemble_init_problem": (ctypes.c_int, [_vp, ctypes.c_int]),
    "mhd_ensemble_set_state": (ctypes.c_int, [_vp, ctypes.c_int, _vp, ctypes.c_int, ctypes.c_int]),
    "mhd_ensemble_set_states": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int]),
    "mhd_ensemble_get_states": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int]),
    "mhd_ensemble_get_state": (ctypes.c_int, [_vp, ctypes.c_int, _vp, ctypes.c_int, ctypes.c_int]),
    "mhd_ensemble_run": (ctypes.c_int, [_vp, ctypes.c_int, _fp]),
    "mhd_ensemble_time": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp, _ip]),
    "mhd_ensemble_diagnostics": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _dp, _dp]),
    "mhd_ensemble_set_mode": (ctypes.c_int, [_vp, ctypes.c_int]),
    "mhd_ensemble_get_mode": (ctypes.c_int, [_vp, _ip]),
    "mhd_ensemble_set_wait_limit": (ctypes.c_int, [_vp, ctypes.c_longlong]),
    "mhd_ensemble_autotune": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_size_t]),
    "mhd_ensemble_profile_step": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_char_p), _fp,
                                                 ctypes.c_int, _ip]),
    "mhd_ensemble_cell_count": (ctypes.c_int, [_vp, _i64p]),
    "mhd_ensemble_launches_per_step": (ctypes.c_int, [_vp, _ip]),
    "mhd_ensemble_last_error": (ctypes.c_char_p, [_vp]),
    "mhd_harvest_faces": (ctypes.c_int, [_vp, ctypes.c_int, _vp, ctypes.c_int64, _i64p]),
    "mhd_checkpoint_save": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_int]),
    "mhd_checkpoint_load": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_int, _ip]),
    "mhd_checkpoint_load_upscaled": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_int, _ip]),
    "mhd_mlp_create": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_double, ctypes.POINTER(_vp)]),
    "mhd_mlp_destroy": (ctypes.c_int, [_vp]),
    "mhd_mlp_set_params": (ctypes.c_int, [_vp, _vp, ctypes.c_int]),
    "mhd_mlp_get_params": (ctypes.c_int, [_vp, _vp, ctypes.c_int]),
    "mhd_mlp_gamma": (ctypes.c_int, [_vp, _dp]),
    "mhd_mlp_encode": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, _vp, _vp]),
    "mhd_mlp_gradient": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int64, ctypes.c_int, _vp, _dp]),
    "mhd_mlp_train": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_float, ctypes.c_float, ctypes.c_uint64, _vp]),
    "mhd_mlp_forward": (ctypes.c_int, [_vp, _vp, ctypes.c_int64, _vp]),
    "mhd_mlp_set_wait_limit": (ctypes.c_int, [_vp, ctypes.c_int]),
    "mhd_mlp_set_forward_form": (ctypes.c_int, [_vp, ctypes.c_int]),
    "mhd_mlp_last_forward_ms": (ctypes.c_int, [_vp, _dp]),
    "mhd_mlp_last_error": (ctypes.c_char_p, [_vp]),
    "mhd_set_surrogate": (ctypes.c_int, [_vp, _vp, ctypes.c_double]),
    "mhd_surrogate_stats": (ctypes.c_int, [_vp, _i64p, _i64p, ctypes.c_int]),
}

_lib = None


def lib():
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -m ppkmhd_gb300.build` "
                "(this package has no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def params_from_ini(ini_text: str) -> MHDParams:
    p = MHDParams()
    err = ctypes.create_string_buffer(512)
    rc = lib().mhd_params_from_ini(ini_text.encode(), ctypes.byref(p), err, len(err))
    if rc != MHD_OK:
        raise MHDError(rc, err.value.decode())
    return p


def initial_state(params: MHDParams) -> np.ndarray:
    """The initial condition of params.problem (host FP64, LayoutLeft, ghosts
    included, before any boundary fill)."""
    g, nv = params.ghost, params.nvar
    shape = (nv, params.ny + 2 * g, params.nx + 2 * g) if params.dim == 2 else \
        (nv, params.nz + 2 * g, params.ny + 2 * g, params.nx + 2 * g)
    U = np.empty(shape, dtype=np.float64)
    rc = lib().mhd_initial_state(ctypes.byref(params), U.ctypes.data)
    if rc != MHD_OK:
        raise MHDError(rc, "invalid parameters")
    return U


def write_vtk(ini_text: str, U: np.ndarray, istep: int = 0) -> str:
    """Write the LayoutLeft FP64 state U as the reference's .vti file (the
    .ini's [output] outputDir / outputPrefix / outputVtkAscii); returns the
    file name.  Host only."""
    U = np.ascontiguousarray(U, dtype=np.float64)
    path = ctypes.create_string_buffer(4096)
    rc = lib().mhd_write_vtk(ini_text.encode(), U.ctypes.data, int(istep), path, len(path))
    if rc != MHD_OK:
        raise MHDError(rc, "mhd_write_vtk failed")
    return path.value.decode()


def default_params() -> MHDParams:
    p = MHDParams()
    lib().mhd_params_default(ctypes.byref(p))
    return p


class MHDSolver:
    """One problem on the GPU (an ``mhd_ctx``): the MHD MUSCL solver, or the
    hydro-only MUSCL solver when ``params.solver`` is MHD_SOLVER_HYDRO_MUSCL
    ([run] solver_name Hydro_Muscl_2D/3D)."""

    def __init__(self, params: MHDParams):
        self.params = params
        self.h = _vp()
        rc = lib().mhd_create(ctypes.byref(params), ctypes.byref(self.h))
        if rc != MHD_OK:
            msg = lib().mhd_last_error(self.h).decode() if self.h else "mhd_create failed"
            if self.h:
                lib().mhd_destroy(self.h)
                self.h = _vp()
            raise MHDError(rc, msg)
        self.real = np.float64 if params.precision == MHD_FP64 else np.float32
        s = (ctypes.c_int * 4)()
        lib().mhd_sizes(self.h, s)
        self.isize, self.jsize, self.ksize, self.nbvar = list(s)

    @classmethod
    def from_ini(cls, ini_text: str, precision: int | None = None, fp_mode: int | None = None):
        p = params_from_ini(ini_text)
        if precision is not None:
            p.precision = precision
        if fp_mode is not None:
            p.fp_mode = fp_mode
        return cls(p)

    # ------------------------------------------------------------------
    def _check(self, rc: int):
        if rc != MHD_OK:
            raise MHDError(rc, lib().mhd_last_error(self.h).decode())

    def close(self):
        if self.h:
            lib().mhd_destroy(self.h)
            self.h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def shape_left(self):
        if self.params.dim == 2:
            return (self.nbvar, self.jsize, self.isize)
        return (self.nbvar, self.ksize, self.jsize, self.isize)

    @property
    def shape_right(self):
        if self.params.dim == 2:
            return (self.isize, self.jsize, self.nbvar)
        return (self.isize, self.jsize, self.ksize, self.nbvar)

    def init_problem(self):
        self._check(lib().mhd_init_problem(self.h))

    def set_state(self, U: np.ndarray, layout: int = MHD_LAYOUT_LEFT):
        U = np.ascontiguousarray(U, dtype=self.real)
        want = self.shape_left if layout == MHD_LAYOUT_LEFT else self.shape_right
        if U.shape != want:
            raise ValueError(f"state shape {U.shape} != {want}")
        self._check(lib().mhd_set_state(self.h, U.ctypes.data, layout, U.itemsize))

    def get_state(self, layout: int = MHD_LAYOUT_LEFT, out: np.ndarray | None = None):
        shape = self.shape_left if layout == MHD_LAYOUT_LEFT else self.shape_right
        U = np.empty(shape, dtype=self.real) if out is None else out
        self._check(lib().mhd_get_state(self.h, U.ctypes.data, layout, U.itemsize))
        return U

    def step(self):
        self._check(lib().mhd_step(self.h))

    def compute_dt(self) -> float:
        """The CFL dt (clipped to tEnd) the next step would take."""
        dt = ctypes.c_double()
        self._check(lib().mhd_compute_dt(self.h, ctypes.byref(dt)))
        return dt.value

    def step_dt(self, dt: float):
        """One iteration with the given dt instead of the CFL dt."""
        self._check(lib().mhd_step_dt(self.h, float(dt)))

    def run(self, n: int) -> int:
        done = ctypes.c_int(0)
        self._check(lib().mhd_run(self.h, int(n), ctypes.byref(done)))
        return done.value

    def step_host(self, U_in: np.ndarray, U_out: np.ndarray, layout: int = MHD_LAYOUT_LEFT):
        self._check(lib().mhd_step_host(self.h, U_in.ctypes.data, U_out.ctypes.data, layout,
                                        U_in.itemsize))

    def step_host_ptr(self, in_ptr: int, out_ptr: int, layout: int = MHD_LAYOUT_LEFT):
        """Same as step_host on raw host pointers (e.g. pinned buffers)."""
        itemsize = 8 if self.params.precision == MHD_FP64 else 4
        self._check(lib().mhd_step_host(self.h, in_ptr, out_ptr, layout, itemsize))

    def set_host_slabs(self, n: int):
        """Slab count of step_host (0 = automatic, 1 = no copy/compute overlap)."""
        self._check(lib().mhd_set_host_slabs(self.h, int(n)))

    def set_fused(self, fused):
        """True: the fused tile form (hydro solver; 2D MHD solver, version 2);
        False: the stage kernels; "timed": the next stepping call times one
        iteration of each and keeps the faster.  Without a call the context
        runs the form its configuration maps to."""
        form = MHD_FORM_TIMED if fused == "timed" else int(bool(fused))
        self._check(lib().mhd_set_fused(self.h, form))

    @property
    def fused(self) -> bool:
        v = ctypes.c_int()
        self._check(lib().mhd_get_fused(self.h, ctypes.byref(v)))
        return bool(v.value)

    def time(self):
        t, dt, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        self._check(lib().mhd_time(self.h, ctypes.byref(t), ctypes.byref(dt), ctypes.byref(it)))
        return t.value, dt.value, it.value

    def diagnostics(self):
        sums = (ctypes.c_double * 8)()
        l1, mx = ctypes.c_double(), ctypes.c_double()
        self._check(lib().mhd_diagnostics(self.h, sums, ctypes.byref(l1), ctypes.byref(mx)))
        return np.array(list(sums)), l1.value, mx.value

    def run_timed(self, n: int) -> float:
        ms = ctypes.c_float()
        self._check(lib().mhd_run_timed(self.h, int(n), ctypes.byref(ms)))
        return ms.value

    def profile_step(self):
        names = (ctypes.c_char_p * 16)()
        ms = (ctypes.c_float * 16)()
        cnt = ctypes.c_int()
        self._check(lib().mhd_profile_step(self.h, names, ms, 16, ctypes.byref(cnt)))
        return [(names[q].decode(), ms[q]) for q in range(cnt.value)]

    def cell_counts(self):
        a, b = ctypes.c_int64(), ctypes.c_int64()
        self._check(lib().mhd_cell_counts(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def launches_per_step(self) -> int:
        n = ctypes.c_int()
        self._check(lib().mhd_launches_per_step(self.h, ctypes.byref(n)))
        return n.value

    def checkpoint_save(self, path: str, times_saved: int = 0):
        self._check(lib().mhd_checkpoint_save(self.h, os.fsencode(path), int(times_saved)))

    def checkpoint_load(self, path: str, reset_time: bool = False) -> int:
        """Restore state and time from a checkpoint; returns its output counter."""
        ts = ctypes.c_int()
        self._check(lib().mhd_checkpoint_load(self.h, os.fsencode(path), int(reset_time),
                                              ctypes.byref(ts)))
        return ts.value

    def checkpoint_load_upscaled(self, path: str, reset_time: bool = False) -> int:
        """Restore from a checkpoint of half the resolution ([run]
        restart_upscale); returns its output counter."""
        ts = ctypes.c_int()
        self._check(lib().mhd_checkpoint_load_upscaled(self.h, os.fsencode(path), int(reset_time),
                                                       ctypes.byref(ts)))
        return ts.value

    def harvest(self, stride: int = 1) -> np.ndarray:
        """Face records of the next iteration, shape (n, MHD_SAMPLE_FLOATS)."""
        cnt = ctypes.c_int64()
        self._check(lib().mhd_harvest_faces(self.h, int(stride), None, 0, ctypes.byref(cnt)))
        out = np.empty((cnt.value, MHD_SAMPLE_FLOATS), dtype=np.float32)
        self._check(lib().mhd_harvest_faces(self.h, int(stride), out.ctypes.data, cnt.value,
                                            ctypes.byref(cnt)))
        return out

    def set_surrogate(self, mlp, tau: float = 0.01):
        """Use the network `mlp` (an ppkmhd_gb300.surrogate.FluxMLP) in the flux
        stage; None restores HLLD everywhere."""
        self._check(lib().mhd_set_surrogate(self.h, mlp.h if mlp is not None else None,
                                            float(tau)))

    def surrogate_stats(self, reset: bool = False):
        a, b = ctypes.c_int64(), ctypes.c_int64()
        self._check(lib().mhd_surrogate_stats(self.h, ctypes.byref(a), ctypes.byref(b),
                                              int(reset)))
        return a.value, b.value


def interior(U: np.ndarray, ghost: int = 3) -> np.ndarray:
    g = ghost
    if U.ndim == 3:
        return U[:, g:-g, g:-g]
    return U[:, g:-g, g:-g, g:-g]


class MHDEnsemble:
    """Many independent problems advanced together (an ``mhd_ensemble``)."""

    def __init__(self, params: list):
        self.params = list(params)
        n = len(self.params)
        arr = (MHDParams * n)(*self.params)
        self.h = _vp()
        rc = lib().mhd_ensemble_create(arr, n, ctypes.byref(self.h))
        if rc != MHD_OK:
            msg = (lib().mhd_ensemble_last_error(self.h).decode() if self.h
                   else "mhd_ensemble_create failed")
            if self.h:
                lib().mhd_ensemble_destroy(self.h)
                self.h = _vp()
            raise MHDError(rc, msg)
        self.real = np.float64 if self.params[0].precision == MHD_FP64 else np.float32

    @classmethod
    def from_ini(cls, ini_texts, precision: int | None = None, fp_mode: int | None = None):
        ps = []
        for t in ini_texts:
            p = params_from_ini(t)
            if precision is not None:
                p.precision = precision
            if fp_mode is not None:
                p.fp_mode = fp_mode
            ps.append(p)
        return cls(ps)

    def _check(self, rc: int):
        if rc != MHD_OK:
            raise MHDError(rc, lib().mhd_ensemble_last_error(self.h).decode())

    def close(self):
        if self.h:
            lib().mhd_ensemble_destroy(self.h)
            self.h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __len__(self):
        return len(self.params)

    def shape_left(self, prob: int):
        p = self.params[prob]
        g = p.ghost
        if p.dim == 2:
            return (8, p.ny + 2 * g, p.nx + 2 * g)
        return (8, p.nz + 2 * g, p.ny + 2 * g, p.nx + 2 * g)

    def shape_right(self, prob: int):
        return tuple(reversed(self.shape_left(prob)[1:])) + (8,)

    def init_problem(self, prob: int):
        self._check(lib().mhd_ensemble_init_problem(self.h, int(prob)))

    def set_state(self, prob: int, U: np.ndarray, layout: int = MHD_LAYOUT_LEFT):
        U = np.ascontiguousarray(U, dtype=self.real)
        want = self.shape_left(prob) if layout == MHD_LAYOUT_LEFT else self.shape_right(prob)
        if U.shape != want:
            raise ValueError(f"state shape {U.shape} != {want}")
        self._check(lib().mhd_ensemble_set_state(self.h, int(prob), U.ctypes.data, layout,
                                                 U.itemsize))

    def get_state(self, prob: int, layout: int = MHD_LAYOUT_LEFT):
        shape = self.shape_left(prob) if layout == MHD_LAYOUT_LEFT else self.shape_right(prob)
        U = np.empty(shape, dtype=self.real)
        self._check(lib().mhd_ensemble_get_state(self.h, int(prob), U.ctypes.data, layout,
                                                 U.itemsize))
        return U

    def set_states(self, states, layout: int = MHD_LAYOUT_LEFT):
        """Every problem's state in one call (one synchronisation)."""
        arrs = []
        for q, U in enumerate(states):
            U = np.ascontiguousarray(U, dtype=self.real)
            want = self.shape_left(q) if layout == MHD_LAYOUT_LEFT else self.shape_right(q)
            if U.shape != want:
                raise ValueError(f"state {q} shape {U.shape} != {want}")
            arrs.append(U)
        if len(arrs) != len(self.params):
            raise ValueError(f"{len(arrs)} states for {len(self.params)} problems")
        self.set_states_ptr([U.ctypes.data for U in arrs], layout)

    def set_states_ptr(self, ptrs, layout: int = MHD_LAYOUT_LEFT):
        """set_states on raw host pointers (e.g. pinned buffers), one per problem."""
        if len(ptrs) != len(self.params):
            raise ValueError(f"{len(ptrs)} pointers for {len(self.params)} problems")
        arr = (ctypes.c_void_p * len(ptrs))(*ptrs)
        self._check(lib().mhd_ensemble_set_states(self.h, arr, layout, np.dtype(self.real).itemsize))

    def get_states(self, layout: int = MHD_LAYOUT_LEFT):
        """Every problem's state in one call (one synchronisation)."""
        out = [np.empty(self.shape_left(q) if layout == MHD_LAYOUT_LEFT else self.shape_right(q),
                        dtype=self.real) for q in range(len(self.params))]
        self.get_states_ptr([U.ctypes.data for U in out], layout)
        return out

    def get_states_ptr(self, ptrs, layout: int = MHD_LAYOUT_LEFT):
        """get_states into raw host pointers, one per problem."""
        if len(ptrs) != len(self.params):
            raise ValueError(f"{len(ptrs)} pointers for {len(self.params)} problems")
        arr = (ctypes.c_void_p * len(ptrs))(*ptrs)
        self._check(lib().mhd_ensemble_get_states(self.h, arr, layout, np.dtype(self.real).itemsize))

    def run(self, n: int) -> float:
        """n iterations of every unfinished problem; returns device milliseconds."""
        ms = ctypes.c_float()
        self._check(lib().mhd_ensemble_run(self.h, int(n), ctypes.byref(ms)))
        return ms.value

    def time(self, prob: int):
        t, dt, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        self._check(lib().mhd_ensemble_time(self.h, int(prob), ctypes.byref(t), ctypes.byref(dt),
                                            ctypes.byref(it)))
        return t.value, dt.value, it.value

    def diagnostics(self, prob: int):
        sums = (ctypes.c_double * 8)()
        l1, mx = ctypes.c_double(), ctypes.c_double()
        self._check(lib().mhd_ensemble_diagnostics(self.h, int(prob), sums, ctypes.byref(l1),
                                                   ctypes.byref(mx)))
        return np.array(list(sums)), l1.value, mx.value

    def set_mode(self, mode: int):
        """MHD_ENSEMBLE_GRAPHS, MHD_ENSEMBLE_PERSISTENT or (2D) MHD_ENSEMBLE_FUSED."""
        self._check(lib().mhd_ensemble_set_mode(self.h, int(mode)))

    @property
    def mode(self) -> int:
        m = ctypes.c_int()
        self._check(lib().mhd_ensemble_get_mode(self.h, ctypes.byref(m)))
        return m.value

    def set_wait_limit(self, cycles: int):
        """Clock-cycle bound of the persistent form's barrier waits (0: give
        up at once)."""
        self._check(lib().mhd_ensemble_set_wait_limit(self.h, int(cycles)))

    def autotune(self) -> str:
        buf = ctypes.create_string_buffer(8192)
        self._check(lib().mhd_ensemble_autotune(self.h, buf, len(buf)))
        return buf.value.decode()

    def profile_step(self):
        names = (ctypes.c_char_p * 16)()
        ms = (ctypes.c_float * 16)()
        cnt = ctypes.c_int()
        self._check(lib().mhd_ensemble_profile_step(self.h, names, ms, 16, ctypes.byref(cnt)))
        return [(names[q].decode(), ms[q]) for q in range(cnt.value)]

    def cell_count(self) -> int:
        a = ctypes.c_int64()
        self._check(lib().mhd_ensemble_cell_count(self.h, ctypes.byref(a)))
        return a.value

    def launches_per_step(self) -> int:
        n = ctypes.c_int()
        self._check(lib().mhd_ensemble_launches_per_step(self.h, ctypes.byref(n)))
        return n.value
