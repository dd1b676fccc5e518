"""ctypes bindings for the CPU oracle (test infrastructure only).

Two checkers live under ``oracle/``:

* ``build/libmhd_oracle.so`` -- the plain-C restatement ``mhd_oracle.c`` of
  ppkMHD's MUSCL-Hancock + HLLD + CT step (built by ``make -C oracle``);
* ``_ref/libppkmhd_ref{64,32}.so`` -- the reference's own functor sources
  compiled against the Kokkos-API shim (built by ``oracle/build_ref.sh``
  where the reference tree is present).

Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
import this module.  Arrays cross the boundary as numpy float64 arrays in the
layout of the library being called: the C oracle uses LayoutLeft
(``[var][k][j][i]``), the compiled reference uses LayoutRight
(``[i][j][k][var]``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "build", "libmhd_oracle.so")
REF_SO = {64: os.path.join(HERE, "_ref", "libppkmhd_ref64.so"),
          32: os.path.join(HERE, "_ref", "libppkmhd_ref32.so")}

_dp = ctypes.POINTER(ctypes.c_double)


class OrcParams(ctypes.Structure):
    """Mirror of ``orc_params`` in mhd_oracle.h."""

    _fields_ = [
        ("dim", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("ghost", ctypes.c_int), ("isize", ctypes.c_int), ("jsize", ctypes.c_int),
        ("ksize", ctypes.c_int),
        ("xmin", ctypes.c_double), ("xmax", ctypes.c_double), ("ymin", ctypes.c_double),
        ("ymax", ctypes.c_double), ("zmin", ctypes.c_double), ("zmax", ctypes.c_double),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
        ("gamma0", ctypes.c_double), ("cfl", ctypes.c_double), ("slope_type", ctypes.c_double),
        ("smallr", ctypes.c_double), ("smallc", ctypes.c_double), ("smallp", ctypes.c_double),
        ("cIso", ctypes.c_double),
        ("riemann", ctypes.c_int), ("version", ctypes.c_int), ("bc", ctypes.c_int * 6),
        ("tEnd", ctypes.c_double), ("tCurrent", ctypes.c_double), ("nStepmax", ctypes.c_int),
        ("ot_kt", ctypes.c_double), ("problem_is_ot", ctypes.c_int),
    ]


def build_oracle() -> None:
    """Compile the C restatement (gcc, seconds)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build_oracle()
        L = ctypes.CDLL(ORACLE_SO)
        L.orc_params_from_ini.argtypes = [ctypes.c_char_p, ctypes.POINTER(OrcParams)]
        L.orc_params_from_ini.restype = ctypes.c_int
        L.orc_create.argtypes = [ctypes.POINTER(OrcParams), ctypes.c_int]
        L.orc_create.restype = ctypes.c_void_p
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_set_state.argtypes = [ctypes.c_void_p, _dp]
        L.orc_get_state.argtypes = [ctypes.c_void_p, _dp]
        L.orc_run.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_run.restype = ctypes.c_int
        L.orc_time.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.POINTER(ctypes.c_int)]
        L.orc_set_dt_ulps.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_nelem.argtypes = [ctypes.POINTER(OrcParams)]
        L.orc_nelem.restype = ctypes.c_int64
        L.orc_init_orszag_tang.argtypes = [ctypes.POINTER(OrcParams), _dp]
        L.orc_make_boundaries.argtypes = [ctypes.POINTER(OrcParams), _dp]
        L.orc_riemann.argtypes = [ctypes.POINTER(OrcParams), _dp, _dp, _dp]
        L.orc_compute_emf.argtypes = [ctypes.POINTER(OrcParams), ctypes.c_int, _dp]
        L.orc_compute_emf.restype = ctypes.c_double
        L.mlp_nparams.restype = ctypes.c_int
        L.mlp_encode.argtypes = [_dp, _dp, ctypes.c_double, _dp, _dp]
        L.mlp_encode.restype = ctypes.c_double
        L.mlp_central_flux.argtypes = [_dp, _dp, ctypes.c_double, ctypes.c_double, _dp]
        L.mlp_forward_batch.argtypes = [_dp, _dp, ctypes.c_long, _dp, ctypes.c_int]
        L.mlp_loss_grad.argtypes = [_dp, _dp, _dp, ctypes.c_long, _dp]
        L.mlp_loss_grad.restype = ctypes.c_double
        L.mlp_bf16.argtypes = [ctypes.c_double]
        L.mlp_bf16.restype = ctypes.c_double
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def params_from_ini(ini_text: str) -> OrcParams:
    p = OrcParams()
    rc = lib().orc_params_from_ini(ini_text.encode(), ctypes.byref(p))
    if rc != 0:
        raise ValueError("oracle: unsupported solver_name in .ini")
    return p


def state_shape(p: OrcParams):
    """LayoutLeft numpy shape [var][k][j][i] (2D: [var][j][i])."""
    if p.dim == 2:
        return (8, p.jsize, p.isize)
    return (8, p.ksize, p.jsize, p.isize)


class OracleSolver:
    """The C restatement driven like the reference solver (ctor + main loop)."""

    def __init__(self, ini_text: str, nthreads: int = 1):
        self.p = params_from_ini(ini_text)
        self.h = lib().orc_create(ctypes.byref(self.p), int(nthreads))

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_state(self, U: np.ndarray):
        U = np.ascontiguousarray(U, dtype=np.float64)
        assert U.shape == state_shape(self.p)
        lib().orc_set_state(self.h, _ptr(U))

    def get_state(self) -> np.ndarray:
        U = np.empty(state_shape(self.p), dtype=np.float64)
        lib().orc_get_state(self.h, _ptr(U))
        return U

    def run(self, n: int) -> int:
        return lib().orc_run(self.h, int(n))

    def set_dt_ulps(self, ulps: int):
        """Test hook: move every later dt up by `ulps` ulps."""
        lib().orc_set_dt_ulps(self.h, int(ulps))

    def time(self):
        t, dt, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        lib().orc_time(self.h, ctypes.byref(t), ctypes.byref(dt), ctypes.byref(it))
        return t.value, dt.value, it.value


def orszag_tang(p: OrcParams) -> np.ndarray:
    U = np.zeros(state_shape(p), dtype=np.float64)
    lib().orc_init_orszag_tang(ctypes.byref(p), _ptr(U))
    return U


def riemann(p: OrcParams, qL, qR) -> np.ndarray:
    l = np.ascontiguousarray(qL, dtype=np.float64)
    r = np.ascontiguousarray(qR, dtype=np.float64)
    f = np.zeros(8)
    lib().orc_riemann(ctypes.byref(p), _ptr(l), _ptr(r), _ptr(f))
    return f


def compute_emf(p: OrcParams, emf_dir: int, q_edge) -> float:
    q = np.ascontiguousarray(q_edge, dtype=np.float64).reshape(4, 8)
    return float(lib().orc_compute_emf(ctypes.byref(p), int(emf_dir), _ptr(q)))


# ---------------------------------------------------------------- hydro solver

class HorcParams(ctypes.Structure):
    """Mirror of ``horc_params`` in hydro_oracle.h."""

    _fields_ = [
        ("dim", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("ghost", ctypes.c_int), ("nvar", ctypes.c_int),
        ("isize", ctypes.c_int), ("jsize", ctypes.c_int), ("ksize", ctypes.c_int),
        ("xmin", ctypes.c_double), ("xmax", ctypes.c_double), ("ymin", ctypes.c_double),
        ("ymax", ctypes.c_double), ("zmin", ctypes.c_double), ("zmax", ctypes.c_double),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
        ("gamma0", ctypes.c_double), ("gamma6", ctypes.c_double), ("cfl", ctypes.c_double),
        ("slope_type", ctypes.c_double), ("smallr", ctypes.c_double), ("smallc", ctypes.c_double),
        ("smallp", ctypes.c_double), ("smallpp", ctypes.c_double),
        ("riemann", ctypes.c_int), ("version", ctypes.c_int), ("bc", ctypes.c_int * 6),
        ("tEnd", ctypes.c_double), ("tCurrent", ctypes.c_double), ("nStepmax", ctypes.c_int),
        ("gravity", ctypes.c_int), ("grav", ctypes.c_double * 3),
        ("point", ctypes.c_int), ("xs", ctypes.c_double), ("ys", ctypes.c_double),
        ("zs", ctypes.c_double), ("GM", ctypes.c_double), ("eps", ctypes.c_double),
        ("xc", ctypes.c_double), ("yc", ctypes.c_double), ("zc", ctypes.c_double),
    ]


_hlib = None


def hlib():
    global _hlib
    if _hlib is None:
        L = lib()
        L.horc_params_from_ini.argtypes = [ctypes.c_char_p, ctypes.POINTER(HorcParams)]
        L.horc_params_from_ini.restype = ctypes.c_int
        L.horc_nelem.argtypes = [ctypes.POINTER(HorcParams)]
        L.horc_nelem.restype = ctypes.c_int64
        L.horc_create.argtypes = [ctypes.POINTER(HorcParams), ctypes.c_int]
        L.horc_create.restype = ctypes.c_void_p
        L.horc_destroy.argtypes = [ctypes.c_void_p]
        L.horc_set_state.argtypes = [ctypes.c_void_p, _dp]
        L.horc_get_state.argtypes = [ctypes.c_void_p, _dp]
        L.horc_run.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.horc_run.restype = ctypes.c_int
        L.horc_time.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.POINTER(ctypes.c_int)]
        L.horc_riemann.argtypes = [ctypes.POINTER(HorcParams), _dp, _dp, _dp]
        _hlib = L
    return _hlib


def hydro_params_from_ini(ini_text: str) -> HorcParams:
    p = HorcParams()
    if hlib().horc_params_from_ini(ini_text.encode(), ctypes.byref(p)) != 0:
        raise ValueError("hydro oracle: unsupported .ini (solver, version 2, 3D hll or point gravity)")
    return p


def hydro_state_shape(p: HorcParams):
    if p.dim == 2:
        return (p.nvar, p.jsize, p.isize)
    return (p.nvar, p.ksize, p.jsize, p.isize)


class HydroOracleSolver:
    """The C restatement of SolverHydroMuscl driven like the reference."""

    def __init__(self, ini_text: str, nthreads: int = 1):
        self.p = hydro_params_from_ini(ini_text)
        self.h = hlib().horc_create(ctypes.byref(self.p), int(nthreads))

    def close(self):
        if self.h:
            hlib().horc_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_state(self, U: np.ndarray):
        U = np.ascontiguousarray(U, dtype=np.float64)
        assert U.shape == hydro_state_shape(self.p)
        hlib().horc_set_state(self.h, _ptr(U))

    def get_state(self) -> np.ndarray:
        U = np.empty(hydro_state_shape(self.p), dtype=np.float64)
        hlib().horc_get_state(self.h, _ptr(U))
        return U

    def run(self, n: int) -> int:
        return hlib().horc_run(self.h, int(n))

    def time(self):
        t, dt, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        hlib().horc_time(self.h, ctypes.byref(t), ctypes.byref(dt), ctypes.byref(it))
        return t.value, dt.value, it.value


def hydro_gravity_field(ini_text: str) -> np.ndarray:
    """The oracle's gravity field for the .ini (dim planes, LayoutLeft)."""
    p = hydro_params_from_ini(ini_text)
    hlib().horc_gravity_field.argtypes = [ctypes.POINTER(HorcParams), _dp]
    shape = hydro_state_shape(p)
    g = np.zeros((p.dim,) + shape[1:], dtype=np.float64)
    hlib().horc_gravity_field(ctypes.byref(p), _ptr(g))
    return g


def ref_hydro_gravity_field(ini_text: str, bits: int = 64) -> np.ndarray:
    """The gravity field the reference's hydro init functor writes (dim
    planes, LayoutLeft float64; zeros for problems that write none)."""
    r = RefSolver(ini_text, bits)
    dim, shape = r.dim, r._right_shape()
    r.close()
    L = ctypes.CDLL(REF_SO[bits])
    L.ref_hydro_gravity_field.argtypes = [ctypes.c_char_p, ctypes.c_void_p]
    L.ref_hydro_gravity_field.restype = ctypes.c_long
    g = np.empty(shape[:-1] + (dim,), dtype=np.float64 if bits == 64 else np.float32)
    n = L.ref_hydro_gravity_field(ini_text.encode(), g.ctypes.data_as(ctypes.c_void_p))
    assert n == g.size
    return np.ascontiguousarray(g.T, dtype=np.float64)


def hydro_riemann(p: HorcParams, qL, qR) -> np.ndarray:
    l = np.ascontiguousarray(qL, dtype=np.float64)
    r = np.ascontiguousarray(qR, dtype=np.float64)
    f = np.zeros(p.nvar)
    hlib().horc_riemann(ctypes.byref(p), _ptr(l), _ptr(r), _ptr(f))
    return f


# ---------------------------------------------------------------- flux surrogate

MLP_NPARAM = 7832
MLP_NFEAT = 40


def mlp_encode(qL, qR, a: float):
    """(features[40], scale[7], J) of one face (mlp_oracle.c)."""
    l = np.ascontiguousarray(qL, dtype=np.float64)
    r = np.ascontiguousarray(qR, dtype=np.float64)
    f = np.zeros(MLP_NFEAT)
    sc = np.zeros(7)
    J = lib().mlp_encode(_ptr(l), _ptr(r), float(a), _ptr(f), _ptr(sc))
    return f, sc, J


def mlp_central_flux(qL, qR, a: float, gamma0: float):
    l = np.ascontiguousarray(qL, dtype=np.float64)
    r = np.ascontiguousarray(qR, dtype=np.float64)
    F = np.zeros(7)
    lib().mlp_central_flux(_ptr(l), _ptr(r), float(a), float(gamma0), _ptr(F))
    return F


def mlp_forward(params, X, rounding: bool = False):
    P = np.ascontiguousarray(params, dtype=np.float64)
    X = np.ascontiguousarray(X, dtype=np.float64)
    Y = np.zeros((X.shape[0], 8))
    lib().mlp_forward_batch(_ptr(P), _ptr(X), X.shape[0], _ptr(Y), int(rounding))
    return Y


def mlp_loss_grad(params, X, T):
    P = np.ascontiguousarray(params, dtype=np.float64)
    X = np.ascontiguousarray(X, dtype=np.float64)
    T = np.ascontiguousarray(T, dtype=np.float64)
    g = np.zeros(MLP_NPARAM)
    loss = lib().mlp_loss_grad(_ptr(P), _ptr(X), _ptr(T), X.shape[0], _ptr(g))
    return loss, g


# ---------------------------------------------------------------- reference

def ref_available(bits: int = 64) -> bool:
    return os.path.exists(REF_SO[bits])


def ref_save_vtk(ini_text: str, U_left: np.ndarray, istep: int, bits: int = 64) -> None:
    """The reference's own VTK writer (save_VTK_2D / save_VTK_3D of
    IO_VTK.cpp, compiled via the shim) on a LayoutLeft state; the file goes
    where the .ini's [output] section says."""
    L = ctypes.CDLL(REF_SO[bits])
    L.ref_save_vtk.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int]
    L.ref_save_vtk.restype = ctypes.c_int
    real = np.float64 if bits == 64 else np.float32
    UR = np.ascontiguousarray(np.asarray(U_left, dtype=real).T)  # LayoutRight (i,j[,k],var)
    if L.ref_save_vtk(ini_text.encode(), UR.ctypes.data_as(ctypes.c_void_p), int(istep)) != 0:
        raise ValueError("reference: unsupported solver_name")


class RefSolver:
    """The reference's own functors (compiled via the Kokkos-API shim)."""

    def __init__(self, ini_text: str, bits: int = 64):
        L = ctypes.CDLL(REF_SO[bits])
        self.real = np.float64 if bits == 64 else np.float32
        L.ref_create.argtypes = [ctypes.c_char_p]
        L.ref_create.restype = ctypes.c_void_p
        L.ref_destroy.argtypes = [ctypes.c_void_p]
        L.ref_sizes.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
        L.ref_get_state.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.ref_set_state.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.ref_run.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.ref_run.restype = ctypes.c_int
        L.ref_time.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.POINTER(ctypes.c_int)]
        self.L = L
        self.h = L.ref_create(ini_text.encode())
        if not self.h:
            raise ValueError("reference: unsupported solver_name")
        sz = (ctypes.c_int * 6)()
        L.ref_sizes(self.h, sz)
        self.isize, self.jsize, self.ksize, self.nbvar, self.dim, self.ghost = list(sz)

    def close(self):
        if self.h:
            self.L.ref_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _right_shape(self):
        if self.dim == 2:
            return (self.isize, self.jsize, self.nbvar)
        return (self.isize, self.jsize, self.ksize, self.nbvar)

    def get_state(self) -> np.ndarray:
        """Returned in LayoutLeft [var][k][j][i] (float64)."""
        U = np.empty(self._right_shape(), dtype=self.real)
        self.L.ref_get_state(self.h, U.ctypes.data_as(ctypes.c_void_p))
        return np.ascontiguousarray(U.T, dtype=np.float64)

    def set_state(self, U_left: np.ndarray):
        U = np.ascontiguousarray(np.asarray(U_left).T, dtype=self.real)
        assert U.shape == self._right_shape()
        self.L.ref_set_state(self.h, U.ctypes.data_as(ctypes.c_void_p))

    def run(self, n: int) -> int:
        return self.L.ref_run(self.h, int(n))

    def time(self):
        t, dt, it = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        self.L.ref_time(self.h, ctypes.byref(t), ctypes.byref(dt), ctypes.byref(it))
        return t.value, dt.value, it.value


def ref_initial_state(ini_text: str, bits: int = 64) -> np.ndarray:
    """The reference init functor's output for the .ini (no boundary fill),
    LayoutLeft float64."""
    r = RefSolver(ini_text, bits)
    shape = r._right_shape()
    r.close()
    L = ctypes.CDLL(REF_SO[bits])
    L.ref_initial_state.argtypes = [ctypes.c_char_p, ctypes.c_void_p]
    L.ref_initial_state.restype = ctypes.c_long
    U = np.empty(shape, dtype=np.float64 if bits == 64 else np.float32)
    n = L.ref_initial_state(ini_text.encode(), U.ctypes.data_as(ctypes.c_void_p))
    assert n == U.size
    return np.ascontiguousarray(U.T, dtype=np.float64)


def ref_probe_lib(bits: int = 64):
    L = ctypes.CDLL(REF_SO[bits])
    real = ctypes.c_double if bits == 64 else ctypes.c_float
    rp = ctypes.POINTER(real)
    L.ref_riemann.argtypes = [ctypes.c_char_p, rp, rp, rp]
    L.ref_compute_emf.argtypes = [ctypes.c_char_p, ctypes.c_int, rp]
    L.ref_compute_emf.restype = real
    L.ref_params.argtypes = [ctypes.c_char_p, _dp]
    L.ref_hydro_riemann.argtypes = [ctypes.c_char_p, rp, rp, rp]
    return L


def interior(U: np.ndarray, ghost: int = 3) -> np.ndarray:
    g = ghost
    if U.ndim == 3:
        return U[:, g:-g, g:-g]
    return U[:, g:-g, g:-g, g:-g]


def rel_l1(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Per-variable relative L1 error sum|a-b| / sum|b| over the interior."""
    ax = tuple(range(1, a.ndim))
    num = np.abs(a - b).sum(axis=ax)
    den = np.abs(b).sum(axis=ax)
    return num / np.where(den > 0, den, 1.0)
