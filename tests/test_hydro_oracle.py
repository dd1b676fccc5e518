"""The hydro-only MUSCL solver (SolverHydroMuscl<dim>) on the CPU: the C
restatement oracle/hydro_oracle.c and the library's host parts against the
reference.

The golden fixtures were produced by the reference's own hydro functors
(tests/golden/make_hydro_golden.py, through oracle/ref_harness_hydro.cpp):
the oracle must reproduce every iteration bit for bit, the library's host
initial conditions must equal the reference's init functors bit for bit, and
the library must parse and validate the hydro .ini keys as the reference
does.  Where the compiled reference (oracle/_ref) is present, the oracle is
also run against it directly on further seeded cases.  No GPU is used.
"""
import glob
import os

import numpy as np
import pytest

from mhd_cases import hydro_ini, hydro_perturbed

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = sorted(glob.glob(os.path.join(GOLDEN, "hydro_*.npz")))
CASES = [p for p in CASES if not p.endswith("hydro_riemann.npz")]
IDS = [os.path.basename(p)[6:-4] for p in CASES]


def interior(U, g=2):
    return U[:, g:-g, g:-g] if U.ndim == 3 else U[:, g:-g, g:-g, g:-g]


@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_hydro_oracle_matches_reference(oracle, path):
    z = np.load(path)
    s = oracle.HydroOracleSolver(str(z["ini"]))
    s.set_state(z["U0"])
    assert s.time()[:2] == (z["t"][0], z["dt"][0])
    s.run(1)
    assert np.array_equal(interior(s.get_state()), z["U1"])
    s.run(int(z["nsteps"]) - 1)
    assert np.array_equal(interior(s.get_state()), z["Un"])
    t, dt, it = s.time()
    assert (t, dt, it) == (z["t"][2], z["dt"][2], int(z["nsteps"]))


@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_hydro_oracle_gravity_field_matches_reference(oracle, path):
    """The gravity field the init functors write (uniform for Rayleigh-Taylor
    and the rising bubble, the softened point source around the disk centre,
    zero otherwise)."""
    z = np.load(path)
    assert np.array_equal(oracle.hydro_gravity_field(str(z["ini"])), z["gravity"])


@pytest.mark.parametrize("path", [p for p in CASES if not np.load(p)["perturbed"]],
                         ids=[i for p, i in zip(CASES, IDS) if not np.load(p)["perturbed"]])
def test_hydro_host_initial_state_matches_reference(mhdlib, path):
    """mhd_initial_state of a hydro .ini = the reference's init functor output."""
    z = np.load(path)
    U = mhdlib.initial_state(mhdlib.params_from_ini(str(z["ini"])))
    assert np.array_equal(U, z["U0"])


@pytest.mark.parametrize("dim,solver", [(2, "approx"), (2, "llf"), (2, "hll"), (2, "hllc"),
                                        (3, "approx"), (3, "llf"), (3, "hllc")])
def test_hydro_riemann_known_answers(oracle, dim, solver):
    z = np.load(os.path.join(GOLDEN, "hydro_riemann.npz"))
    p = oracle.hydro_params_from_ini(hydro_ini(dim=dim, nx=8, riemann=solver))
    F = np.array([oracle.hydro_riemann(p, l, r) for l, r in zip(z[f"qL{dim}"], z[f"qR{dim}"])])
    assert np.array_equal(F, z[f"{solver}{dim}"])


def test_hydro_versions_0_and_1_agree_without_gravity():
    """The version-1 fixture equals the version-0 one bit for bit: both
    versions compute the same fluxes and additions in the same order."""
    a = np.load(os.path.join(GOLDEN, "hydro_implode2d.npz"))
    b = np.load(os.path.join(GOLDEN, "hydro_implode2d_v1.npz"))
    assert np.array_equal(a["Un"], b["Un"]) and np.array_equal(a["dt"], b["dt"])


def test_hydro_3d_version_1_gravity_quirk():
    """In 3D with gravity, version 1 omits the predictor on the right state of
    z faces (HydroRunFunctors3D.h:1344-1346): the two versions differ."""
    a = np.load(os.path.join(GOLDEN, "hydro_rb3d_gravity_v0.npz"))
    b = np.load(os.path.join(GOLDEN, "hydro_rb3d_gravity_v1.npz"))
    assert np.array_equal(a["U0"], b["U0"])
    assert not np.array_equal(a["Un"], b["Un"])


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref",
                                                    "libppkmhd_ref64.so")),
                    reason="compiled reference (oracle/_ref) not built here")
@pytest.mark.parametrize("dim,kw", [
    (2, dict(riemann="hllc", bc=(2, 1, 3, 3), version=1)),
    (2, dict(riemann="approx", slope_type="1", gravity=True, problem="rising_bubble")),
    (3, dict(riemann="approx", bc=(3, 3, 1, 2, 2, 1))),
    (3, dict(riemann="hllc", gravity=True, problem="rayleigh_taylor", version=1)),
])
def test_hydro_oracle_against_compiled_reference(oracle, dim, kw):
    ini = hydro_ini(dim=dim, nx=20 if dim == 2 else 9, **kw)
    U0 = hydro_perturbed(oracle.ref_initial_state(ini), 90 + dim)
    r = oracle.RefSolver(ini)
    s = oracle.HydroOracleSolver(ini)
    r.set_state(U0)
    s.set_state(U0)
    for _ in range(6):
        r.run(1)
        s.run(1)
        assert np.array_equal(r.get_state(), s.get_state())
        assert r.time() == s.time()
    r.close()
    s.close()


def test_hydro_params_parse_like_reference(mhdlib):
    ini = hydro_ini(dim=3, nx=12, riemann="hllc", gamma0="1.666", cfl="0.7", version=1,
                    bc=(1, 2, 3, 1, 2, 3), problem="rising_bubble", gravity=True,
                    extra="[rising_bubble]\ngz=-0.3\n")
    p = mhdlib.params_from_ini(ini)
    assert p.solver == mhdlib.MHD_SOLVER_HYDRO_MUSCL and p.dim == 3 and p.ghost == 2
    assert p.nvar == 5 and p.riemann == mhdlib.MHD_RIEMANN_HLLC and p.implementation_version == 1
    assert p.gamma0 == float(np.float32(1.666)) and p.cfl == float(np.float32(0.7))
    assert list(p.boundary) == [1, 2, 3, 1, 2, 3]
    assert p.problem == mhdlib.MHD_PROBLEM_RISING_BUBBLE and p.gravity == 1
    assert list(p.gravity_field) == [0.0, float(np.float32(-0.1)), float(np.float32(-0.3))]
    # names of 2D problems run implode in 3D, as the reference's dispatch does
    assert mhdlib.params_from_ini(hydro_ini(dim=3, problem="four_quadrant")).problem == \
        mhdlib.MHD_PROBLEM_IMPLODE
    assert mhdlib.params_from_ini(hydro_ini(dim=2, problem="orszag_tang")).problem == \
        mhdlib.MHD_PROBLEM_IMPLODE


@pytest.mark.parametrize("kw,extra,why", [
    (dict(dim=3, riemann="hll"), "", "no hll"),
    (dict(dim=2, riemann="hlld"), "", "approx, llf, hll or hllc"),
    (dict(dim=2, version=2), "", "0 or 1"),
    (dict(dim=2, problem="rayleigh_taylor"), "", "[gravity] static"),
    (dict(dim=2, problem="disk"), "", "point=true"),
    (dict(dim=2, slope_type="3"), "", "slope_type"),
    (dict(dim=2, problem="kelvin_helmholtz"), "[KH]\nperturbation_sine_robertson=false\n",
     "robertson"),
    (dict(dim=2, problem="kelvin_helmholtz"), "[KH]\nperturbation_rand=true\n", "rand"),
])
def test_hydro_create_rejects_unsupported(mhdlib, kw, extra, why):
    """Validation runs before any device is touched (no GPU here)."""
    p = mhdlib.params_from_ini(hydro_ini(**kw) + extra)
    with pytest.raises(mhdlib.MHDError) as e:
        mhdlib.MHDSolver(p)
    assert e.value.code == mhdlib.MHD_ERR_INVALID_ARG
    assert why in str(e.value)


def test_hydro_ensembles_and_noalloc_refuse_hydro(mhdlib):
    import ctypes

    p = mhdlib.params_from_ini(hydro_ini(dim=2, nx=16))
    with pytest.raises(mhdlib.MHDError):
        mhdlib.MHDEnsemble([p])
    dt = ctypes.c_double(0)
    rc = mhdlib.lib().mhd_step_noalloc(ctypes.byref(p), ctypes.c_void_p(16), ctypes.c_void_p(32),
                                       0.0, ctypes.byref(dt), None)
    assert rc == mhdlib.MHD_ERR_INVALID_ARG
