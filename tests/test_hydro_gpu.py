"""The hydro-only MUSCL solver on the GPU against the reference and the
oracle (SolverHydroMuscl<dim>, Hydro_Muscl_2D/3D, through the C ABI).

* FMA-free FP64 build (MHD_FP_EXACT): bitwise equal to the reference's own
  functors on every golden fixture (tests/golden/hydro_*.npz: 2D/3D,
  approx/LLF/HLL/HLLC, versions 0 and 1, slope types 0/1/2, periodic,
  reflecting, outflow and mixed walls, static gravity, all problems), and to
  the C oracle on larger seeded cases.
* Fast FP64 build: within 1e-11 of the oracle (relative L1 per variable).
* FP32 build: within 2e-4 of the oracle after 20 iterations (momenta
  relative to the acoustic momentum scale sum(rho c) where that is larger).
* The fused form (one tile kernel per iteration, intermediates in shared
  memory) and the stage kernels give the same state bit for bit in the
  FMA-free build (and within round-off in the FMA builds, which contract
  each kernel's expressions independently), on tiles cut by the domain edge
  too.
* CUDA-graph runs, single steps and host-array steps agree bit for bit;
  checkpoints restart bitwise; periodic runs conserve mass and energy to
  round-off at 1024^2.
"""
import glob
import os

import numpy as np
import pytest

from mhd_cases import hydro_ini, hydro_perturbed

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = sorted(p for p in glob.glob(os.path.join(GOLDEN, "hydro_*.npz"))
               if not p.endswith("hydro_riemann.npz"))
IDS = [os.path.basename(p)[6:-4] for p in CASES]


def interior(U, g=2):
    return U[:, g:-g, g:-g] if U.ndim == 3 else U[:, g:-g, g:-g, g:-g]


def rel_l1(a, b, gamma0=1.4):
    """Per-variable L1 error relative to the variable's own L1 norm; the
    momenta are measured against the acoustic momentum scale sum(rho c)
    when that is larger (a near-static state, e.g. a stratified atmosphere
    in hydrostatic balance, has momenta far below rho c)."""
    ax = tuple(range(1, a.ndim))
    num = np.abs(a - b).sum(axis=ax)
    den = np.abs(b).sum(axis=ax)
    rho_c = np.sqrt(gamma0 * (gamma0 - 1) * np.abs(b[0] * b[1])).sum()
    den[2:] = np.maximum(den[2:], rho_c)
    return num / np.maximum(den, 1e-300)


@pytest.mark.parametrize("fused", [True, False], ids=["fused", "stages"])
@pytest.mark.parametrize("path", CASES, ids=IDS)
def test_hydro_exact_build_matches_reference_bitwise(mhdlib, path, fused):
    m = mhdlib
    z = np.load(path)
    s = m.MHDSolver.from_ini(str(z["ini"]), precision=64, fp_mode=m.MHD_FP_EXACT)
    s.set_fused(fused)
    assert s.fused == fused
    if bool(z["perturbed"]):
        s.set_state(z["U0"])
    else:
        s.init_problem()
    assert s.time()[:2] == (z["t"][0], z["dt"][0])
    s.run(1)
    assert np.array_equal(interior(s.get_state()), z["U1"])
    s.run(int(z["nsteps"]) - 1)
    assert np.array_equal(interior(s.get_state()), z["Un"])
    t, dt, it = s.time()
    assert (t, dt, it) == (z["t"][2], z["dt"][2], int(z["nsteps"]))
    s.close()


ORACLE_CASES = [
    ("2d_approx_v0", dict(dim=2, nx=96, ny=80, bc=(1, 2, 3, 3)), 20),
    ("2d_hllc_v1_gravity", dict(dim=2, nx=64, ny=72, riemann="hllc", version=1, gravity=True,
                                problem="rayleigh_taylor", bc=(3, 3, 1, 1)), 20),
    ("2d_llf_slope1", dict(dim=2, nx=70, ny=64, riemann="llf", slope_type="1"), 20),
    ("2d_hll_fourquad", dict(dim=2, nx=64, riemann="hll", problem="four_quadrant",
                             bc=(2, 2, 2, 2)), 20),
    ("3d_approx_v0", dict(dim=3, nx=24, ny=20, nz=22, bc=(3, 3, 1, 2, 2, 1)), 6),
    ("3d_hllc_v1_gravity", dict(dim=3, nx=20, riemann="hllc", version=1, gravity=True,
                                problem="rising_bubble", bc=(2, 2, 1, 1, 2, 2)), 6),
    ("3d_llf_blast", dict(dim=3, nx=22, riemann="llf", problem="blast"), 6),
    ("2d_disk_point_gravity", dict(dim=2, nx=64, ny=64, problem="disk", bc=(2, 2, 2, 2),
                                   mesh="xmin=-0.5\nxmax=0.5\nymin=-0.5\nymax=0.5",
                                   extra="[gravity]\npoint=true\n"), 20),
    ("3d_disk_point_gravity_v1", dict(dim=3, nx=24, ny=20, nz=16, problem="disk", version=1,
                                      riemann="hllc", bc=(2, 2, 2, 2, 2, 2),
                                      mesh="xmin=-0.5\nxmax=0.5\nymin=-0.5\nymax=0.5\n"
                                           "zmin=-0.5\nzmax=0.5",
                                      extra="[gravity]\npoint=true\n"), 6),
]


def _oracle_run(oracle, ini, U0, n):
    s = oracle.HydroOracleSolver(ini, nthreads=8)
    s.set_state(U0)
    s.run(n)
    out = s.get_state(), s.time()
    s.close()
    return out


@pytest.mark.parametrize("name,kw,n", ORACLE_CASES, ids=[c[0] for c in ORACLE_CASES])
def test_hydro_builds_against_oracle(mhdlib, oracle, name, kw, n):
    """Exact build bitwise, fast FP64 to 1e-11, FP32 to 2e-4 (relative L1 per
    variable) against the C oracle on a seeded perturbed state."""
    m = mhdlib
    ini = hydro_ini(**kw)
    U0 = m.initial_state(m.params_from_ini(ini))
    if kw.get("problem") != "disk":
        # (the disk's 1e-6 density floor outside the disk leaves no room for
        # the momentum perturbation)
        U0 = hydro_perturbed(U0, 7)
    ref, (t, dt, it) = _oracle_run(oracle, ini, U0, n)
    for prec, mode, tol in ((64, m.MHD_FP_EXACT, 0.0), (64, m.MHD_FP_FAST, 1e-11),
                            (32, m.MHD_FP_FAST, 2e-4)):
        s = m.MHDSolver.from_ini(ini, precision=prec, fp_mode=mode)
        s.set_state(U0.astype(np.float64 if prec == 64 else np.float32))
        s.run(n)
        got = s.get_state().astype(np.float64)
        ts = s.time()
        s.close()
        if tol == 0.0:
            assert np.array_equal(interior(got), interior(ref))
            assert ts == (t, dt, it)
        else:
            err = rel_l1(interior(got), interior(ref))
            assert err.max() <= tol, (prec, mode, err)
            assert ts[2] == it


def test_hydro_graph_step_and_host_steps_agree(mhdlib):
    m = mhdlib
    ini = hydro_ini(dim=2, nx=40, ny=36, riemann="hllc", bc=(1, 2, 3, 3))
    U0 = hydro_perturbed(m.initial_state(m.params_from_ini(ini)), 3)
    a = m.MHDSolver.from_ini(ini)
    a.set_state(U0)
    a.run(5)
    b = m.MHDSolver.from_ini(ini)
    b.set_state(U0)
    for _ in range(5):
        b.step()
    assert np.array_equal(a.get_state(), b.get_state())
    assert a.time() == b.time()
    # godunov_unsplit_impl on host arrays, both layouts
    c = m.MHDSolver.from_ini(ini)
    c.set_state(U0)
    U = U0.copy()
    for q in range(5):
        out = np.empty_like(U)
        if q % 2:
            c._check(m.lib().mhd_step_host(c.h, np.ascontiguousarray(U).ctypes.data,
                                           out.ctypes.data, m.MHD_LAYOUT_LEFT, 8))
            U = out
        else:
            UR = np.ascontiguousarray(U.T)
            outR = np.empty_like(UR)
            c._check(m.lib().mhd_step_host(c.h, UR.ctypes.data, outR.ctypes.data,
                                           m.MHD_LAYOUT_RIGHT, 8))
            U = np.ascontiguousarray(outR.T)
    assert np.array_equal(interior(U), interior(a.get_state()))
    for s in (a, b, c):
        s.close()


def test_hydro_compute_dt_and_step_dt(mhdlib):
    m = mhdlib
    ini = hydro_ini(dim=3, nx=16, riemann="approx")
    a = m.MHDSolver.from_ini(ini, fp_mode=m.MHD_FP_EXACT)
    a.init_problem()
    b = m.MHDSolver.from_ini(ini, fp_mode=m.MHD_FP_EXACT)
    b.init_problem()
    for _ in range(3):
        dt = b.compute_dt()
        b.step_dt(dt)
        a.step()
    assert np.array_equal(a.get_state(), b.get_state())
    assert a.time() == b.time()
    a.close()
    b.close()


def test_hydro_checkpoint_restart_is_bitwise(mhdlib, tmp_path):
    m = mhdlib
    ini = hydro_ini(dim=2, nx=48, problem="kelvin_helmholtz", riemann="hllc")
    a = m.MHDSolver.from_ini(ini)
    a.init_problem()
    a.run(4)
    path = str(tmp_path / "h.ckpt")
    a.checkpoint_save(path)
    a.run(6)
    b = m.MHDSolver.from_ini(ini)
    b.checkpoint_load(path)
    b.run(6)
    assert np.array_equal(interior(a.get_state()), interior(b.get_state()))
    assert a.time()[0] == b.time()[0]
    a.close()
    b.close()


def test_hydro_periodic_conservation_full_size(mhdlib):
    """Mass, energy and momentum totals of a periodic 1024^2 run: the flux
    form conserves them to round-off (size-independent property).  The totals
    are exactly rounded sums (math.fsum), so the check sees the scheme's
    round-off, not the summation's."""
    import math

    m = mhdlib
    ini = hydro_ini(dim=2, nx=1024, ny=1024, problem="kelvin_helmholtz", riemann="hllc")
    s = m.MHDSolver.from_ini(ini)
    s.init_problem()

    def totals():
        U = interior(s.get_state())
        return [math.fsum(U[v].ravel()) for v in range(4)]

    before = totals()
    s.run(50)
    after = totals()
    for v in range(4):
        # relative 1e-12 of the total, and 1e-9 absolute for totals near zero
        # (the x momentum of the two counter-flowing layers)
        assert abs(after[v] - before[v]) <= 1e-12 * abs(before[v]) + 1e-9, (v, before[v], after[v])
    s.close()


def test_hydro_numeric_status_on_bad_state(mhdlib):
    m = mhdlib
    ini = hydro_ini(dim=2, nx=16)
    s = m.MHDSolver.from_ini(ini)
    U = m.initial_state(m.params_from_ini(ini))
    U[0, 8, 8] = -1.0
    with pytest.raises(m.MHDError) as e:
        s.set_state(U)
        s.run(1)
    assert e.value.code == m.MHD_ERR_NUMERIC
    s.close()


FUSED_CASES = [
    # partial tiles along every axis (the tile is 32 x 16 in 2D, 16 x 8 x 4 /
    # 8 x 8 x 4 in 3D), every build, gravity, both versions, all solvers
    ("2d_partial", dict(dim=2, nx=77, ny=41, riemann="hllc", bc=(1, 2, 3, 3))),
    ("2d_gravity_v1", dict(dim=2, nx=40, ny=35, riemann="approx", gravity=True, version=1,
                           problem="rayleigh_taylor", bc=(3, 3, 1, 1))),
    ("2d_hll_slope1", dict(dim=2, nx=33, ny=17, riemann="hll", slope_type="1")),
    ("3d_partial", dict(dim=3, nx=19, ny=13, nz=7, riemann="approx", bc=(1, 2, 3, 3, 2, 1))),
    ("3d_gravity_v1", dict(dim=3, nx=17, ny=9, nz=10, riemann="llf", gravity=True, version=1,
                           problem="rising_bubble", bc=(2, 2, 1, 1, 2, 2))),
    ("3d_slope0", dict(dim=3, nx=16, ny=16, nz=8, riemann="hllc", slope_type="0")),
]


@pytest.mark.parametrize("prec,mode", [(64, 1), (64, 0), (32, 0)], ids=["exact", "fast", "fp32"])
@pytest.mark.parametrize("name,kw", FUSED_CASES, ids=[c[0] for c in FUSED_CASES])
def test_hydro_fused_form_equals_stage_form(mhdlib, name, kw, prec, mode):
    m = mhdlib
    ini = hydro_ini(**kw)
    U0 = hydro_perturbed(m.initial_state(m.params_from_ini(ini)), 5)
    out = []
    for fused in (True, False, None, "timed"):
        s = m.MHDSolver.from_ini(ini, precision=prec, fp_mode=mode)
        if fused is not None:
            s.set_fused(fused)
        else:
            # the configuration's default form: fused for 2D FP32
            assert s.fused == (kw["dim"] == 2 and prec == 32)
        s.set_state(U0.astype(s.real))
        s.run(6)  # "timed": the first run times both forms on a snapshot and keeps the faster
        out.append((s.get_state(), s.time()))
        s.close()
    for q in (1, 2, 3):
        if mode == m.MHD_FP_EXACT:
            # no contraction: the same operations in the same order
            assert np.array_equal(out[0][0], out[q][0])
            assert out[0][1] == out[q][1]
        else:
            # the FMA builds contract the same expressions independently in
            # each kernel: round-off level differences
            tol = 1e-13 if prec == 64 else 1e-5
            a, b = out[0][0].astype(np.float64), out[q][0].astype(np.float64)
            assert rel_l1(interior(a), interior(b)).max() <= tol
            assert out[0][1][2] == out[q][1][2]


def test_form_requests(mhdlib):
    """The 3D MHD solver has the stage form only; form values outside
    stages / fused / timed are refused."""
    m = mhdlib
    from mhd_cases import ot_ini

    s = m.MHDSolver.from_ini(ot_ini(dim=3, nx=8))
    assert not s.fused
    s.set_fused(False)
    with pytest.raises(m.MHDError):
        s.set_fused(True)
    s.set_fused("timed")
    s.init_problem()
    s.run(1)
    assert not s.fused
    s.close()
    h = m.MHDSolver.from_ini(hydro_ini(dim=2, nx=16))
    for bad in (3, -1):
        with pytest.raises(m.MHDError):
            h._check(m.lib().mhd_set_fused(h.h, bad))
    h.close()
