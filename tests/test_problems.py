"""Initial conditions of the other problems of SolverMHDMuscl<dim>::init
(blast, implode, Kelvin-Helmholtz, rotor, field loop, linear wave; unknown
names fall back to Orszag-Tang) against fixtures made by the reference's own
init functors (tests/golden/make_golden.py): the host initial state bitwise
on the CPU; on the GPU the boundary-filled state and the state after n steps
of the FMA-free FP64 build bitwise, the fast FP64 build within 1e-12."""
import glob
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(os.path.basename(p)[len("problem_"):-4]
               for p in glob.glob(os.path.join(GOLDEN, "problem_*.npz")))


def load(name):
    return np.load(os.path.join(GOLDEN, f"problem_{name}.npz"))


def test_cases_present():
    assert {"rotor2d", "blast2d", "implode2d", "field_loop2d", "kh2d", "blast3d", "rotor3d",
            "field_loop3d", "kh3d", "wave3d_fast", "wave3d_alfven"} <= set(CASES)


@pytest.mark.parametrize("name", CASES)
def test_initial_state_bitwise(mhdlib, name):
    z = load(name)
    p = mhdlib.params_from_ini(str(z["ini"]))
    U = mhdlib.initial_state(p)
    assert U.shape == z["Uinit"].shape
    diff = np.argwhere(U != z["Uinit"])
    assert diff.size == 0, (name, diff[:5], U[tuple(diff[0])], z["Uinit"][tuple(diff[0])])


def test_problem_validation(mhdlib):
    from mhd_cases import ot_ini

    base = ot_ini(dim=2, nx=16).replace("problem=orszag_tang", "problem=kelvin_helmholtz")
    bad = base + "\n[KH]\nperturbation_rand=1\n"
    p = mhdlib.params_from_ini(bad)
    with pytest.raises(mhdlib.MHDError):
        mhdlib.initial_state(p)
    none = base + "\n[KH]\nperturbation_sine_robertson=0\n"
    with pytest.raises(mhdlib.MHDError):
        mhdlib.initial_state(mhdlib.params_from_ini(none))


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_problem_steps_bitwise(mhdlib, name):
    z = load(name)
    s = mhdlib.MHDSolver.from_ini(str(z["ini"]), fp_mode=mhdlib.MHD_FP_EXACT)
    s.init_problem()
    assert np.array_equal(s.get_state(), z["U0"]), name
    assert s.run(int(z["nsteps"])) == int(z["nsteps"])
    assert np.array_equal(mhdlib.interior(s.get_state()), z["Un"]), name
    assert s.time()[0] == z["t"][1]
    if name == "rotor3d":
        return  # at the edge of the reference's own NaN (see the fixture note): exact build only
    f = mhdlib.MHDSolver.from_ini(str(z["ini"]), fp_mode=mhdlib.MHD_FP_FAST)
    f.init_problem()
    f.run(int(z["nsteps"]))
    a, b = mhdlib.interior(f.get_state()), z["Un"]
    ax = tuple(range(1, a.ndim))
    # each variable against its own L1 norm, or the density's where the
    # variable is a small perturbation (the waves' momenta are ~1e-6)
    den = np.maximum(np.abs(b).sum(axis=ax), np.abs(b[0]).sum())
    assert (np.abs(a - b).sum(axis=ax) / den).max() <= 1e-12, name


def wave_ini(nx, wave_type, tend, version=2):
    """The reference's convergence-test setup (test/convergence/
    mhd_wave_3D.ini.skel with NY = NZ = NX / 2)."""
    return "\n".join([
        "[run]", "solver_name=MHD_Muscl_3D", f"tEnd={tend}", "nStepmax=100000", "nOutput=0",
        "[mesh]", f"nx={nx}", f"ny={nx // 2}", f"nz={nx // 2}", "xmax=3.0", "ymax=1.5",
        "zmax=1.5"] + [f"boundary_type_{f}=3" for f in ("xmin", "xmax", "ymin", "ymax", "zmin",
                                                       "zmax")] + [
        "[hydro]", "gamma0=1.6666666667", "cfl=0.4", "niter_riemann=10", "iorder=2",
        "slope_type=2", "problem=wave", "riemann=hlld", "smallr=1e-8", "smallc=1e-8",
        "[wave]", f"type={wave_type}", "[OTHER]", f"implementationVersion={version}"]) + "\n"


def _wave_errors(mhdlib, wave_type, tend, version, sizes):
    errs = []
    for nx in sizes:
        s = mhdlib.MHDSolver.from_ini(wave_ini(nx, wave_type, tend, version=version))
        s.init_problem()
        U0 = mhdlib.interior(s.get_state())
        s.run(100000)
        t, _, _ = s.time()
        assert abs(t - float(tend)) < 1e-9
        U1 = mhdlib.interior(s.get_state())
        # error of the perturbed quantities (amplitude 1e-6): all conserved variables
        errs.append(np.abs(U1 - U0).mean())
        s.close()
    return errs, np.log2(np.array(errs[:-1]) / np.array(errs[1:]))


@pytest.mark.gpu
@pytest.mark.parametrize("wave_type,tend", [(0, "0.5"), (1, "1.0")])
def test_linear_wave_convergence_second_order(mhdlib, wave_type, tend):
    """The reference's convergence test (test/convergence/mhd_wave_3D.ini.skel:
    implementationVersion=0, NY = NZ = NX / 2, one period of a linear fast /
    Alfven wave; its plot draws a second-order slope): the L1 error against
    the initial state falls at second order.  Measured with the reference
    itself (compiled here) at N = 16, 32, 64: orders 2.46, 1.81 (fast) and
    2.52, 2.13 (Alfven); the library is bitwise that path (version-0 wave
    fixtures).  The finest pair must reach order 1.8."""
    errs, orders = _wave_errors(mhdlib, wave_type, tend, 0, (16, 32, 64, 128))
    print(f"\nversion 0 wave type {wave_type}: L1 errors {errs}, orders {orders}")
    assert np.all(orders > 1.5), (errs, orders)
    assert orders[-1] >= 1.8, (errs, orders)


@pytest.mark.gpu
@pytest.mark.parametrize("wave_type,tend", [(0, "0.5"), (1, "1.0")])
def test_linear_wave_convergence_version2_first_order(mhdlib, wave_type, tend):
    """The same waves through implementation version 2 converge at first
    order in 3D, in the reference as here (the library is bitwise the
    reference on this path): its edge reconstruction takes the face-centred
    field's z slope with the minus sample at k + 1 (compute_limited_slope,
    MHDBaseFunctor3D.h:142), so Bx and By are piecewise constant along z on x
    and y edges, and y / x edges add transverse slopes twice
    (MHDRunFunctors3D.h:1490-1524).  Orders 1.50, 1.16, 1.02, 1.00 (fast) from
    N = 16 to 256; the reference's C restatement gives the same errors.  The
    test holds the errors to falling at first order at least."""
    errs, orders = _wave_errors(mhdlib, wave_type, tend, 2, (16, 32, 64, 128))
    print(f"\nversion 2 wave type {wave_type}: L1 errors {errs}, orders {orders}")
    assert np.all(orders > 0.9), (errs, orders)


@pytest.mark.gpu
def test_non_finite_reference_state_is_reported(mhdlib, oracle):
    """The reference's 3D rotor at 12x12x6 turns NaN from its third step
    (the oracle, bitwise the reference, shows it); the library stops with
    MHD_ERR_NUMERIC instead of carrying NaN on."""
    z = load("rotor3d")
    ini = str(z["ini"])
    o = oracle.OracleSolver(ini)
    o.set_state(z["U0"])
    o.run(4)
    assert np.isnan(o.get_state()).any()
    s = mhdlib.MHDSolver.from_ini(ini, fp_mode=mhdlib.MHD_FP_EXACT)
    s.init_problem()
    with pytest.raises(mhdlib.MHDError) as e:
        s.run(4)
    assert e.value.code == mhdlib.MHD_ERR_NUMERIC
