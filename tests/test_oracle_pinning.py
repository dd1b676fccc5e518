"""The CPU oracle (oracle/mhd_oracle.c) against the reference.

The golden fixtures were produced by the reference's own functors
(tests/golden/make_golden.py); the oracle must reproduce them bit for bit.
When the compiled reference (oracle/_ref) is present, the oracle is also
compared with it directly on further cases.
"""
import glob
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
STEP_FILES = sorted(glob.glob(os.path.join(GOLDEN, "steps_*.npz")))


V2_STEP_FILES = [p for p in STEP_FILES if not os.path.basename(p).startswith(("steps_v0_", "steps_v1_"))]


@pytest.mark.parametrize("path", V2_STEP_FILES,
                         ids=[os.path.basename(p)[6:-4] for p in V2_STEP_FILES])
def test_oracle_matches_reference_steps(oracle, path):
    """The C restatement covers implementation version 2; the version 0/1
    fixtures pin the GPU's FMA-free build directly (tests/test_gpu_parity.py)."""
    z = np.load(path)
    ini = str(z["ini"])
    s = oracle.OracleSolver(ini)
    if bool(z["perturbed"]):
        s.set_state(z["U0"])
    else:
        # the oracle's own initial condition must equal the reference's
        U0 = s.get_state()
        assert np.array_equal(U0, z["U0"])
    t0, dt0, _ = s.time()
    assert (t0, dt0) == (z["t"][0], z["dt"][0])
    s.run(1)
    assert np.array_equal(oracle.interior(s.get_state()), z["U1"])
    s.run(int(z["nsteps"]) - 1)
    assert np.array_equal(oracle.interior(s.get_state()), z["Un"])
    t, dt, it = s.time()
    assert (t, dt, it) == (z["t"][2], z["dt"][2], int(z["nsteps"]))


@pytest.mark.parametrize("solver", ["hlld", "hll", "llf"])
def test_oracle_riemann_kat(oracle, solver):
    z = np.load(os.path.join(GOLDEN, "riemann.npz"))
    from mhd_cases import ot_ini

    p = oracle.params_from_ini(ot_ini(dim=2, nx=8, riemann=solver))
    F = np.array([oracle.riemann(p, l, r) for l, r in zip(z["qL"], z["qR"])])
    assert np.array_equal(F, z[solver])


def test_oracle_emf_kat(oracle):
    z = np.load(os.path.join(GOLDEN, "emf.npz"))
    p = oracle.params_from_ini(str(z["ini"]))
    E = np.array([[oracle.compute_emf(p, d, q) for d in range(3)] for q in z["qEdge"]])
    assert np.array_equal(E, z["emf"])


def test_oracle_params_match_reference(oracle):
    z = np.load(os.path.join(GOLDEN, "params.npz"))
    for name, ini, ref in zip(z["names"], z["inis"], z["values"]):
        p = oracle.params_from_ini(str(ini))
        got = [p.gamma0, p.cfl, p.slope_type, p.smallr, p.smallc, p.smallp, p.dx, p.dy, p.dz,
               p.tEnd]
        # dz of a 2D run is (zmax - zmin) / nz with nz defaulting to 1
        assert np.array_equal(np.array(got), ref), name


def test_oracle_float_rounded_parameters(oracle):
    """ConfigMap::getFloat goes through strtof: gamma0=5/3 is float-rounded."""
    from mhd_cases import ot_ini

    p = oracle.params_from_ini(ot_ini(gamma0="1.6666666666666667"))
    assert p.gamma0 == float(np.float32(5.0 / 3.0))
    assert p.cfl == float(np.float32(0.8))


@pytest.mark.skipif(not os.path.exists(os.path.join(os.path.dirname(__file__), "..", "oracle",
                                                    "_ref", "libppkmhd_ref64.so")),
                    reason="compiled reference (oracle/_ref) not present on this machine")
@pytest.mark.parametrize("dim,kw", [
    (2, dict(nx=13, ny=7)), (2, dict(nx=9, ny=17, riemann="llf", bc=(2, 2, 1, 1, 3, 3))),
    (3, dict(nx=7, ny=5, nz=6)), (3, dict(nx=6, ny=7, nz=5, riemann="hll", bc=(3, 3, 1, 2, 2, 1))),
])
def test_oracle_matches_compiled_reference_live(oracle, dim, kw):
    from mhd_cases import ot_ini, perturb

    ini = ot_ini(dim=dim, **kw)
    o = oracle.OracleSolver(ini)
    r = oracle.RefSolver(ini)
    U = perturb(o.get_state(), 5)
    o.set_state(U)
    r.set_state(U)
    o.run(6)
    r.run(6)
    assert np.array_equal(oracle.interior(o.get_state()), oracle.interior(r.get_state()))
    assert o.time() == r.time()


def test_oracle_threads_deterministic(oracle):
    """The gather-form oracle gives the same bits with 1 and 4 OpenMP threads."""
    from mhd_cases import ot_ini

    ini = ot_ini(dim=3, nx=12, ny=10, nz=8)
    a = oracle.OracleSolver(ini, nthreads=1)
    b = oracle.OracleSolver(ini, nthreads=4)
    a.run(3)
    b.run(3)
    assert np.array_equal(a.get_state(), b.get_state())


def test_oracle_periodic_conservation(oracle):
    """Periodic Orszag-Tang: mass and total energy are conserved to round-off."""
    from mhd_cases import ot_ini

    s = oracle.OracleSolver(ot_ini(dim=2, nx=32))
    m0 = oracle.interior(s.get_state()).reshape(8, -1).sum(1)
    s.run(20)
    m1 = oracle.interior(s.get_state()).reshape(8, -1).sum(1)
    assert abs(m1[0] - m0[0]) <= 1e-12 * abs(m0[0])
    assert abs(m1[1] - m0[1]) <= 1e-12 * abs(m0[1])


def test_fp64_round_off_floor_of_the_seeded_components(oracle):
    """Why only a bitwise FP64 build meets 1e-12 on the benchmark case's z
    momentum and z field after 100 steps: the reference's own update adds the
    O(1) z fluxes (total pressure times dt/dz) to rho*w, which is only the
    1e-3 seed (about 1e-4 in size), so every rounding of that sum sits at
    about 1e-13 of rho*w.  Planting a single change in the oracle -- dt moved
    up by one ulp at every step, nothing else -- moves rho*w and Bz by more
    than 1e-12 after 100 steps of the 48^3 perturbed Orszag-Tang case, while
    the six order-one variables stay within 1e-14."""
    from mhd_cases import ot_ini
    from ppkmhd_gb300 import workloads

    ini = ot_ini(dim=3, nx=48, ny=48, nz=48)
    a = oracle.OracleSolver(ini, nthreads=8)
    U0 = workloads.perturbed_ot_3d(a.get_state().astype(np.float64))
    b = oracle.OracleSolver(ini, nthreads=8)
    a.set_state(U0)
    b.set_state(U0)
    b.set_dt_ulps(1)
    a.run(100)
    b.run(100)
    A, Bs = oracle.interior(a.get_state()), oracle.interior(b.get_state())
    err = np.abs(Bs - A).sum(axis=(1, 2, 3)) / np.abs(A).sum(axis=(1, 2, 3))
    seeded = [4, 7]  # rho*w, Bz
    order_one = [0, 1, 2, 3, 5, 6]
    assert err[seeded].min() > 1e-12, err
    assert err[order_one].max() < 1e-14, err
