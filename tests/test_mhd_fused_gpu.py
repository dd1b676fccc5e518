"""The fused 2D tile form of the MHD solver (k_dt_only + k_mfused2d, every
intermediate in shared memory) against the reference and the stage kernels.

* MHD_FP_EXACT: the fused form is bitwise the reference's golden fixtures
  (version 2 Orszag-Tang cases, HLLD / HLL / LLF, mixed boundaries, slope
  type 1; every 2D problem fixture) and bitwise the stage form on grids with
  partial tiles (the tile is 32 x 8 cells).
* FMA builds: each kernel contracts its own expressions, so fused and stage
  forms differ at round-off (1e-13 relative L1 in FP64, 1e-5 in FP32 with the
  compensated state) and take the same number of iterations.
* The form is a fixed function of the configuration (fused for 2D FP32),
  set by mhd_set_fused, or chosen by timing both on request; 3D, versions
  0/1 and the flux surrogate have the stage form only.
"""
import glob
import os

import numpy as np
import pytest

from mhd_cases import ot_ini, perturb

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
V2_2D = [p for p in sorted(glob.glob(os.path.join(GOLDEN, "steps_ot2d_*.npz")))]
PROBLEMS_2D = [p for p in sorted(glob.glob(os.path.join(GOLDEN, "problem_*2d*.npz")))]


def rel_l1(a, b):
    ax = tuple(range(1, a.ndim))
    den = np.abs(b).sum(axis=ax)
    den = np.where(den > 1e-12 * den[0], den, den[0])
    return np.abs(a - b).sum(axis=ax) / den


@pytest.mark.parametrize("path", V2_2D, ids=[os.path.basename(p)[6:-4] for p in V2_2D])
def test_fused_exact_matches_reference_golden_bitwise(mhdlib, path):
    m = mhdlib
    z = np.load(path)
    s = m.MHDSolver.from_ini(str(z["ini"]), fp_mode=m.MHD_FP_EXACT)
    s.set_fused(True)
    assert s.fused
    if bool(z["perturbed"]):
        s.set_state(z["U0"])
    else:
        s.init_problem()
    assert s.run(1) == 1
    assert np.array_equal(m.interior(s.get_state()), z["U1"])
    s.run(int(z["nsteps"]) - 1)
    assert np.array_equal(m.interior(s.get_state()), z["Un"])
    assert s.time() == (z["t"][2], z["dt"][2], int(z["nsteps"]))
    s.close()


@pytest.mark.parametrize("path", PROBLEMS_2D, ids=[os.path.basename(p)[8:-4] for p in PROBLEMS_2D])
def test_fused_exact_problems_bitwise(mhdlib, path):
    m = mhdlib
    z = np.load(path)
    ini = str(z["ini"])
    if "implementationVersion=0" in ini or "implementationVersion=1" in ini:
        pytest.skip("versions 0 and 1 have the stage form only")
    s = m.MHDSolver.from_ini(ini, fp_mode=m.MHD_FP_EXACT)
    s.set_fused(True)
    s.init_problem()
    assert s.run(int(z["nsteps"])) == int(z["nsteps"])
    assert np.array_equal(m.interior(s.get_state()), z["Un"])
    assert s.time()[0] == z["t"][1]
    s.close()


FUSED_CASES = [
    # partial tiles along both axes, every boundary type, the three solvers,
    # both limiters, a non-square domain
    ("partial_hlld", dict(dim=2, nx=77, ny=41, bc=(1, 2, 3, 3))),
    ("partial_llf", dict(dim=2, nx=33, ny=9, riemann="llf", bc=(2, 2, 1, 1))),
    ("hll_slope1", dict(dim=2, nx=40, ny=23, riemann="hll", slope_type="1")),
    ("one_tile_row", dict(dim=2, nx=64, ny=8, bc=(3, 3, 2, 1))),
    ("small", dict(dim=2, nx=5, ny=7)),
]


@pytest.mark.parametrize("prec,mode", [(64, 1), (64, 0), (32, 0)], ids=["exact", "fast", "fp32"])
@pytest.mark.parametrize("name,kw", FUSED_CASES, ids=[c[0] for c in FUSED_CASES])
def test_fused_form_equals_stage_form(mhdlib, name, kw, prec, mode):
    m = mhdlib
    ini = ot_ini(**kw)
    U0 = perturb(m.initial_state(m.params_from_ini(ini)), 3)
    out = []
    for fused in (True, False, None, "timed"):
        s = m.MHDSolver.from_ini(ini, precision=prec, fp_mode=mode)
        if fused is not None:
            s.set_fused(fused)
        else:
            assert s.fused == (prec == 32)  # the configuration's default form
        s.set_state(U0.astype(s.real))
        s.run(7)  # "timed": the first run times both forms on a snapshot and keeps the faster
        out.append((s.get_state(), s.time(), s.diagnostics()))
        s.close()
    for q in (1, 2, 3):
        if mode == m.MHD_FP_EXACT:
            assert np.array_equal(out[0][0], out[q][0])
            assert out[0][1] == out[q][1]
        else:
            tol = 1e-13 if prec == 64 else 1e-5
            a, b = out[0][0].astype(np.float64), out[q][0].astype(np.float64)
            assert rel_l1(m.interior(a), m.interior(b)).max() <= tol
            assert out[0][1][2] == out[q][1][2]


@pytest.mark.parametrize("prec,mode", [(64, 1), (32, 0)], ids=["exact", "fp32"])
def test_fused_entry_points(mhdlib, prec, mode):
    """step, step_dt, compute_dt and the host-buffer step in the fused form
    give the states of the graph-replayed run of the same form."""
    m = mhdlib
    ini = ot_ini(dim=2, nx=70, ny=50, bc=(3, 3, 1, 2))
    U0 = perturb(m.initial_state(m.params_from_ini(ini)), 9).astype(np.float64 if prec == 64
                                                                      else np.float32)

    def make():
        s = m.MHDSolver.from_ini(ini, precision=prec, fp_mode=mode)
        s.set_fused(True)
        s.set_state(U0)
        return s

    a = make()
    a.run(3)
    ref = a.get_state()
    b = make()
    for _ in range(3):
        b.step()
    assert np.array_equal(b.get_state(), ref)
    # host-buffer steps: the state goes through the host every iteration
    # (FP32 contexts then start each step without the low parts, as the
    # stage form's host step does)
    c = make()
    hin = U0.copy()
    hout = np.empty_like(U0)
    c.step_host(hin, hout)
    d = make()
    d.run(1)
    assert np.array_equal(m.interior(hout), m.interior(d.get_state()))
    # the caller's dt, and the CFL dt of the next iteration
    e = make()
    f = m.MHDSolver.from_ini(ini, precision=prec, fp_mode=mode)
    f.set_fused(False)
    f.set_state(U0)
    dt = 0.5 * e.compute_dt()
    assert dt == 0.5 * f.compute_dt()
    e.step_dt(dt)
    f.step_dt(dt)
    if mode == m.MHD_FP_EXACT:
        assert np.array_equal(e.get_state(), f.get_state())
    else:
        assert rel_l1(m.interior(e.get_state().astype(np.float64)),
                      m.interior(f.get_state().astype(np.float64))).max() <= 1e-5
    for s in (a, b, c, d, e, f):
        s.close()


def test_fused_form_availability(mhdlib):
    m = mhdlib
    s = m.MHDSolver.from_ini(ot_ini(dim=2, nx=16))
    s.set_fused(True)
    assert s.fused
    s.set_fused(False)
    assert not s.fused
    s.close()
    for ini in (ot_ini(dim=3, nx=8), ot_ini(dim=2, nx=16, version=0),
                ot_ini(dim=2, nx=16, version=1)):
        s = m.MHDSolver.from_ini(ini)
        with pytest.raises(m.MHDError):
            s.set_fused(True)
        s.set_fused(False)
        s.init_problem()
        s.run(1)
        assert not s.fused
        s.close()


def test_fused_numeric_status(mhdlib):
    """A non-positive density is reported by the fused form's CFL pass."""
    m = mhdlib
    ini = ot_ini(dim=2, nx=40, ny=24)
    U0 = m.initial_state(m.params_from_ini(ini))
    U0[0, 10, 10] = -1.0
    s = m.MHDSolver.from_ini(ini)
    s.set_fused(True)
    s.set_state(U0)
    with pytest.raises(m.MHDError) as e:
        s.run(1)
    assert e.value.code == m.MHD_ERR_NUMERIC
    s.close()


def test_fused_conserves_and_keeps_div_b(mhdlib):
    """Periodic 2D run in the fused form: mass and the mean field conserved to
    round-off, div B at round-off (constrained transport)."""
    m = mhdlib
    ini = ot_ini(dim=2, nx=96, ny=80)
    s = m.MHDSolver.from_ini(ini)
    s.set_fused(True)
    s.init_problem()
    s0, _, _ = s.diagnostics()
    s.run(40)
    s1, divb_l1, divb_max = s.diagnostics()
    for v in (0, 5, 6):
        assert abs(s1[v] - s0[v]) <= 1e-11 * max(1.0, abs(s0[v]))
    assert divb_max < 1e-10, divb_max
    s.close()


@pytest.mark.parametrize("prec,mode,nslab", [(64, 1, 3), (32, 0, 5), (64, 0, 16)],
                         ids=["exact_3", "fp32_5", "fast_16"])
def test_fused_step_host_slabs_match_run(mhdlib, prec, mode, nslab):
    """The host-buffer step of the fused form in slabs of tile rows (uploads
    overlapping the ghost fill and CFL rates, downloads overlapping the tile
    kernel) gives the state of run() in the same form, bitwise: uneven
    slabs, more slabs requested than tile rows, reflecting / outflow faces.
    (A host state has no low parts: each FP32 step is compared with one run()
    step from the same float state.)"""
    m = mhdlib
    ini = ot_ini(dim=2, nx=45, ny=37, bc=(1, 2, 3, 3))
    a = m.MHDSolver.from_ini(ini, precision=prec, fp_mode=mode)
    c = m.MHDSolver.from_ini(ini, precision=prec, fp_mode=mode)
    for s in (a, c):
        s.set_fused(True)
        s.init_problem()
    c.set_host_slabs(nslab)
    U = c.get_state()
    out = np.zeros_like(U)
    for q in range(4):
        a.set_state(U)
        a.run(1)
        c.step_host(U, out)
        assert np.array_equal(m.interior(a.get_state()), m.interior(out)), q
        assert a.time()[1] == c.time()[1]
        U, out = out, U
    assert c.time()[2] == 4
    a.close()
    c.close()
