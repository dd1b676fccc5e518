"""Ensembles of independent 2D problems of uneven size (mhd_ensemble_*).

Each ensemble problem runs the single-problem iteration, so the FP64 exact
build must agree bitwise with separate mhd_ctx runs; the FP32 ensemble is
checked against the FP64 oracle on a seeded subset of the 512-problem
workload.  The CPU tests cover the workload generator and the parameter
checks of mhd_ensemble_create.
"""
import ctypes

import numpy as np
import pytest

from mhd_cases import ot_ini
from ppkmhd_gb300 import workloads

TOL_FP32 = 1e-3


def rel_l1(a, b):
    ax = tuple(range(1, a.ndim))
    den = np.abs(b).sum(axis=ax)
    den = np.where(den > 1e-12 * den[0], den, den[0])
    return np.abs(a - b).sum(axis=ax) / den


# ---------------------------------------------------------------- CPU

def test_ensemble_specs_seeded_and_in_range():
    a = workloads.ensemble_specs(512, seed=2024)
    b = workloads.ensemble_specs(512, seed=2024)
    assert a == b
    sizes = np.array([s["n"] for s in a])
    assert sizes.min() >= 64 and sizes.max() <= 512
    # E[N^2] for log-uniform N on [64, 512] = (512^2 - 64^2) / (2 ln 8) ~ 6.2e4
    assert 4.5e4 < np.mean(sizes.astype(float) ** 2) < 8e4
    scales = np.array([s["b0_scale"] for s in a])
    assert scales.min() >= 0.5 and scales.max() <= 1.5
    assert workloads.ensemble_specs(512, seed=7) != a


def test_ensemble_problem_state():
    spec = dict(n=40, b0_scale=1.3, seed=11)
    ini, U = workloads.ensemble_problem(spec)
    assert "nx=40" in ini and U.shape == (8, 46, 46)
    g = 3
    # face-centred B of Orszag-Tang is divergence-free on the grid
    div = (U[5, g:-g, g + 1:-g + 1] - U[5, g:-g, g:-g]) + (U[6, g + 1:-g + 1, g:-g] - U[6, g:-g, g:-g])
    assert np.abs(div).max() < 1e-14
    # B0 scaled by b0_scale, everything else but the velocity unchanged
    unit = workloads.orszag_tang_2d(40)
    assert np.allclose(U[5:7], 1.3 * unit[5:7], rtol=1e-15, atol=0)
    assert np.array_equal(U[0], unit[0])
    # velocity perturbation: rms 5 % of v0 = 1 on the interior
    rho = U[0]
    _, U0 = workloads.ensemble_problem(dict(n=40, b0_scale=1.3, seed=11))
    assert np.array_equal(U, U0)
    base = workloads.orszag_tang_2d(40, b0_scale=1.3)
    dvx = (U[2] - base[2]) / rho
    dvy = (U[3] - base[3]) / rho
    rms = np.sqrt(np.mean(dvx[g:-g, g:-g] ** 2 + dvy[g:-g, g:-g] ** 2))
    assert abs(rms - 0.05) < 1e-12
    # periodic perturbation: the ghost columns repeat the interior
    assert np.allclose(dvx[:, :g], dvx[:, -2 * g:-g], atol=1e-12)
    # pressure stays positive
    e_kin = 0.5 * (U[2] ** 2 + U[3] ** 2) / rho
    assert np.all(U[1][g:-g, g:-g] > e_kin[g:-g, g:-g])


def test_orszag_tang_matches_library_init(oracle):
    """workloads.orszag_tang_2d with scale 1 is the reference's initial condition."""
    ini = ot_ini(dim=2, nx=24)
    p = oracle.params_from_ini(ini)
    U_ref = oracle.orszag_tang(p)
    U = workloads.orszag_tang_2d(24)
    g = 3
    assert np.allclose(U[:, g:-g, g:-g], U_ref[:, g:-g, g:-g], rtol=0, atol=2e-15)


def test_create_rejects_mixed_problems(mhdlib):
    a = mhdlib.params_from_ini(ot_ini(dim=2, nx=16))
    b = mhdlib.params_from_ini(ot_ini(dim=3, nx=8))
    with pytest.raises(mhdlib.MHDError) as e:
        mhdlib.MHDEnsemble([a, b])
    assert e.value.code == mhdlib.MHD_ERR_INVALID_ARG
    assert "same for all problems" in str(e.value)
    c = mhdlib.params_from_ini(ot_ini(dim=2, nx=16, version=1))
    with pytest.raises(mhdlib.MHDError) as e:
        mhdlib.MHDEnsemble([a, c])
    assert "version 2" in str(e.value)
    d = mhdlib.params_from_ini(ot_ini(dim=2, nx=16))
    d.gamma0 = 0.5
    with pytest.raises(mhdlib.MHDError) as e:
        mhdlib.MHDEnsemble([a, d])
    assert "problem 1" in str(e.value)
    h = ctypes.c_void_p()
    assert mhdlib.lib().mhd_ensemble_create(ctypes.byref(a), 0, ctypes.byref(h)) == \
        mhdlib.MHD_ERR_INVALID_ARG


def test_create_without_device_reports_no_device(mhdlib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    a = mhdlib.params_from_ini(ot_ini(dim=2, nx=16))
    with pytest.raises(mhdlib.MHDError) as e:
        mhdlib.MHDEnsemble([a, a])
    assert e.value.code == mhdlib.MHD_ERR_NO_DEVICE


# ---------------------------------------------------------------- GPU

def _small_specs():
    return [dict(n=n, b0_scale=s, seed=q) for q, (n, s) in
            enumerate([(16, 0.7), (37, 1.2), (24, 1.0), (50, 0.55), (19, 1.45), (31, 0.9)])]


@pytest.mark.gpu
@pytest.mark.parametrize("precision,exact", [(64, True), (64, False), (32, False)])
def test_ensemble_equals_independent_runs(mhdlib, precision, exact):
    fp = "exact" if exact else "fast"
    probs = [workloads.ensemble_problem(s, precision=precision, fp_mode=fp) for s in _small_specs()]
    ens = mhdlib.MHDEnsemble.from_ini([ini for ini, _ in probs])
    for q, (_, U) in enumerate(probs):
        ens.set_state(q, U)
    # 2D FP32 ensembles run the fused tile form by default (5 launches)
    assert ens.launches_per_step() == (5 if precision == 32 else 8)
    ens.run(9)
    for q, (ini, U) in enumerate(probs):
        s = mhdlib.MHDSolver.from_ini(ini)
        s.set_state(U.astype(s.real))
        s.run(9)
        a, b = ens.get_state(q), s.get_state()
        if exact:
            # identical kernel bodies and arithmetic without contraction: bitwise
            assert np.array_equal(a, b), (q, np.abs(a - b).max())
            assert ens.time(q) == s.time()
        elif precision == 64:
            # FMA contraction may differ between the two instantiations
            assert rel_l1(a, b).max() <= 1e-13
            assert np.allclose(ens.time(q), s.time(), rtol=1e-14, atol=0)
        else:
            # FP32 with contraction: a few ulp after 9 iterations
            assert rel_l1(a.astype(np.float64), b.astype(np.float64)).max() <= 2e-6, q
            assert np.allclose(ens.time(q), s.time(), rtol=1e-6, atol=0)


@pytest.mark.gpu
def test_ensemble_layout_right_and_stop_rules(mhdlib):
    specs = _small_specs()[:3]
    inis = []
    for q, s in enumerate(specs):
        ini, _ = workloads.ensemble_problem(s, precision=64, fp_mode="exact")
        if q == 1:
            ini = ini.replace("nStepmax=1000000", "nStepmax=3")
        inis.append(ini)
    ens = mhdlib.MHDEnsemble.from_ini(inis)
    states = [workloads.ensemble_problem(s)[1] for s in specs]
    for q, U in enumerate(states):
        # LayoutRight (i, j, var) input
        ens.set_state(q, np.ascontiguousarray(U.transpose(2, 1, 0)), layout=mhdlib.MHD_LAYOUT_RIGHT)
    ens.run(6)
    assert [ens.time(q)[2] for q in range(3)] == [6, 3, 6]
    for q, U in enumerate(states):
        s = mhdlib.MHDSolver.from_ini(inis[q])
        s.set_state(U)
        s.run(6)
        ref = s.get_state(layout=mhdlib.MHD_LAYOUT_RIGHT)
        assert np.array_equal(ens.get_state(q, layout=mhdlib.MHD_LAYOUT_RIGHT), ref)
    # the other stop rule: tEnd reached on device, dt clipped
    t3 = ens.time(0)[0]
    ini0 = inis[0].replace("tEnd=100.0", f"tEnd={t3 * 1.5!r}")
    e2 = mhdlib.MHDEnsemble.from_ini([ini0, inis[2]])
    e2.set_state(0, states[0])
    e2.set_state(1, states[2])
    e2.run(12)
    t_a, _, it_a = e2.time(0)
    assert it_a < 12 and abs(t_a - np.float32(t3 * 1.5)) < 1e-12
    assert e2.time(1)[2] == 12


@pytest.mark.gpu
@pytest.mark.parametrize("layout", ["left", "right"])
def test_ensemble_batched_state_calls_match_per_problem_calls(mhdlib, layout):
    """set_states / get_states (one synchronisation per call) give what the
    per-problem calls give, bitwise, in both layouts; a mismatched count or
    precision is rejected."""
    lay = mhdlib.MHD_LAYOUT_LEFT if layout == "left" else mhdlib.MHD_LAYOUT_RIGHT
    probs = [workloads.ensemble_problem(s, precision=64, fp_mode="exact") for s in _small_specs()]
    a = mhdlib.MHDEnsemble.from_ini([ini for ini, _ in probs])
    b = mhdlib.MHDEnsemble.from_ini([ini for ini, _ in probs])
    states = [U if lay == mhdlib.MHD_LAYOUT_LEFT else np.ascontiguousarray(U.transpose(2, 1, 0))
              for _, U in probs]
    for q, U in enumerate(states):
        a.set_state(q, U, layout=lay)
    b.set_states(states, layout=lay)
    assert [a.time(q) for q in range(len(probs))] == [b.time(q) for q in range(len(probs))]
    a.run(4)
    b.run(4)
    got = b.get_states(layout=lay)
    for q in range(len(probs)):
        assert np.array_equal(a.get_state(q, layout=lay), got[q]), q
        assert a.time(q) == b.time(q)
    with pytest.raises(ValueError):
        b.set_states(states[:-1], layout=lay)
    bad = (ctypes.c_void_p * len(states))(*[U.ctypes.data for U in states])
    assert mhdlib.lib().mhd_ensemble_set_states(b.h, bad, lay, 4) == mhdlib.MHD_ERR_INVALID_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("precision,fp", [(64, "exact"), (32, "fast")])
def test_ensemble_autotune_keeps_results(mhdlib, precision, fp):
    """Autotuning (block sizes, then the form) leaves the states, the FP32
    low parts and the records as they were: afterwards the run continues
    exactly as in an ensemble that was not tuned and takes the same form."""
    probs = [workloads.ensemble_problem(s, precision=precision, fp_mode=fp)
             for s in _small_specs()]
    a = mhdlib.MHDEnsemble.from_ini([ini for ini, _ in probs])
    b = mhdlib.MHDEnsemble.from_ini([ini for ini, _ in probs])
    for q, (_, U) in enumerate(probs):
        a.set_state(q, U)
        b.set_state(q, U)
    a.run(2)
    b.run(2)
    report = a.autotune()
    assert "uses" in report and "emf" in report
    b.set_mode(a.mode)
    a.run(5)
    b.run(5)
    for q in range(len(probs)):
        assert np.array_equal(a.get_state(q), b.get_state(q))
        assert a.time(q) == b.time(q)


@pytest.mark.gpu
def test_ensemble_conservation_and_div_b(mhdlib):
    probs = [workloads.ensemble_problem(s, precision=64) for s in _small_specs()]
    ens = mhdlib.MHDEnsemble.from_ini([ini for ini, _ in probs])
    for q, (_, U) in enumerate(probs):
        ens.set_state(q, U)
    d0 = [ens.diagnostics(q)[0] for q in range(len(probs))]
    ens.run(20)
    for q in range(len(probs)):
        d1, l1, mx = ens.diagnostics(q)
        for v in (0, 1, 2, 3):
            assert abs(d1[v] - d0[q][v]) <= 1e-12 * np.abs(d0[q]).max(), (q, v)
        assert mx < 1e-10


@pytest.mark.gpu
def test_ensemble_512_fp32_subset_against_fp64_oracle(mhdlib, oracle):
    """The 512-problem workload in FP32 (autotuned, graph replay); the
    smallest, the largest and 6 seeded random problems are re-run by the FP64
    oracle."""
    steps = 40
    specs = workloads.ensemble_specs(512, seed=2024)
    probs = [workloads.ensemble_problem(s, precision=32) for s in specs]
    ens = mhdlib.MHDEnsemble.from_ini([ini for ini, _ in probs])
    for q, (_, U) in enumerate(probs):
        ens.set_state(q, U.astype(np.float32))
    ens.autotune()
    ens.run(steps)
    sizes = [s["n"] for s in specs]
    rng = np.random.default_rng(99)
    subset = {int(np.argmin(sizes)), int(np.argmax(sizes))}
    subset |= set(int(x) for x in rng.choice(512, 6, replace=False))
    for q in sorted(subset):
        ini, U = workloads.ensemble_problem(specs[q])
        o = oracle.OracleSolver(ini, nthreads=16)
        o.set_state(U)
        o.run(steps)
        err = rel_l1(mhdlib.interior(ens.get_state(q)).astype(np.float64),
                     oracle.interior(o.get_state()))
        assert err.max() <= TOL_FP32, (q, sizes[q], err)
        assert ens.time(q)[2] == steps


@pytest.mark.gpu
@pytest.mark.parametrize("precision,exact", [(64, True), (32, False)])
def test_persistent_form_equals_graph_form(mhdlib, precision, exact):
    """One cooperative launch for the whole run (grid-wide barriers between
    the stages) gives the states of the per-stage graph form bit for bit (the
    same kernel bodies), and in the FMA-free build those of independent
    single-problem runs."""
    fp = "exact" if exact else "fast"
    probs = [workloads.ensemble_problem(s, precision=precision, fp_mode=fp) for s in _small_specs()]
    a = mhdlib.MHDEnsemble.from_ini([ini for ini, _ in probs])
    b = mhdlib.MHDEnsemble.from_ini([ini for ini, _ in probs])
    for q, (_, U) in enumerate(probs):
        a.set_state(q, U)
        b.set_state(q, U)
    a.set_mode(mhdlib.MHD_ENSEMBLE_GRAPHS)
    b.set_mode(mhdlib.MHD_ENSEMBLE_PERSISTENT)
    assert a.mode == mhdlib.MHD_ENSEMBLE_GRAPHS and b.mode == mhdlib.MHD_ENSEMBLE_PERSISTENT
    a.run(7)
    b.run(4)
    b.run(3)  # a second launch continues where the first stopped
    for q, (ini, U) in enumerate(probs):
        assert np.array_equal(a.get_state(q), b.get_state(q)), q
        assert a.time(q) == b.time(q)
        if exact:
            s = mhdlib.MHDSolver.from_ini(ini)
            s.set_state(U.astype(s.real))
            s.run(7)
            assert np.array_equal(b.get_state(q), s.get_state()), q


@pytest.mark.gpu
def test_persistent_barrier_wait_limit_reports_and_recovers(mhdlib):
    """A grid-barrier wait of the persistent form that runs out (wait limit
    0: every wait gives up at once) stops the launch early and is reported as
    an error; the ensemble stays usable and, with the states set again, runs
    to the graph form's result."""
    probs = [workloads.ensemble_problem(s, precision=32) for s in _small_specs()]
    ref = mhdlib.MHDEnsemble.from_ini([ini for ini, _ in probs])
    ens = mhdlib.MHDEnsemble.from_ini([ini for ini, _ in probs])
    for q, (_, U) in enumerate(probs):
        ref.set_state(q, U)
        ens.set_state(q, U)
    ref.set_mode(mhdlib.MHD_ENSEMBLE_GRAPHS)
    ref.run(3)
    ens.set_mode(mhdlib.MHD_ENSEMBLE_PERSISTENT)
    ens.set_wait_limit(0)
    with pytest.raises(mhdlib.MHDError) as e:
        ens.run(3)
    assert e.value.code == mhdlib.MHD_ERR_CUDA and "gave up" in str(e.value)
    ens.set_wait_limit(1 << 34)
    for q, (_, U) in enumerate(probs):
        ens.set_state(q, U)
    ens.run(3)
    for q in range(len(probs)):
        assert np.array_equal(ens.get_state(q), ref.get_state(q)), q


@pytest.mark.gpu
def test_autotune_times_both_forms(mhdlib):
    probs = [workloads.ensemble_problem(s, precision=32) for s in _small_specs()]
    ens = mhdlib.MHDEnsemble.from_ini([ini for ini, _ in probs])
    for q, (_, U) in enumerate(probs):
        ens.set_state(q, U)
    before = [ens.get_state(q) for q in range(len(probs))]
    report = ens.autotune()
    assert "form graphs:" in report and "persistent" in report and "fused tiles" in report
    assert ens.mode in (mhdlib.MHD_ENSEMBLE_GRAPHS, mhdlib.MHD_ENSEMBLE_PERSISTENT,
                        mhdlib.MHD_ENSEMBLE_FUSED)
    # tuning leaves the states as they were
    for q in range(len(probs)):
        assert np.array_equal(mhdlib.interior(ens.get_state(q)), mhdlib.interior(before[q]))
        assert ens.time(q)[2] == 0


@pytest.mark.gpu
@pytest.mark.parametrize("precision,exact", [(64, True), (64, False), (32, False)])
def test_fused_ensemble_form(mhdlib, precision, exact):
    """The fused tile form over all problems: the FMA-free build gives the
    per-stage graph form's states bit for bit and those of independent
    single-problem runs in the fused form; the FMA builds agree to
    round-off."""
    fp = "exact" if exact else "fast"
    probs = [workloads.ensemble_problem(s, precision=precision, fp_mode=fp) for s in _small_specs()]
    a = mhdlib.MHDEnsemble.from_ini([ini for ini, _ in probs])
    b = mhdlib.MHDEnsemble.from_ini([ini for ini, _ in probs])
    for q, (_, U) in enumerate(probs):
        a.set_state(q, U)
        b.set_state(q, U)
    a.set_mode(mhdlib.MHD_ENSEMBLE_GRAPHS)
    b.set_mode(mhdlib.MHD_ENSEMBLE_FUSED)
    assert b.launches_per_step() == 5 and a.launches_per_step() == 8
    a.run(7)
    b.run(4)
    b.run(3)
    for q, (ini, U) in enumerate(probs):
        s = mhdlib.MHDSolver.from_ini(ini)
        s.set_fused(True)
        s.set_state(U.astype(s.real))
        s.run(7)
        ga, gb = a.get_state(q), b.get_state(q)
        if exact:
            assert np.array_equal(ga, gb), q
            assert a.time(q) == b.time(q)
            assert np.array_equal(gb, s.get_state()), q
        else:
            tol = 1e-13 if precision == 64 else 2e-6
            assert rel_l1(ga.astype(np.float64), gb.astype(np.float64)).max() <= tol, q
            assert rel_l1(gb.astype(np.float64), s.get_state().astype(np.float64)).max() <= tol
            assert a.time(q)[2] == b.time(q)[2]
        s.close()
    # (profile_step runs a real iteration)
    names = [k for k, _ in b.profile_step()]
    assert names == ["kb_boundaries", "kb_dt_only", "kb_finalize_dt", "kb_mfused2d", "kb_advance"]


@pytest.mark.gpu
def test_fused_ensemble_form_is_2d_only(mhdlib):
    ini = ot_ini(dim=3, nx=8)
    ens = mhdlib.MHDEnsemble.from_ini([ini, ini])
    with pytest.raises(mhdlib.MHDError):
        ens.set_mode(mhdlib.MHD_ENSEMBLE_FUSED)
    assert ens.mode == mhdlib.MHD_ENSEMBLE_GRAPHS
