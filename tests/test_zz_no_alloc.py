"""mhd_step_noalloc: the one entry point that allocates nothing.

Some callers cannot call cudaMalloc: a host application that hands every
library its device memory from its own pool, a loop with a latency bound in
which an allocation could stall or fail, a job on a shared GPU that must keep
the footprint it had at start-up.  They pass their own device arrays for the
state; the intermediates live in the library's static device scratch array.

The test allocates its device arrays itself (through torch) and checks two
calls in a row against the context-based entry point (mhd_run on an mhd_ctx):
both run the same kernel bodies of the fast build, so the states must be
equal bit for bit and dt exactly.  Each case first runs a larger grid of the
other precision through the same scratch array, so that it also shows that
leftovers of an earlier call do not leak into the result.  Collected last so
that a failure here does not hide the other tests; it also passes alone in a
fresh process.
"""
import ctypes

import numpy as np
import pytest

from mhd_cases import ot_ini

pytestmark = pytest.mark.gpu


def _noalloc(m, p, a, b, t, dt):
    return m.lib().mhd_step_noalloc(ctypes.byref(p), ctypes.c_void_p(a.data_ptr()),
                                    ctypes.c_void_p(b.data_ptr()), t, ctypes.byref(dt), None)


def _fill_scratch(m, torch, precision):
    """One call on a larger grid of the other precision (writes most of the
    scratch array with values of another problem)."""
    other = 32 if precision == 64 else 64
    ini = ot_ini(dim=3, nx=30, ny=28, nz=26)
    s = m.MHDSolver.from_ini(ini, precision=other, fp_mode=m.MHD_FP_FAST)
    s.init_problem()
    U = s.get_state()
    p = s.params
    s.close()
    tdt = torch.float64 if other == 64 else torch.float32
    a = torch.from_numpy(U).to("cuda", dtype=tdt).contiguous()
    b = torch.zeros_like(a)
    dt = ctypes.c_double(0.0)
    assert _noalloc(m, p, a, b, 0.0, dt) == m.MHD_OK
    torch.cuda.synchronize()


@pytest.mark.parametrize("dim,n,precision", [(2, 64, 64), (3, 20, 64), (3, 20, 32), (2, 48, 32)])
def test_noalloc_matches_context_path_two_calls(mhdlib, dim, n, precision):
    torch = pytest.importorskip("torch")
    m = mhdlib
    ini = ot_ini(dim=dim, nx=n, ny=n + 4, nz=n - 2)
    ref = m.MHDSolver.from_ini(ini, precision=precision, fp_mode=m.MHD_FP_FAST)
    ref.init_problem()
    U0 = ref.get_state()
    t0, _, _ = ref.time()
    # one context step from each state the caller holds (set_state: an FP32
    # state from outside has no low parts, as for the caller's arrays here)
    expected, dts = [], []
    state = U0
    for _ in range(2):
        ref.set_state(state)
        ref.run(1)
        state = ref.get_state()
        expected.append(m.interior(state))
        dts.append(ref.time()[1])
    p = ref.params
    ref.close()

    _fill_scratch(m, torch, precision)
    tdt = torch.float64 if precision == 64 else torch.float32
    a = torch.from_numpy(U0.copy()).to("cuda", dtype=tdt).contiguous()
    b = torch.zeros_like(a)
    dt = ctypes.c_double(0.0)
    t = t0
    for call in range(2):
        torch.cuda.synchronize()
        assert _noalloc(m, p, a, b, t, dt) == m.MHD_OK
        got = m.interior(b.cpu().numpy())
        assert np.array_equal(got, expected[call]), call
        assert dt.value == dts[call]
        t += dt.value
        a, b = b, a


def test_noalloc_finished_leaves_output_untouched(mhdlib):
    torch = pytest.importorskip("torch")
    m = mhdlib
    p = m.params_from_ini(ot_ini(dim=2, nx=32, tend="0.5"))
    a = torch.ones((8, 38, 38), dtype=torch.float64, device="cuda")
    b = torch.full_like(a, 7.0)
    dt = ctypes.c_double(-1.0)
    assert _noalloc(m, p, a, b, 0.5, dt) == m.MHD_FINISHED
    assert dt.value == 0.0
    assert bool((b == 7.0).all())


def test_noalloc_rejects_oversized_grid_and_bad_args(mhdlib):
    m = mhdlib
    p = m.params_from_ini(ot_ini(dim=3, nx=64))
    dt = ctypes.c_double(0.0)
    # no device memory is touched before the size check
    rc = m.lib().mhd_step_noalloc(ctypes.byref(p), ctypes.c_void_p(16), ctypes.c_void_p(32),
                                  0.0, ctypes.byref(dt), None)
    assert rc == m.MHD_ERR_TOO_LARGE
    rc = m.lib().mhd_step_noalloc(ctypes.byref(p), None, None, 0.0, ctypes.byref(dt), None)
    assert rc == m.MHD_ERR_INVALID_ARG
    p.fp_mode = m.MHD_FP_EXACT
    rc = m.lib().mhd_step_noalloc(ctypes.byref(p), ctypes.c_void_p(16), ctypes.c_void_p(32),
                                  0.0, ctypes.byref(dt), None)
    assert rc == m.MHD_ERR_INVALID_ARG
