"""mhd_step_noalloc: the one entry point that allocates nothing.

Callers that cannot call cudaMalloc (a host owning all device memory through
its own pool, latency-bounded loops, fixed-footprint jobs) pass their own
device arrays for the state; intermediates live in the library's static
device scratch array.  The test allocates its device arrays itself (through
torch) and checks two calls in a row against the context-based entry points
(mhd_run on an mhd_ctx) at the FP64 test tolerance.  Collected last so that a
failure here does not hide the other tests; it also passes alone in a fresh
process.
"""
import ctypes

import numpy as np
import pytest

from mhd_cases import ot_ini

pytestmark = pytest.mark.gpu

TOL = {64: 1e-12, 32: 1e-6}  # relative L1 per variable


def rel_l1(a, b):
    ax = tuple(range(1, a.ndim))
    den = np.abs(b).sum(axis=ax)
    den = np.where(den > 1e-12 * den[0], den, den[0])
    return np.abs(a - b).sum(axis=ax) / den


@pytest.mark.parametrize("dim,n,precision", [(2, 64, 64), (3, 20, 64), (3, 20, 32)])
def test_noalloc_matches_context_path_two_calls(mhdlib, dim, n, precision):
    torch = pytest.importorskip("torch")
    m = mhdlib
    ini = ot_ini(dim=dim, nx=n, ny=n + 4, nz=n - 2)
    ref = m.MHDSolver.from_ini(ini, precision=precision, fp_mode=m.MHD_FP_FAST)
    ref.init_problem()
    U0 = ref.get_state()
    t0, _, _ = ref.time()
    expected, dts = [], []
    for _ in range(2):
        ref.run(1)
        expected.append(m.interior(ref.get_state()))
        dts.append(ref.time()[1])

    tdt = torch.float64 if precision == 64 else torch.float32
    a = torch.from_numpy(U0.copy()).to("cuda", dtype=tdt).contiguous()
    b = torch.zeros_like(a)
    p = ref.params
    dt = ctypes.c_double(0.0)
    t = t0
    for call in range(2):
        torch.cuda.synchronize()
        rc = m.lib().mhd_step_noalloc(ctypes.byref(p), ctypes.c_void_p(a.data_ptr()),
                                      ctypes.c_void_p(b.data_ptr()), t, ctypes.byref(dt), None)
        assert rc == m.MHD_OK
        got = m.interior(b.cpu().numpy())
        err = rel_l1(got.astype(np.float64), expected[call].astype(np.float64))
        assert err.max() <= TOL[precision], (call, err)
        assert abs(dt.value - dts[call]) <= 1e-12 * dts[call]
        t += dt.value
        a, b = b, a
    ref.close()


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
