"""The FP64 operation counter (oracle/flop_count.cpp) is the C restatement
compiled with a counting scalar: its results must be the oracle's bit for
bit (the counting type changes no value), and its per-unit counts are the
algorithmic FP64 work behind the bench line's FP64-arithmetic roofline.
"""
import ctypes
import json
import os

import numpy as np

from mhd_cases import ot_ini

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_counting_build_matches_oracle_bitwise(oracle):
    import flop_count

    L = flop_count._lib()
    ini = ot_ini(dim=3, nx=12, ny=10, nz=8)
    o = oracle.OracleSolver(ini)
    from ppkmhd_gb300 import workloads

    U0 = np.ascontiguousarray(workloads.perturbed_ot_3d(o.get_state().astype(np.float64)))
    o.set_state(U0)
    o.run(3)
    p = oracle.OrcParams()
    assert L.orc_params_from_ini(ini.encode(), ctypes.byref(p)) == 0
    dp = ctypes.POINTER(ctypes.c_double)
    h = L.orc_create(ctypes.byref(p), 1)
    L.orc_set_state(h, U0.ctypes.data_as(dp))
    assert L.orc_run(h, 3) == 3
    U = np.empty_like(U0)
    L.orc_get_state(h, U.ctypes.data_as(dp))
    L.orc_destroy(h)
    assert np.array_equal(U, o.get_state())


def test_counts_per_unit_and_committed_summary():
    import flop_count

    pu = flop_count.count(16)
    # the 2D HLLD EMF dominates: more divides and square roots per edge than
    # any other unit, and the update is pure add/multiply
    assert pu["emf"]["div"] > pu["flux"]["div"] > pu["half_step"]["div"] > 0
    assert pu["emf"]["sqrt"] >= 16 and pu["update"]["div"] == pu["update"]["sqrt"] == 0
    assert pu["slopes"]["div"] == 0 and pu["slopes"]["cmp"] > 0
    tot = flop_count.per_cell(pu, 256, minimal=True)
    assert 3000 < tot["flop"] < 5000
    with open(os.path.join(ROOT, "profiles", "fp64_ops_ot3d_256.json")) as f:
        ref = json.load(f)["per_cell_update"]["minimal"]
    # the committed summary (counted at 32^3) agrees with this 16^3 count to
    # within the data-dependent branches of the Riemann solvers
    assert abs(tot["flop"] - ref["flop"]) <= 0.02 * ref["flop"]
