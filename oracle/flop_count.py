"""FP64 operation counts of the reference's 3D step (measurement infrastructure).

Runs one iteration of the C restatement compiled with a counting scalar type
(flop_count.cpp) on the benchmark's initial condition (3D Orszag-Tang with
the seeded 1e-3 velocity perturbation) and reports, per stage, the FP64
additions/subtractions, multiplications, divisions, square roots and
comparisons per unit of work (cell, face or edge), then the total per
interior cell-update at a given grid size in two forms:

* ``reference_loops``: the reference's own loop ranges (its halo work
  included, SolverMHDMuscl.cpp:465-572 and the functors' ranges);
* ``minimal``: the same per-unit counts over the units an update of n^3
  interior cells needs at least (primitives on (n+4)^3 cells, slopes and
  half step on (n+2)^3, edge field on (n+3)^3, face sources on (n+2)^3,
  fluxes on 3 n^2 (n+1) faces, EMFs on 3 n (n+1)^2 edges, dt and update on
  n^3) -- the algorithmic FP64 work behind the FP64-arithmetic roofline.

    python oracle/flop_count.py [--n 32] [--at 256] [--out profiles/fp64_ops_ot3d.json]
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))
import oracle_py  # noqa: E402

SO = os.path.join(HERE, "build", "libflop_count.so")
STAGES = ["other", "prim", "dt", "slopes", "half_step", "edge_field", "face_source", "flux",
          "emf", "update"]
KINDS = ["add", "mul", "div", "sqrt", "cmp"]


def _lib():
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    L = ctypes.CDLL(SO)
    L.orc_params_from_ini.argtypes = [ctypes.c_char_p, ctypes.POINTER(oracle_py.OrcParams)]
    L.orc_create.argtypes = [ctypes.POINTER(oracle_py.OrcParams), ctypes.c_int]
    L.orc_create.restype = ctypes.c_void_p
    L.orc_destroy.argtypes = [ctypes.c_void_p]
    L.orc_set_state.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
    L.orc_get_state.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
    L.orc_init_orszag_tang.argtypes = [ctypes.POINTER(oracle_py.OrcParams),
                                       ctypes.POINTER(ctypes.c_double)]
    L.orc_run.argtypes = [ctypes.c_void_p, ctypes.c_int]
    L.orc_run.restype = ctypes.c_int
    L.flop_counts.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_uint64)]
    return L


def units(n: int, g: int = 3) -> dict:
    """Units each stage loop of the reference covers (3D, n^3 interior)."""
    return {"prim": (n + 2 * g - 1) ** 3, "dt": n ** 3, "slopes": (n + 2 * g - 2) ** 3,
            "half_step": (n + 3) ** 3, "edge_field": (n + 2 * g - 2) ** 3,
            "face_source": (n + 2 * g - 2) ** 3, "flux": 3 * (n + 1) ** 3,
            "emf": 3 * (n + 1) ** 3, "update": n ** 3}


def minimal_units(n: int) -> dict:
    return {"prim": (n + 4) ** 3, "dt": n ** 3, "slopes": (n + 2) ** 3, "half_step": (n + 2) ** 3,
            "edge_field": (n + 3) ** 3, "face_source": (n + 2) ** 3, "flux": 3 * n * n * (n + 1),
            "emf": 3 * n * (n + 1) ** 2, "update": n ** 3}


def count(n: int = 32) -> dict:
    """Per-unit FP64 operation counts of one 3D iteration on the perturbed
    Orszag-Tang state at n^3 (second iteration: the first is run to leave
    the initial condition)."""
    from mhd_cases import ot_ini  # tests/ helper: the reference-style .ini
    from ppkmhd_gb300 import workloads

    L = _lib()
    p = oracle_py.OrcParams()
    assert L.orc_params_from_ini(ot_ini(dim=3, nx=n, ny=n, nz=n).encode(), ctypes.byref(p)) == 0
    U = np.zeros(oracle_py.state_shape(p))
    dp = ctypes.POINTER(ctypes.c_double)
    L.orc_init_orszag_tang(ctypes.byref(p), U.ctypes.data_as(dp))
    U = np.ascontiguousarray(workloads.perturbed_ot_3d(U))
    h = L.orc_create(ctypes.byref(p), 1)
    L.orc_set_state(h, U.ctypes.data_as(dp))
    assert L.orc_run(h, 1) == 1
    L.flop_reset()
    assert L.orc_run(h, 1) == 1
    L.orc_destroy(h)
    u = units(n)
    out = {}
    buf = (ctypes.c_uint64 * len(KINDS))()
    for s, name in enumerate(STAGES):
        L.flop_counts(s, buf)
        if name == "other":
            continue
        out[name] = {k: buf[i] / u[name] for i, k in enumerate(KINDS)}
    return out


def per_cell(per_unit: dict, n: int, minimal: bool) -> dict:
    u = minimal_units(n) if minimal else units(n)
    tot = {k: sum(per_unit[s][k] * u[s] for s in per_unit) / n ** 3 for k in KINDS}
    tot["flop"] = tot["add"] + tot["mul"] + tot["div"] + tot["sqrt"]
    return tot


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=32, help="grid of the counting run")
    ap.add_argument("--at", type=int, default=256, help="grid the per-cell totals are for")
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "tests"))
    pu = count(a.n)
    res = {"workload": f"3D Orszag-Tang + 1e-3 perturbation, counted at {a.n}^3 (one iteration)",
           "per_unit": pu, "grid": a.at,
           "per_cell_update": {"minimal": per_cell(pu, a.at, True),
                               "reference_loops": per_cell(pu, a.at, False)},
           "fp64_peak_tflops": 1.259,
           "fp64_peak_note": "152 SMs x 2 DFMA/cycle x 2 flop x 2.07 GHz; flop = add+mul+div+sqrt"}
    txt = json.dumps(res, indent=1)
    if a.out:
        with open(a.out, "w") as f:
            f.write(txt + "\n")
    print(txt)


if __name__ == "__main__":
    main()
