"""Full-length runs of the five benchmark configurations with their invariants.

The timing lines of ``bench.py`` step each configuration for a few dozen
iterations; this module runs them for the step counts the configurations
are defined with and reports what must hold at the end:

* C0  2D Orszag-Tang 256^2 FP64, 100 steps
* C1  3D Orszag-Tang 256^3 (+ seeded 1e-3 velocity perturbation), 200 steps
      in FP64 and in FP32 (relative L1 of FP32 against FP64 per variable)
* C2  512-problem 2D ensemble FP32, 500 steps
* C3  3D turbulence 512^3 FP32 with the flux surrogate, 300 steps (relative
      L1 against plain FP32 HLLD per variable)
* C4  2D Kelvin-Helmholtz 4096^2 FP32, 2000 steps, plain and with the flux
      surrogate, relative L1 of both against FP64 (4096^2, and 512^2 against
      the bitwise-reference FP64 build)

For every run: the largest |div B| (FP64 sums of the face-centred field),
and the relative drift of the conserved totals that the boundary conditions
conserve (mass and total energy; all periodic or reflecting walls).

    python -m ppkmhd_gb300.validate [--configs C0,C1,...] [--device N]

prints one JSON object per configuration.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import MHDEnsemble, MHDSolver, interior, params_from_ini, workloads
from . import surrogate

ID, IP = 0, 1


def _rel_l1(a: np.ndarray, b: np.ndarray) -> list[float]:
    """Relative L1 per variable of a against b (interior arrays, var first)."""
    ax = tuple(range(1, a.ndim))
    den = np.abs(b).sum(axis=ax)
    den = np.where(den > 1e-12 * den.max(), den, den.max())
    return [float(x) for x in (np.abs(a.astype(np.float64) - b.astype(np.float64)).sum(axis=ax)
                               / den)]


def _drift(s0: np.ndarray, s1: np.ndarray) -> dict:
    return {"mass": float(abs(s1[ID] - s0[ID]) / abs(s0[ID])),
            "energy": float(abs(s1[IP] - s0[IP]) / abs(s0[IP]))}


def _solver(ini: str, U: np.ndarray, device: int, mlp=None) -> MHDSolver:
    p = params_from_ini(ini)
    p.device = device
    s = MHDSolver(p)
    s.set_state(U.astype(s.real))
    if mlp is not None:
        s.set_surrogate(mlp, tau=0.01)
    return s


def _run(s: MHDSolver, steps: int) -> dict:
    sums0, _, _ = s.diagnostics()
    t0 = time.perf_counter()
    done = s.run(steps)
    wall = time.perf_counter() - t0
    sums1, divb_l1, divb_max = s.diagnostics()
    return {"steps": done, "wall_s": wall, "divb_max": divb_max, "divb_l1": divb_l1,
            "drift": _drift(sums0, sums1)}


def c0(device: int) -> dict:
    ini = workloads.ot_ini(2, 256, precision=64)
    s = MHDSolver(_params(ini, device))
    s.init_problem()
    out = {"config": "C0 2D Orszag-Tang 256^2 FP64"} | _run(s, 100)
    s.close()
    return out


def _params(ini: str, device: int):
    p = params_from_ini(ini)
    p.device = device
    return p


def c1(device: int) -> dict:
    n, steps = 256, 200
    s = MHDSolver(_params(workloads.ot_ini(3, n, precision=64), device))
    s.init_problem()
    U0 = workloads.perturbed_ot_3d(s.get_state().astype(np.float64))
    s.set_state(U0)
    r64 = _run(s, steps)
    ref = interior(s.get_state())
    s.close()
    s = _solver(workloads.ot_ini(3, n, precision=32), U0, device)
    r32 = _run(s, steps)
    err = _rel_l1(interior(s.get_state()), ref)
    s.close()
    return {"config": "C1 3D Orszag-Tang 256^3 + 1e-3 perturbation, FP64 and FP32",
            "fp64": r64, "fp32": r32, "fp32_rel_l1_vs_fp64": err}


def c2(device: int) -> dict:
    steps = 500
    specs = workloads.ensemble_specs(512, seed=2024)
    params, states = [], []
    for sp in specs:
        ini, U = workloads.ensemble_problem(sp, precision=32)
        params.append(_params(ini, device))
        states.append(U.astype(np.float32))
    ens = MHDEnsemble(params)
    for q, U in enumerate(states):
        ens.set_state(q, U)
    sums0 = [ens.diagnostics(q)[0] for q in range(len(specs))]
    t0 = time.perf_counter()
    ens.run(steps)
    wall = time.perf_counter() - t0
    divb, mass, energy, its = [], [], [], []
    for q in range(len(specs)):
        sums1, _, dmax = ens.diagnostics(q)
        d = _drift(sums0[q], sums1)
        divb.append(dmax)
        mass.append(d["mass"])
        energy.append(d["energy"])
        its.append(ens.time(q)[2])
    ens.close()
    return {"config": "C2 512 2D Orszag-Tang problems FP32", "steps": steps, "wall_s": wall,
            "problems": len(specs), "iterations_min": int(min(its)),
            "divb_max": float(max(divb)),
            "drift_max": {"mass": float(max(mass)), "energy": float(max(energy))}}


def c3(device: int) -> dict:
    n, steps = 512, 300
    U = workloads.turbulence_3d(n, seed=11)
    ini = workloads.ot_ini(3, n, gamma0="1.6666666666666667", precision=32)
    s = _solver(ini, U, device)
    r_plain = _run(s, steps)
    ref = interior(s.get_state())
    s.close()
    s = _solver(ini, U, device, mlp=surrogate.FluxMLP.load())
    r_mlp = _run(s, steps)
    used, total = s.surrogate_stats()
    err = _rel_l1(interior(s.get_state()), ref)
    s.close()
    return {"config": "C3 3D turbulence 512^3 FP32 with the flux surrogate",
            "surrogate": r_mlp | {"faces_by_network": used / max(total, 1)},
            "plain_fp32": r_plain, "rel_l1_vs_plain_fp32": err}


def _kh(n: int, steps: int, device: int, precision: int, mlp=None, fp_mode=None):
    U = workloads.kelvin_helmholtz(n)
    s = _solver(workloads.kh_ini(n, precision=precision, fp_mode=fp_mode), U, device, mlp=mlp)
    out = _run(s, steps)
    if mlp is not None:
        used, total = s.surrogate_stats()
        out["faces_by_network"] = used / max(total, 1)
    state = interior(s.get_state())
    s.close()
    return out, state


def c4(device: int) -> dict:
    """Kelvin-Helmholtz 4096^2, 2000 steps: FP32, FP32 with the flux surrogate
    (the gamma0 = 1.4 network), and FP64 as the accuracy reference; the same
    three at 512^2 with the bitwise-reference FP64 build."""
    steps = 2000
    mlp = surrogate.FluxMLP.load(surrogate.KH_WEIGHTS)
    out = {"config": "C4 2D Kelvin-Helmholtz 4096^2 FP32 (+ flux surrogate)"}
    for n, mode in ((4096, "fast"), (512, "exact")):
        r64, ref = _kh(n, steps, device, 64, fp_mode=mode)
        r32, s32 = _kh(n, steps, device, 32)
        rmlp, smlp = _kh(n, steps, device, 32, mlp=mlp)
        tag = "" if n == 4096 else "_512"
        out[f"fp32{tag}"] = r32 | {"rel_l1_vs_fp64": _rel_l1(s32, ref)}
        out[f"fp32_surrogate{tag}"] = rmlp | {"rel_l1_vs_fp64": _rel_l1(smlp, ref)}
        out[f"fp64{tag}"] = r64 | {"fp_mode": mode}
    return out


RUNS = {"C0": c0, "C1": c1, "C2": c2, "C3": c3, "C4": c4}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--configs", default="C0,C1,C2,C3,C4")
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args()
    for name in a.configs.split(","):
        print(json.dumps(RUNS[name.strip()](a.device)), flush=True)


if __name__ == "__main__":
    main()
