"""Benchmark of the MUSCL-Hancock + HLLD + CT MHD step on GB300.

Default workload: 3D Orszag-Tang 256^3 (periodic, HLLD, CFL 0.8, gamma0 5/3
float-rounded as the reference's ConfigMap does, seeded 1e-3 uniform velocity
perturbation), FP64 plain path in the FMA-free build (`--fp-mode exact`, the
default: the reference's operation order, bitwise equal to the reference; the
FMA-contracted build is `--fp-mode fast` and the line's `variants.fp64_fast`).
A "step" is one full iteration of the solver (boundaries, primitives, CFL dt,
slopes, half step, HLLD fluxes, CT EMFs, update).  Metric: interior
cell-updates per second.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--fp-mode exact|fast]
                  [--workload ot3d_256_fp64|ot3d_256_fp32|ot2d_256_fp64|
                              ensemble512_fp32|kh2d_4096_fp32|ot3d_128_fp64|ot3d_128_fp32|
                              kh2d_2048_fp32|turb3d_512_fp32_mlp|hydro_*]

Other workloads: the 512-problem 2D Orszag-Tang ensemble in FP32 (one
ensemble context, autotuned launch shapes) and the 2D magnetised
Kelvin-Helmholtz shear layer at 4096^2 in FP32.

One JSON line is printed by rank 0.  Multi-GPU runs (torchrun) are independent
replicas of the workload, one per GPU ("replicas only": the path has no
exchange step on one problem per GPU).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0

WORKLOADS = {
    # name: (dim, n, precision, label)
    "ot3d_256_fp64": (3, 256, 64, "3D Orszag-Tang 256^3, FP64 plain MUSCL-Hancock+HLLD+CT"),
    "ot3d_256_fp32": (3, 256, 32, "3D Orszag-Tang 256^3, FP32 plain MUSCL-Hancock+HLLD+CT"),
    "ot2d_256_fp64": (2, 256, 64, "2D Orszag-Tang 256^2, FP64 plain MUSCL-Hancock+HLLD+CT"),
    "ensemble512_fp32": (2, 0, 32, "512 independent 2D Orszag-Tang problems, N ~ logU[64,512] "
                                    "(seed 2024), B0 ~ U[0.5,1.5]/sqrt(4 pi), 5% random-phase "
                                    "Fourier velocity on |k|<=4, FP32, one ensemble context"),
    "kh2d_4096_fp32": (2, 4096, 32, "2D magnetised Kelvin-Helmholtz 4096^2 (periodic x, "
                                    "reflecting y, gamma 1.4, Bx 0.1), FP32 plain "
                                    "MUSCL-Hancock+HLLD+CT"),
    "turb3d_512_fp32_mlp": (3, 512, 32, "3D MHD turbulence 512^3 (random-phase solenoidal v and B, "
                                        "E(k)~k^-2 on 1<=|k|<=8, rms v 1, rms B 0.5), FP32 with "
                                        "the HLLD flux surrogate (tau 0.01)"),
    # reduced size for ncu captures (a few GB on the device, inputs still > L2)
    "ot3d_128_fp64": (3, 128, 64, "3D Orszag-Tang 128^3, FP64 plain MUSCL-Hancock+HLLD+CT"),
    "ot3d_128_fp32": (3, 128, 32, "3D Orszag-Tang 128^3, FP32 plain MUSCL-Hancock+HLLD+CT"),
    "kh2d_2048_fp32": (2, 2048, 32, "2D magnetised Kelvin-Helmholtz 2048^2 (periodic x, "
                                    "reflecting y, gamma 1.4, Bx 0.1), FP32 plain "
                                    "MUSCL-Hancock+HLLD+CT"),
    # the hydro-only MUSCL solver (Hydro_Muscl_3D / _2D), run_hydro
    "hydro_blast3d_fp64": (3, 0, 64, "Hydro_Muscl_3D blast, settings/test_blast_3D.ini at 4x its "
                                      "resolution (256 x 192 x 128), FP64"),
    "hydro_blast3d_fp32": (3, 0, 32, "Hydro_Muscl_3D blast, settings/test_blast_3D.ini at 4x its "
                                      "resolution (256 x 192 x 128), FP32"),
    "hydro_kh2d_4096_fp32": (2, 4096, 32, "Hydro_Muscl_2D Kelvin-Helmholtz 4096^2 (Robertson "
                                          "seed, HLLC, periodic), FP32"),
    "hydro_kh2d_4096_fp64": (2, 4096, 64, "Hydro_Muscl_2D Kelvin-Helmholtz 4096^2 (Robertson "
                                          "seed, HLLC, periodic), FP64"),
}


def ot_ini(dim: int, n: int, precision: int) -> str:
    lines = ["[run]", f"solver_name=MHD_Muscl_{dim}D", "tEnd=1000.0", "nStepmax=100000000",
             "nOutput=0", "[mesh]", f"nx={n}", f"ny={n}"]
    if dim == 3:
        lines.append(f"nz={n}")
    for f in ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax")[: 2 * dim]:
        lines.append(f"boundary_type_{f}=3")
    lines += ["[hydro]", "gamma0=1.6666666666666667", "cfl=0.8", "slope_type=2",
              "problem=orszag_tang", "riemann=hlld", "smallr=1e-8", "smallc=1e-8",
              "[OTHER]", "implementationVersion=2", "[gb300]", f"precision={precision}"]
    return "\n".join(lines) + "\n"


def perturbed_ot_state(U: np.ndarray, seed: int = 1234, amp: float = 1e-3) -> np.ndarray:
    """Seeded uniform(-amp, amp) velocity perturbation of every cell, density
    kept, total energy recomputed with the perturbed kinetic energy."""
    rng = np.random.default_rng(seed)
    U = U.astype(np.float64, copy=True)
    rho = U[0]
    ekin_old = 0.5 * (U[2] ** 2 + U[3] ** 2 + U[4] ** 2) / rho
    for v in (2, 3, 4):
        U[v] += rho * rng.uniform(-amp, amp, size=rho.shape)
    ekin_new = 0.5 * (U[2] ** 2 + U[3] ** 2 + U[4] ** 2) / rho
    U[1] += ekin_new - ekin_old
    return U


def workload_setup(name: str, precision: int):
    """(.ini text, state transform or None, data description) of a
    single-problem workload; the transform maps the Orszag-Tang initial state
    to the workload's (FP64, LayoutLeft)."""
    dim, n, _, _ = WORKLOADS[name]
    if name.startswith("turb"):
        from ppkmhd_gb300 import workloads

        return (workloads.ot_ini(3, n, gamma0="1.6666666666666667", precision=precision),
                lambda U: workloads.turbulence_3d(n, seed=11),
                "synthetic: seeded random-phase solenoidal MHD turbulence")
    if name.startswith("kh2d"):
        from ppkmhd_gb300 import workloads

        return (workloads.kh_ini(n, precision=precision),
                lambda U: workloads.kelvin_helmholtz(n),
                "synthetic: seeded magnetised Kelvin-Helmholtz shear layer")
    if dim == 3:
        return (ot_ini(dim, n, precision), perturbed_ot_state,
                "synthetic: Orszag-Tang initial condition + seeded 1e-3 velocity perturbation")
    return ot_ini(dim, n, precision), None, "synthetic: Orszag-Tang initial condition"


# ---------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- helpers

def load_peaks():
    try:
        with open(PEAKS_FILE) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def link_bandwidth(h_src, h_dst) -> dict:
    """GB/s of one plain host->device and one device->host copy of a pinned
    host tensor (the host<->device link the host-buffer step uses), timed
    after one untimed copy each way (the first touch of fresh pages is slow)."""
    import torch

    d = torch.empty_like(h_src, device="cuda")
    nb = h_src.numel() * h_src.element_size()
    d.copy_(h_src, non_blocking=True)
    h_dst.copy_(d, non_blocking=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d.copy_(h_src, non_blocking=True)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    h_dst.copy_(d, non_blocking=True)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    del d
    return {"h2d": round(nb / (t1 - t0) / 1e9, 1), "d2h": round(nb / (t2 - t1) / 1e9, 1)}


def max_over_ranks(t_sec: float, world: int, device: str) -> float:
    """The slowest rank's time (every rank times the same replica work)."""
    if world <= 1:
        return t_sec
    import torch

    tt = torch.tensor([t_sec], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
    return float(tt.item())


def replica_value(units_per_rank: float, t_sec: float, world: int) -> float:
    """Whole-job throughput of N independent replicas: all ranks' units over
    the slowest rank's time."""
    return world * units_per_rank / t_sec


def emit(obj):
    print(json.dumps(obj), flush=True)


# ---------------------------------------------------------------- CPU side

def cpu_baseline_run(name: str, steps: int | None, warmup: int, nthreads: int,
                     target_s: float = 8.0, want_state: bool = False):
    """The oracle port of the reference step (oracle/mhd_oracle.c) on the host
    cores: same workload, full grid.  steps=None sizes the timed sample to
    about target_s seconds from the duration of the warm-up steps (and caps a
    given count there).  Returns
    (cell-updates/s, seconds timed, steps timed), plus the interior state
    after the warm-up and timed steps when want_state."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py

    oracle_py.build_oracle()
    dim, n, _, _ = WORKLOADS[name]
    ini, transform, _ = workload_setup(name, 64)
    s = oracle_py.OracleSolver(ini, nthreads=nthreads)
    if transform is not None:
        s.set_state(transform(s.get_state()))
    t0 = time.perf_counter()
    s.run(max(warmup, 1))
    t_one = (time.perf_counter() - t0) / max(warmup, 1)
    cap = int(min(5000, max(2, target_s / max(t_one, 1e-6))))
    steps = cap if steps is None else min(steps, cap)
    t0 = time.perf_counter()
    s.run(steps)
    el = time.perf_counter() - t0
    state = oracle_py.interior(s.get_state()) if want_state else None
    s.close()
    cells = n ** dim
    if want_state:
        return cells * steps / el, el, steps, state
    return cells * steps / el, el, steps


# ---------------------------------------------------------------- GPU side

def run_gb300(args):
    world, rank, local = dist_setup()
    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import ppkmhd_gb300 as m

    dim, n, precision, label = WORKLOADS[args.workload]
    ini, transform, data_desc = workload_setup(args.workload, precision)
    p = m.params_from_ini(ini)
    p.device = local
    # FP64 headline: the FMA-free build, bitwise equal to the reference
    exact = precision == 64 and args.fp_mode == "exact"
    p.fp_mode = m.MHD_FP_EXACT if exact else m.MHD_FP_FAST
    s = m.MHDSolver(p)
    s.init_problem()
    U0 = s.get_state()
    if transform is not None:
        s.set_state(transform(U0.astype(np.float64)).astype(s.real))
        U0 = s.get_state()
    interior_cells, ghost_cells = s.cell_counts()
    state_bytes = U0.nbytes
    real_bytes = 8 if precision == 64 else 4

    # warm-up (device-resident, graph replay)
    s.run_timed(max(args.warmup, 3))

    # ---- timed region: device-resident state, CUDA events on the library stream
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = s.run_timed(args.steps)
    torch.cuda.synchronize()
    t_sec = ms / 1e3
    t_sec = max_over_ranks(t_sec, world, "cuda")
    value = replica_value(interior_cells * args.steps, t_sec, world)

    # ---- per-kernel timing of one iteration (events around every launch)
    prof = {}
    for _ in range(3):
        for name, kms in s.profile_step():
            prof.setdefault(name, []).append(kms)
    prof = {k: float(np.median(v)) for k, v in prof.items()}
    step_ms = sum(prof.values())
    dom = max(prof, key=prof.get)

    hbm_peak, peak_kind = load_peaks()
    alg_bytes_per_cell = 16 * real_bytes
    achieved = alg_bytes_per_cell * interior_cells / (prof[dom] / 1e3) / 1e9
    step_achieved = alg_bytes_per_cell * interior_cells / (step_ms / 1e3) / 1e9
    traffic = load_profile_traffic(args.workload, dom)

    # Companion figures for the same workload (device-resident): the other
    # FP64 build, FP32 and FP32 + flux surrogate, each with its relative L1
    # per variable against the exact FP64 state after the same steps
    variants = {}
    accuracy = None
    if args.workload == "ot3d_256_fp64" and not args.no_variants:
        from ppkmhd_gb300 import surrogate

        acc_steps = 20
        px = m.params_from_ini(ini)
        px.device = local
        px.fp_mode = m.MHD_FP_EXACT
        sx = m.MHDSolver(px)
        sx.set_state(U0)
        sx.run(acc_steps)
        ref = m.interior(sx.get_state())
        sx.close()
        den = np.abs(ref).sum(axis=(1, 2, 3))
        den = np.where(den > 1e-12 * den[0], den, den[0])
        other = "fp64_fast" if exact else "fp64_exact"
        po = m.params_from_ini(ini)
        po.device = local
        po.fp_mode = m.MHD_FP_FAST if exact else m.MHD_FP_EXACT
        so = m.MHDSolver(po)
        so.set_state(U0)
        so.run(acc_steps)
        err_o = np.abs(m.interior(so.get_state()) - ref).sum(axis=(1, 2, 3)) / den
        so.set_state(U0)
        so.run_timed(3)
        mso = so.run_timed(args.steps)
        so.close()
        variants[other] = {"value": interior_cells * args.steps / (mso / 1e3),
                           "ms_per_step": mso / args.steps, "dtype": "f64",
                           "rel_l1_vs_exact_per_variable": [float(x) for x in err_o],
                           "accuracy_steps": acc_steps,
                           "note": ("FMA-contracted build with shared reciprocals: within 1e-12 "
                                    "of the reference on the order-one variables; the seeded z "
                                    "momentum and z field differ at the FP64 round-off floor of "
                                    "the reference's own update, which a 1-ulp change of dt alone "
                                    "reproduces (tests/test_oracle_pinning.py)")
                           if exact else "FMA-free build in the reference's operation order: "
                                         "bitwise equal to the reference"}
        for tag, use_mlp in (("fp32", False), ("fp32_surrogate", True)):
            p32 = m.params_from_ini(ot_ini(dim, n, 32))
            p32.device = local
            s32 = m.MHDSolver(p32)
            s32.set_state(U0.astype(np.float32))
            if use_mlp:
                s32.set_surrogate(surrogate.FluxMLP.load(), tau=0.01)
            s32.run(acc_steps)
            err = np.abs(m.interior(s32.get_state()).astype(np.float64) - ref).sum(axis=(1, 2, 3))
            s32.set_state(U0.astype(np.float32))
            s32.run_timed(3)
            ms32 = s32.run_timed(args.steps)
            v = {"value": interior_cells * args.steps / (ms32 / 1e3),
                 "ms_per_step": ms32 / args.steps, "dtype": "f32",
                 "rel_l1_vs_fp64": float((err / den).max()),
                 "rel_l1_vs_fp64_per_variable": [float(x) for x in err / den],
                 "accuracy_steps": acc_steps,
                 "note": "FP32 arithmetic, compensated FP32 state (float pair), FP64 dt/sums/div B"}
            if use_mlp:
                used, total = s32.surrogate_stats()
                v["faces_by_network"] = used / max(total, 1)
                v["note"] += "; HLLD flux surrogate (BF16 tensor-core MLP, tau 0.01)"
                v["dtype"] = "f32+bf16"
            variants[tag] = v
            s32.close()

    hydro = None
    if args.workload == "ot3d_256_fp64" and not args.no_variants and world == 1:
        hydro = hydro_companion(m, local, 10, cpu=not args.no_cpu_baseline)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        nthreads = os.cpu_count() or 1
        v, el, ns, cpu_state = cpu_baseline_run(args.workload, steps=args.cpu_steps, warmup=1,
                                                nthreads=nthreads, want_state=True)
        cpu = {"value": v, "unit": "cell-updates/s", "cores": nthreads, "kind": "port",
               "sample": f"{ns} steps of the same {n}^{dim} grid after 1 warm-up "
                         f"step, oracle/mhd_oracle.c with {nthreads} OpenMP threads "
                         f"({el:.1f} s timed)"}
        if precision == 64:
            # the headline build against the CPU run of the same steps
            pc = m.params_from_ini(ini)
            pc.device = local
            pc.fp_mode = p.fp_mode
            sc = m.MHDSolver(pc)
            sc.set_state(U0)
            sc.run(ns + 1)
            mine = m.interior(sc.get_state())
            sc.close()
            dn = np.abs(cpu_state).sum(axis=tuple(range(1, dim + 1)))
            dn = np.where(dn > 1e-12 * dn[0], dn, dn[0])
            accuracy = {"steps": ns + 1, "reference": "oracle/mhd_oracle.c (bitwise the "
                        "reference compiled without FMA contraction), same initial state",
                        "bitwise_equal": bool(np.array_equal(mine, cpu_state)),
                        "rel_l1_per_variable": [float(x) for x in
                                                np.abs(mine - cpu_state).sum(
                                                    axis=tuple(range(1, dim + 1))) / dn]}

    # ---- end to end through the host-buffer ABI call (H2D + step + D2H per
    # step), measured last: right after a process that freed much device
    # memory exits, the GPU's background clearing of that memory competes
    # with host<->device copies for the first seconds of the next process
    e2e_steps = max(2, min(args.steps, 10))
    h_in = torch.empty(U0.size, dtype=torch.float64 if precision == 64 else torch.float32,
                       pin_memory=True)
    h_out = torch.empty_like(h_in, pin_memory=True)
    h_in.numpy()[:] = U0.reshape(-1)
    link = link_bandwidth(h_in, h_out)
    for _ in range(2):  # warm
        s.step_host_ptr(h_in.data_ptr(), h_out.data_ptr())
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    per_step = []
    t0 = time.perf_counter()
    for q in range(e2e_steps):
        a, b = (h_in, h_out) if q % 2 == 0 else (h_out, h_in)
        tq = time.perf_counter()
        s.step_host_ptr(a.data_ptr(), b.data_ptr())
        per_step.append((time.perf_counter() - tq) * 1e3)
    e2e_sec = max_over_ranks(time.perf_counter() - t0, world, "cuda")
    e2e_value = world * interior_cells * e2e_steps / e2e_sec

    if rank == 0:
        out = {
            "metric": "MHD cell-updates/s (interior cells), plain MUSCL-Hancock+HLLD+CT step",
            "value": value,
            "unit": "cell-updates/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": max(args.warmup, 3),
            "ms_per_step": t_sec * 1e3 / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64" if precision == 64 else "f32",
            "fp_mode": ("exact (FMA-free, the reference's operation order)" if exact
                        else "fast (FMA contraction)") if precision == 64 else "fp32",
            "data": data_desc,
            "config": {"workload": label, "grid": [n] * dim, "cells": interior_cells,
                       "cells_with_ghosts": ghost_cells, "state_bytes": state_bytes,
                       "l2": "inputs larger than L2 (state %.2f GB per array)" % (state_bytes / 1e9),
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "kernels_per_step": s.launches_per_step(),
                       "form": ("fused tile kernel (k_mfused2d)" if s.fused
                                else "stage kernels"),
                       "per_kernel_ms": prof},
            "e2e": {"value": e2e_value, "unit": "cell-updates/s",
                    "h2d_bytes_per_step": state_bytes, "d2h_bytes_per_step": state_bytes,
                    "steps": e2e_steps,
                    "call": "mhd_step_host (pinned host buffers, copies inside the timed region; "
                            "uploads and downloads overlap the step slab by slab, one slab "
                            "per 64 MiB of state, at most 16)",
                    "link_gbs": link,
                    "ms_each_step": [round(x, 2) for x in per_step]},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak,
                         "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": traffic,
                         "peak_source": f"hbm_gbs of {peak_kind}",
                         "algorithmic_bytes_per_cell": alg_bytes_per_cell,
                         "step_achieved": step_achieved,
                         "step_frac": step_achieved / hbm_peak},
            "alu_roofline": fp64_roofline(args.workload, value, dom, exact)
            if precision == 64 and dim == 3 else None,
            "clocks": clk.summary(),
            "gpu_launches": s.launches_per_step() * args.steps,
            "cpu_baseline": cpu,
            "variants": variants,
        }
        if accuracy is not None:
            out["accuracy"] = accuracy
        if hydro is not None:
            out["hydro"] = hydro
        emit(out)
    s.close()
    if world > 1:
        torch.distributed.destroy_process_group()


HYDRO_WORKLOAD = ("Hydro_Muscl_3D blast with the settings of the reference's "
                  "settings/test_blast_3D.ini (HLLC, slope_type 2, reflecting walls, gamma0 "
                  "1.666, cfl 0.8, implementation version 0) at four times its resolution: "
                  "256 x 192 x 128 interior cells")


def hydro_bench_ini(nx: int = 256, ny: int = 192, nz: int = 128) -> str:
    return f"""[run]
solver_name=Hydro_Muscl_3D
tEnd=50.0
nStepmax=100000
nOutput=0
[mesh]
nx={nx}
ny={ny}
nz={nz}
xmax=2.0
ymax=1.5
zmax=1.0
boundary_type_xmin=1
boundary_type_xmax=1
boundary_type_ymin=1
boundary_type_ymax=1
boundary_type_zmin=1
boundary_type_zmax=1
[hydro]
gamma0=1.666
cfl=0.8
niter_riemann=10
iorder=2
slope_type=2
problem=blast
riemann=hllc
[blast]
density_in=1.0
density_out=1.2
[other]
implementationVersion=0
"""


def hydro_companion(m, local: int, steps: int, cpu: bool):
    """The hydro-only MUSCL solver (row f4) on HYDRO_WORKLOAD: the three
    builds device-resident (CUDA events), per-kernel times of the exact
    build, the exact build against the C oracle (bitwise, 2 iterations of the
    full grid), the other builds' relative L1 per variable against the exact
    state after 10 iterations, and the oracle's CPU rate on the same grid."""
    ini = hydro_bench_ini()
    out = {"workload": HYDRO_WORKLOAD, "builds": {}}
    states = {}
    for tag, prec, mode in (("fp64_exact", 64, m.MHD_FP_EXACT), ("fp64_fast", 64, m.MHD_FP_FAST),
                            ("fp32", 32, m.MHD_FP_FAST)):
        p = m.params_from_ini(ini)
        p.device, p.precision, p.fp_mode = local, prec, mode
        s = m.MHDSolver(p)
        s.init_problem()
        cells, _ = s.cell_counts()
        s.run(10)
        states[tag] = m.interior(s.get_state(), ghost=2).astype(np.float64)
        s.init_problem()
        s.run_timed(3)
        ms = s.run_timed(steps)
        out["builds"][tag] = {"value": cells * steps / (ms / 1e3), "ms_per_step": ms / steps,
                              "dtype": "f64" if prec == 64 else "f32",
                              "form": "fused tile kernel" if s.fused else "stage kernels"}
        if tag == "fp64_exact":
            prof = {}
            for _ in range(3):
                for name, kms in s.profile_step():
                    prof.setdefault(name, []).append(kms)
            out["per_kernel_ms"] = {k: float(np.median(v)) for k, v in prof.items()}
            s.init_problem()
            s.run(2)
            exact2 = m.interior(s.get_state(), ghost=2)
            U0 = m.initial_state(m.params_from_ini(ini))
        s.close()
        out["cells"] = cells
    ref = states["fp64_exact"]
    den = np.maximum(np.abs(ref).sum(axis=(1, 2, 3)), 1e-300)
    for tag in ("fp64_fast", "fp32"):
        err = np.abs(states[tag] - ref).sum(axis=(1, 2, 3)) / den
        out["builds"][tag]["rel_l1_vs_exact_per_variable"] = [float(x) for x in err]
        out["builds"][tag]["accuracy_steps"] = 10
    ms_exact = out["builds"]["fp64_exact"]["ms_per_step"]
    hbm_peak, peak_kind = load_peaks()
    alg = 2 * 5 * 8  # read and write the 5 FP64 conservative variables per cell
    out["roofline"] = {"bound": "fp64 alu (exact build; see the MHD alu_roofline)",
                       "algorithmic_bytes_per_cell": alg,
                       "step_achieved_gbs": alg * out["cells"] / (ms_exact / 1e3) / 1e9,
                       "hbm_peak_gbs": hbm_peak, "peak_source": f"hbm_gbs of {peak_kind}"}
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py

    oracle_py.build_oracle()
    nthreads = os.cpu_count() or 1
    o = oracle_py.HydroOracleSolver(ini, nthreads=nthreads)
    o.set_state(U0)
    t0 = time.perf_counter()
    o.run(2)
    el = time.perf_counter() - t0
    out["accuracy"] = {"steps": 2, "bitwise_equal_exact_vs_oracle": bool(np.array_equal(
        oracle_py.interior(o.get_state(), 2), exact2)),
        "reference": "oracle/hydro_oracle.c, bitwise the reference's hydro functors compiled "
                     "without FMA contraction (tests/test_hydro_oracle.py)"}
    if cpu:
        ns = int(min(50, max(2, 8.0 / max(el / 2, 1e-6))))
        t0 = time.perf_counter()
        o.run(ns)
        el = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": out["cells"] * ns / el, "unit": "cell-updates/s",
                               "cores": nthreads, "kind": "port",
                               "sample": f"{ns} iterations of the same grid after 2, "
                                         f"oracle/hydro_oracle.c with {nthreads} OpenMP threads "
                                         f"({el:.1f} s timed)"}
    o.close()
    return out


def hydro_kh2d_ini(n: int = 4096) -> str:
    return f"""[run]
solver_name=Hydro_Muscl_2D
tEnd=10.0
nStepmax=100000
nOutput=0
[mesh]
nx={n}
ny={n}
boundary_type_xmin=3
boundary_type_xmax=3
boundary_type_ymin=3
boundary_type_ymax=3
[hydro]
gamma0=1.4
cfl=0.8
slope_type=2
problem=kelvin_helmholtz
riemann=hllc
[other]
implementationVersion=0
"""


def run_hydro(args):
    """A hydro-only MUSCL workload as its own line: device-resident rate
    (CUDA events), per-kernel times, the form the context chose (fused tile
    kernel or stage kernels), the HBM roofline of the dominant kernel, the
    host-buffer rate (mhd_step_host, pinned buffers), the FMA-free build
    against the oracle (bitwise, 2 iterations) and the oracle on the host
    cores."""
    import torch
    import ppkmhd_gb300 as m

    dim, _, precision, label = WORKLOADS[args.workload]
    ini = hydro_bench_ini() if "blast3d" in args.workload else hydro_kh2d_ini()
    exact = precision == 64 and args.fp_mode == "exact"
    p = m.params_from_ini(ini)
    p.precision = precision
    p.fp_mode = m.MHD_FP_EXACT if exact else m.MHD_FP_FAST
    s = m.MHDSolver(p)
    s.init_problem()
    cells, ghost_cells = s.cell_counts()
    U0 = s.get_state()
    s.run_timed(max(args.warmup, 3))
    s.init_problem()
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        ms = s.run_timed(args.steps)
    torch.cuda.synchronize()
    value = cells * args.steps / (ms / 1e3)
    prof = {}
    for _ in range(3):
        for name, kms in s.profile_step():
            prof.setdefault(name, []).append(kms)
    prof = {k: float(np.median(v)) for k, v in prof.items()}
    dom = max(prof, key=prof.get)
    rb = 8 if precision == 64 else 4
    alg = 2 * (dim + 2) * rb
    hbm_peak, peak_kind = load_peaks()
    achieved = alg * cells / (prof[dom] / 1e3) / 1e9
    form = "fused tile kernel" if s.fused else "stage kernels"
    # host-buffer steps
    h_in = torch.empty(U0.size, dtype=torch.float64 if precision == 64 else torch.float32,
                       pin_memory=True)
    h_out = torch.empty_like(h_in, pin_memory=True)
    h_in.numpy()[:] = U0.reshape(-1)
    s.init_problem()
    for _ in range(2):
        s.step_host_ptr(h_in.data_ptr(), h_out.data_ptr())
    n_e2e = max(2, min(args.steps, 10))
    t0 = time.perf_counter()
    for q in range(n_e2e):
        a, b = (h_in, h_out) if q % 2 == 0 else (h_out, h_in)
        s.step_host_ptr(a.data_ptr(), b.data_ptr())
    e2e = cells * n_e2e / (time.perf_counter() - t0)
    accuracy, cpu = None, None
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle_py

        oracle_py.build_oracle()
        nthreads = os.cpu_count() or 1
        o = oracle_py.HydroOracleSolver(ini, nthreads=nthreads)
        o.set_state(U0.astype(np.float64))
        t0 = time.perf_counter()
        o.run(2)
        el2 = time.perf_counter() - t0
        if precision == 64:
            s.set_state(U0)
            s.run(2)
            mine = m.interior(s.get_state(), ghost=2)
            ref = oracle_py.interior(o.get_state(), 2)
            den = np.maximum(np.abs(ref).sum(axis=tuple(range(1, dim + 1))), 1e-300)
            accuracy = {"steps": 2, "bitwise_equal": bool(np.array_equal(mine, ref)),
                        "rel_l1_per_variable": [float(x) for x in np.abs(mine - ref).sum(
                            axis=tuple(range(1, dim + 1))) / den],
                        "reference": "oracle/hydro_oracle.c (bitwise the reference's hydro "
                                     "functors compiled without FMA contraction)"}
        ns = int(min(50, max(2, 8.0 / max(el2 / 2, 1e-6))))
        t0 = time.perf_counter()
        o.run(ns)
        el = time.perf_counter() - t0
        o.close()
        cpu = {"value": cells * ns / el, "unit": "cell-updates/s", "cores": nthreads,
               "kind": "port", "sample": f"{ns} iterations of the same grid after 2, "
                                         f"oracle/hydro_oracle.c with {nthreads} OpenMP threads "
                                         f"({el:.1f} s timed)"}
    out = {
        "metric": "hydro cell-updates/s (interior cells), MUSCL-Hancock hydro step "
                  f"(Hydro_Muscl_{dim}D)",
        "value": value, "unit": "cell-updates/s", "n_gpus": 1, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if precision == 64 else "f32",
        "fp_mode": ("exact" if exact else "fast") if precision == 64 else "fp32",
        "data": "synthetic (the problem's own initial condition)",
        "config": {"workload": label, "cells": cells, "cells_with_ghosts": ghost_cells,
                   "state_bytes": U0.nbytes, "form": form, "per_kernel_ms": prof,
                   "kernels_per_step": s.launches_per_step(),
                   "l2": "inputs larger than L2 (state %.2f GB per array)" % (U0.nbytes / 1e9)},
        "e2e": {"value": e2e, "unit": "cell-updates/s", "h2d_bytes_per_step": U0.nbytes,
                "d2h_bytes_per_step": U0.nbytes, "steps": n_e2e,
                "call": "mhd_step_host (pinned host buffers, copies inside the timed region)"},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak,
                     "unit": "GB/s", "frac": achieved / hbm_peak,
                     "traffic": load_profile_traffic(args.workload, dom),
                     "peak_source": f"hbm_gbs of {peak_kind}",
                     "algorithmic_bytes_per_cell": alg},
        "clocks": clk.summary(),
        "gpu_launches": s.launches_per_step() * args.steps,
        "cpu_baseline": cpu,
    }
    if accuracy is not None:
        out["accuracy"] = accuracy
    s.close()
    emit(out)


def ensemble_sample(specs):
    """Problems the CPU legs time: the smallest, the largest and 6 seeded
    random ones."""
    sizes = [sp["n"] for sp in specs]
    rng = np.random.default_rng(99)
    sub = {int(np.argmin(sizes)), int(np.argmax(sizes))}
    sub |= set(int(x) for x in rng.choice(len(specs), 6, replace=False))
    return sorted(sub)


def cpu_ensemble_run(specs, steps: int, nthreads: int):
    """The oracle port on the sample problems of the ensemble, one after the
    other (the reference has no batching), `steps` timed iterations each."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py
    from ppkmhd_gb300 import workloads

    oracle_py.build_oracle()
    cells = 0
    el = 0.0
    sample = ensemble_sample(specs)
    for q in sample:
        ini, U = workloads.ensemble_problem(specs[q])
        o = oracle_py.OracleSolver(ini, nthreads=nthreads)
        o.set_state(U)
        o.run(1)
        t0 = time.perf_counter()
        o.run(steps)
        el += time.perf_counter() - t0
        cells += specs[q]["n"] ** 2 * steps
        o.close()
    desc = (f"{len(sample)} of the 512 problems (N = "
            + ", ".join(str(specs[q]["n"]) for q in sample)
            + f"), {steps} steps each after 1 warm-up step, oracle/mhd_oracle.c with {nthreads} "
              f"OpenMP threads, FP64, one problem at a time ({el:.1f} s timed)")
    return cells / el, el, desc


def run_ensemble(args):
    """The 512-problem FP32 ensemble: one context, autotuned launch shapes,
    CUDA-graph replay; value = interior cell-updates/s over all problems."""
    world, rank, local = dist_setup()
    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import ppkmhd_gb300 as m
    from ppkmhd_gb300 import workloads

    specs = workloads.ensemble_specs(512, seed=2024)
    params, states = [], []
    for sp in specs:
        ini, U = workloads.ensemble_problem(sp, precision=32)
        p = m.params_from_ini(ini)
        p.device = local
        params.append(p)
        states.append(U.astype(np.float32))
    ens = m.MHDEnsemble(params)
    for q, U in enumerate(states):
        ens.set_state(q, U)
    cells = ens.cell_count()
    state_bytes = int(sum(U.nbytes for U in states))
    tune = ens.autotune()

    ens.run(max(args.warmup, 3))
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = ens.run(args.steps)
    torch.cuda.synchronize()
    t_sec = ms / 1e3
    t_sec = max_over_ranks(t_sec, world, "cuda")
    value = replica_value(cells * args.steps, t_sec, world)

    prof = {}
    for _ in range(3):
        for name, kms in ens.profile_step():
            prof.setdefault(name, []).append(kms)
    prof = {k: float(np.median(v)) for k, v in prof.items()}
    step_ms = sum(prof.values())
    dom = max(prof, key=prof.get)

    hbm_peak, peak_kind = load_peaks()
    alg = 16 * 4
    achieved = alg * cells / (prof[dom] / 1e3) / 1e9
    step_achieved = alg * cells / (step_ms / 1e3) / 1e9

    hydro = None
    if args.workload == "ot3d_256_fp64" and not args.no_variants and world == 1:
        hydro = hydro_companion(m, local, 10, cpu=not args.no_cpu_baseline)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        nthreads = os.cpu_count() or 1
        v, el, desc = cpu_ensemble_run(specs, steps=args.cpu_steps, nthreads=nthreads)
        cpu = {"value": v, "unit": "cell-updates/s", "cores": nthreads, "kind": "port",
               "sample": desc}

    # end to end through the public API: upload every problem from pinned
    # host memory, run the steps, read every problem back (measured last, as
    # for the single-problem workloads: right after a process that freed much
    # device memory exits, the clearing of that memory slows host<->device
    # copies for some seconds)
    e2e_steps = args.steps
    pinned = []
    for U in states:
        h = torch.empty(U.shape, dtype=torch.float32, pin_memory=True)
        h.numpy()[:] = U
        pinned.append(h)
    ptrs = [h.data_ptr() for h in pinned]
    ens.set_states_ptr(ptrs)  # untimed: first touch of the pinned pages
    ens.get_states_ptr(ptrs)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ens.set_states_ptr(ptrs)
    ens.run(e2e_steps)
    ens.get_states_ptr(ptrs)
    e2e_sec = max_over_ranks(time.perf_counter() - t0, world, "cuda")
    e2e_value = world * cells * e2e_steps / e2e_sec

    if rank == 0:
        sizes = [sp["n"] for sp in specs]
        emit({
            "metric": "MHD cell-updates/s (interior cells), 512-problem 2D ensemble",
            "value": value,
            "unit": "cell-updates/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": max(args.warmup, 3),
            "ms_per_step": t_sec * 1e3 / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32",
            "data": "synthetic: seeded Orszag-Tang ensemble (sizes, B0, Fourier velocity)",
            "config": {"workload": WORKLOADS["ensemble512_fp32"][3], "problems": len(specs),
                       "n_min": min(sizes), "n_max": max(sizes), "cells": cells,
                       "state_bytes": state_bytes,
                       "l2": "inputs larger than L2 (%.2f GB of state per array)" % (state_bytes / 1e9),
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "kernels_per_step": ens.launches_per_step(),
                       "per_kernel_ms": prof,
                       "autotune": [ln for ln in tune.splitlines()
                                    if ln.startswith("->") or ln.startswith("form")]},
            "e2e": {"value": e2e_value, "unit": "cell-updates/s",
                    "h2d_bytes_per_step": state_bytes / e2e_steps,
                    "d2h_bytes_per_step": state_bytes / e2e_steps, "steps": e2e_steps,
                    "call": "mhd_ensemble_set_states + mhd_ensemble_run + "
                            "mhd_ensemble_get_states (512 pinned host buffers, inside the timed "
                            "region)"},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak,
                         "unit": "GB/s", "frac": achieved / hbm_peak,
                         "traffic": load_profile_traffic("ensemble512_fp32", dom),
                         "peak_source": f"hbm_gbs of {peak_kind}",
                         "algorithmic_bytes_per_cell": alg,
                         "step_achieved": step_achieved, "step_frac": step_achieved / hbm_peak},
            "clocks": clk.summary(),
            "gpu_launches": ens.launches_per_step() * args.steps,
            "cpu_baseline": cpu,
        })
    ens.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def run_turbulence(args):
    """FP32 turbulence with the flux surrogate: throughput of the surrogate
    run and of plain FP32, accuracy of both against the FP64 solution of the
    same steps (GPU FP64 path, equal to the oracle within 1e-12)."""
    world, rank, local = dist_setup()
    import torch

    torch.cuda.set_device(local)
    import ppkmhd_gb300 as m
    from ppkmhd_gb300 import surrogate, workloads

    dim, n, precision, label = WORKLOADS[args.workload]
    g = "1.6666666666666667"
    ini32 = workloads.ot_ini(3, n, gamma0=g, precision=32)
    ini64 = workloads.ot_ini(3, n, gamma0=g, precision=64)
    U = workloads.turbulence_3d(n, seed=11)
    mlp = surrogate.FluxMLP.load()
    tau = 0.01

    def ctx(ini, with_mlp):
        p = m.params_from_ini(ini)
        p.device = local
        s = m.MHDSolver(p)
        s.set_state(U.astype(s.real))
        if with_mlp:
            s.set_surrogate(mlp, tau=tau)
        return s

    # throughput (device-resident, graph replay)
    s = ctx(ini32, True)
    cells, _ = s.cell_counts()
    s.run_timed(max(args.warmup, 3))
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        ms = s.run_timed(args.steps)
    torch.cuda.synchronize()
    value = cells * args.steps / (ms / 1e3)
    prof = {}
    for _ in range(3):
        for name, kms in s.profile_step():
            prof.setdefault(name, []).append(kms)
    prof = {k: float(np.median(v)) for k, v in prof.items()}
    dom = max(prof, key=prof.get)
    used, total = s.surrogate_stats()
    # e2e through the host-buffer call
    U0 = s.get_state()
    h_in = torch.empty(U0.size, dtype=torch.float32, pin_memory=True)
    h_out = torch.empty_like(h_in, pin_memory=True)
    h_in.numpy()[:] = U0.reshape(-1)
    link = link_bandwidth(h_in, h_out)
    for _ in range(2):  # warm
        s.step_host_ptr(h_in.data_ptr(), h_out.data_ptr())
    e2e_steps = 3
    per_step = []
    t0 = time.perf_counter()
    for q in range(e2e_steps):
        a, b = (h_in, h_out) if q % 2 == 0 else (h_out, h_in)
        tq = time.perf_counter()
        s.step_host_ptr(a.data_ptr(), b.data_ptr())
        per_step.append((time.perf_counter() - tq) * 1e3)
    e2e_value = cells * e2e_steps / (time.perf_counter() - t0)
    s.close()
    p32 = ctx(ini32, False)
    p32.run_timed(3)
    ms_plain = p32.run_timed(args.steps)
    p32.close()

    # accuracy against FP64 after the same number of steps from the same state
    acc_steps = args.acc_steps
    out = {}
    for tag, ini, with_mlp in (("fp64", ini64, False), ("fp32", ini32, False),
                               ("fp32_mlp", ini32, True)):
        c = ctx(ini, with_mlp)
        c.run(acc_steps)
        out[tag] = m.interior(c.get_state()).astype(np.float64)
        c.close()
    ref = out.pop("fp64")

    def rel_l1(a):
        ax = (1, 2, 3)
        return float((np.abs(a - ref).sum(axis=ax) / np.abs(ref).sum(axis=ax)).max())

    hbm_peak, peak_kind = load_peaks()
    alg = 64
    achieved = alg * cells / (prof[dom] / 1e3) / 1e9
    step_ms = sum(prof.values())
    hydro = None
    if args.workload == "ot3d_256_fp64" and not args.no_variants and world == 1:
        hydro = hydro_companion(m, local, 10, cpu=not args.no_cpu_baseline)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle_py

        oracle_py.build_oracle()
        nthreads = os.cpu_count() or 1
        o = oracle_py.OracleSolver(ini64, nthreads=nthreads)
        o.set_state(U)
        t0 = time.perf_counter()
        o.run(1)
        el = time.perf_counter() - t0
        o.close()
        cpu = {"value": cells / el, "unit": "cell-updates/s", "cores": nthreads, "kind": "port",
               "sample": f"1 step of the full {n}^3 grid, FP64, oracle/mhd_oracle.c with "
                         f"{nthreads} OpenMP threads ({el:.1f} s)"}
    if rank == 0:
        emit({
            "metric": "MHD cell-updates/s (interior cells), FP32 + HLLD flux surrogate",
            "value": value, "unit": "cell-updates/s", "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+bf16",
            "data": "synthetic: seeded random-phase solenoidal MHD turbulence",
            "config": {"workload": label, "grid": [n] * 3, "cells": cells, "tau": tau,
                       "faces_by_network": used / max(total, 1),
                       "l2": "inputs larger than L2", "per_kernel_ms": prof,
                       "kernels_per_step": len(prof)},
            "accuracy": {"steps": acc_steps, "rel_l1_vs_fp64_fp32_mlp": rel_l1(out["fp32_mlp"]),
                         "rel_l1_vs_fp64_fp32_hlld": rel_l1(out["fp32"])},
            "variants": {"fp32_hlld": {"value": cells * args.steps / (ms_plain / 1e3),
                                       "ms_per_step": ms_plain / args.steps}},
            "e2e": {"value": e2e_value, "unit": "cell-updates/s",
                    "h2d_bytes_per_step": U0.nbytes, "d2h_bytes_per_step": U0.nbytes,
                    "steps": e2e_steps,
                    "call": "mhd_step_host (pinned host buffers, copies inside the timed region; "
                            "uploads and downloads overlap the step slab by slab, one slab "
                            "per 64 MiB of state, at most 16)",
                    "link_gbs": link,
                    "ms_each_step": [round(x, 2) for x in per_step]},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak,
                         "unit": "GB/s", "frac": achieved / hbm_peak,
                         "traffic": load_profile_traffic(args.workload, dom),
                         "peak_source": f"hbm_gbs of {peak_kind}", "algorithmic_bytes_per_cell": alg,
                         "step_achieved": alg * cells / (step_ms / 1e3) / 1e9},
            "clocks": clk.summary(),
            "gpu_launches": len(prof) * args.steps,
            "cpu_baseline": cpu,
        })


def fp64_roofline(workload: str, value: float, kernel: str, exact: bool):
    """FP64-arithmetic roofline of a 3D FP64 line: the reference algorithm's
    FP64 operations per cell-update (additions, multiplications, divisions
    and square roots, each one flop; counted by the oracle compiled with a
    counting scalar, profiles/fp64_ops_ot3d_256.json) times the cell-update
    rate, against 1.26 TFLOP/s (2 DFMA per SM per cycle, 152 SMs, 2.07 GHz;
    an FMA-free build issues at most half of that as separate operations).
    Beside it the FP64-pipe utilisation ncu measured on the kernels."""
    try:
        with open(os.path.join(ROOT, "profiles", "fp64_ops_ot3d_256.json")) as f:
            ops = json.load(f)
    except (OSError, ValueError):
        return None
    per = ops["per_cell_update"]["minimal"]
    peak = float(ops["fp64_peak_tflops"])
    achieved = per["flop"] * value / 1e12
    out = {"bound": "fp64 pipe (2 DFMA/SM/cycle, 1.26 TFLOP/s at 2070 MHz)",
           "flop_per_cell_update": round(per["flop"], 1),
           "div_per_cell_update": round(per["div"], 1),
           "sqrt_per_cell_update": round(per["sqrt"], 1),
           "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
           "source": "oracle/flop_count.py (the reference's operations, minimal halo)"}
    if exact:
        out["fma_free_ceiling_frac"] = 0.5
    a = load_alu_profile(workload.replace("256", "128"))
    if a is not None and not exact:
        out["pipe_active_frac"] = a.get("pipe_active", {}).get(kernel)
        out["pipe_source"] = a.get("source")
    return out


def load_alu_profile(workload: str):
    """FP64-pipe utilisation of the kernels from the committed ncu summary
    (profiles/fp64_pipe_<workload>.json), or None."""
    path = os.path.join(ROOT, "profiles", f"fp64_pipe_{workload}.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


def load_profile_traffic(workload: str, kernel: str):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary (profiles/*.json), or None."""
    path = os.path.join(ROOT, "profiles", f"traffic_{workload}.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return d.get(kernel)
    except (OSError, ValueError):
        return None


# ---------------------------------------------------------------- reference arm

def run_reference(args):
    world, rank, local = dist_setup()
    if rank != 0:
        return
    dim, n, precision, label = WORKLOADS[args.workload]
    nthreads = os.cpu_count() or 1
    steps = args.ref_steps
    if args.workload.startswith("ensemble"):
        from ppkmhd_gb300 import workloads

        v, el, desc = cpu_ensemble_run(workloads.ensemble_specs(512, seed=2024), steps, nthreads)
        emit({"impl": "reference",
              "metric": "MHD cell-updates/s (interior cells), 512-problem 2D ensemble",
              "value": v, "unit": "cell-updates/s", "n_gpus": world, "steps": steps,
              "warmup": 1, "ms_per_step": el * 1e3 / steps, "higher_is_better": True,
              "scaling": "weak", "vs_baseline": None, "dtype": "f64",
              "data": "synthetic: seeded Orszag-Tang ensemble (sizes, B0, Fourier velocity)",
              "config": {"workload": label,
                         "implementation": "CPU port of the reference step (oracle/mhd_oracle.c), "
                                           "problems one at a time, OpenMP"},
              "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": nthreads,
                               "kind": "port", "sample": desc},
              "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                      "d2h_bytes_per_step": 0}})
        return
    if args.workload.startswith("hydro"):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle_py

        oracle_py.build_oracle()
        ini = hydro_bench_ini() if "blast3d" in args.workload else hydro_kh2d_ini()
        o = oracle_py.HydroOracleSolver(ini, nthreads=nthreads)
        import ppkmhd_gb300 as m

        o.set_state(m.initial_state(m.params_from_ini(ini)))
        cells = o.p.nx * o.p.ny * (o.p.nz if dim == 3 else 1)
        t0 = time.perf_counter()
        o.run(max(args.warmup, 1))
        t_one = (time.perf_counter() - t0) / max(args.warmup, 1)
        ns = int(min(steps or args.steps, max(2, 150.0 / max(t_one, 1e-6))))
        t0 = time.perf_counter()
        o.run(ns)
        el = time.perf_counter() - t0
        o.close()
        v = cells * ns / el
        emit({"impl": "reference",
              "metric": "hydro cell-updates/s (interior cells), MUSCL-Hancock hydro step "
                        f"(Hydro_Muscl_{dim}D)",
              "value": v, "unit": "cell-updates/s", "n_gpus": world, "steps": ns,
              "warmup": args.warmup, "ms_per_step": el * 1e3 / ns, "higher_is_better": True,
              "scaling": "weak", "vs_baseline": None, "dtype": "f64",
              "data": "synthetic (the problem's own initial condition)",
              "config": {"workload": label,
                         "implementation": "CPU port of the reference hydro step "
                                           "(oracle/hydro_oracle.c, bitwise equal to the "
                                           "reference functors), OpenMP"},
              "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": nthreads,
                               "kind": "port", "sample": f"{ns} iterations of the full grid "
                                                         f"after {args.warmup} ({el:.1f} s)"},
              "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                      "d2h_bytes_per_step": 0}})
        return
    if steps is None:
        # the GPU arm's K steps after W warm-up steps, unless that exceeds a
        # few minutes of host work (then ~150 s worth, stated in "steps")
        steps = args.steps
    v, el, steps = cpu_baseline_run(args.workload, steps=steps, warmup=args.warmup,
                                    nthreads=nthreads, target_s=150.0)
    emit({
        "impl": "reference",
        "metric": "MHD cell-updates/s (interior cells), plain MUSCL-Hancock+HLLD+CT step",
        "value": v,
        "unit": "cell-updates/s",
        "n_gpus": world,
        "steps": steps,
        "warmup": args.warmup,
        "ms_per_step": el * 1e3 / steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": workload_setup(args.workload, 64)[2],
        "config": {"workload": label, "grid": [n] * dim,
                   "implementation": "CPU port of the reference step (oracle/mhd_oracle.c, "
                                     "bitwise equal to the reference functors), OpenMP"},
        "cpu_baseline": {"value": v, "unit": "cell-updates/s", "cores": nthreads, "kind": "port",
                         "sample": f"{steps} steps of the full {n}^{dim} grid after "
                                   f"{args.warmup} warm-up steps ({el:.1f} s timed)"},
        "e2e": {"value": v, "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    })


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="ot3d_256_fp64", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-steps", type=int, default=None,
                    help="CPU leg iterations (default: about 8 s of host work)")
    ap.add_argument("--ref-steps", type=int, default=None,
                    help="reference-arm iterations (default: about 20 s of host work; 150 "
                         "iterations of the 8-problem sample for the ensemble)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--acc-steps", type=int, default=40,
                    help="steps of the accuracy comparison of the turbulence workload")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--fp-mode", default="exact", choices=["exact", "fast"],
                    help="FP64 build of the headline line (exact: bitwise the reference)")
    args = ap.parse_args()
    if args.cpu_steps is None and args.workload.startswith("ensemble"):
        args.cpu_steps = 150
    if args.ref_steps is None and args.workload.startswith("ensemble"):
        args.ref_steps = 150
    if args.impl == "reference":
        run_reference(args)
    elif args.workload.startswith("ensemble"):
        run_ensemble(args)
    elif args.workload.startswith("turb"):
        run_turbulence(args)
    elif args.workload.startswith("hydro"):
        run_hydro(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
