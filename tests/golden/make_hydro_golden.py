"""Regenerate the hydro-solver golden fixtures in tests/golden/ from the
REFERENCE.

Runs ppkMHD's own hydro MUSCL functors (SolverHydroMuscl<2>/<3>,
src/muscl/Hydro*.h, src/shared/RiemannSolvers.h), compiled through the
Kokkos-API shim into oracle/_ref/libppkmhd_ref64.so (oracle/build_ref.sh,
oracle/ref_harness_hydro.cpp), serially, on small cases:

  hydro_<case>.npz   the init functor's output (ghost cells included, before
                     the boundary fill) and the gravity field it writes, the
                     interior after 1 and after n iterations, t and dt along
                     the way; perturbed cases add a seeded smooth
                     perturbation to the initial state
  hydro_riemann.npz  riemann_hydro fluxes (approx, llf, hll, hllc; 2D and 3D
                     states) for random and edge-case face states

usage (from the repository root, where the reference tree is present):
    oracle/build_ref.sh && python tests/golden/make_hydro_golden.py
"""
from __future__ import annotations

import ctypes
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle_py as op  # noqa: E402
from mhd_cases import hydro_ini, hydro_perturbed as perturbed  # noqa: E402

SQUARE = "xmin=-0.5\nxmax=0.5\nymin=-0.5\nymax=0.5\nzmin=-0.5\nzmax=0.5"
# name, hydro_ini kwargs, iterations, perturbation seed (None: the plain init)
CASES = [
    ("implode2d", dict(dim=2), 10, None),
    ("implode2d_v1", dict(dim=2, version=1), 10, None),
    ("implode2d_pert", dict(dim=2, bc=(1, 2, 3, 3)), 8, 41),
    ("implode2d_llf", dict(dim=2, riemann="llf"), 8, 42),
    ("implode2d_hll", dict(dim=2, riemann="hll", version=1), 8, 43),
    ("implode2d_hllc", dict(dim=2, riemann="hllc"), 8, 44),
    ("implode2d_slope1", dict(dim=2, slope_type="1", bc=(2, 2, 1, 1)), 8, None),
    ("blast2d_slope0", dict(dim=2, problem="blast", slope_type="0", extra="[blast]\nradius=0.2\n"), 8, None),
    ("blast2d_reflect", dict(dim=2, problem="blast", bc=(1, 1, 1, 1), extra="[blast]\nradius=0.25\n"), 10, None),
    ("kh2d", dict(dim=2, problem="kelvin_helmholtz", riemann="hllc"), 8, None),
    ("gresho2d", dict(dim=2, problem="gresho_vortex", mesh=SQUARE), 8, None),
    ("isentropic2d", dict(dim=2, problem="isentropic_vortex",
                          mesh="xmin=-5\nxmax=5\nymin=-5\nymax=5"), 8, None),
    ("fourquad2d", dict(dim=2, problem="four_quadrant", bc=(2, 2, 2, 2),
                        extra="[riemann2d]\nconfig_number=3\nx=0.5\ny=0.5\n"), 8, None),
    ("rt2d_gravity", dict(dim=2, problem="rayleigh_taylor", gravity=True, bc=(3, 3, 1, 1)), 10, None),
    ("rb2d_gravity_v1", dict(dim=2, problem="rising_bubble", gravity=True, riemann="hllc",
                             version=1, bc=(1, 1, 2, 2)), 10, None),
    ("implode2d_gravity_zero", dict(dim=2, gravity=True), 6, None),
    ("implode3d", dict(dim=3, nx=12), 5, None),
    ("implode3d_v1_pert", dict(dim=3, nx=12, version=1, bc=(1, 2, 3, 3, 2, 1)), 4, 51),
    ("implode3d_llf", dict(dim=3, nx=10, riemann="llf"), 4, 52),
    ("implode3d_hllc", dict(dim=3, nx=10, riemann="hllc"), 4, 53),
    ("blast3d", dict(dim=3, nx=12, problem="blast", bc=(2, 2, 2, 2, 2, 2),
                     extra="[blast]\nradius=0.3\n"), 5, None),
    ("kh3d", dict(dim=3, nx=10, problem="kelvin_helmholtz", riemann="hllc"), 4, None),
    ("gresho3d", dict(dim=3, nx=10, problem="gresho_vortex", mesh=SQUARE), 4, None),
    ("rt3d_gravity", dict(dim=3, nx=10, problem="rayleigh_taylor", gravity=True,
                          bc=(3, 3, 3, 3, 1, 1),
                          extra="[rayleigh_taylor]\ngy=0.0\ngz=-0.1\n"), 5, None),
    # version 1 in 3D gives the right state of z faces no gravity predictor
    ("rb3d_gravity_v1", dict(dim=3, nx=10, problem="rising_bubble", gravity=True, version=1,
                             riemann="llf", bc=(2, 2, 1, 1, 2, 2)), 5, None),
    ("rb3d_gravity_v0", dict(dim=3, nx=10, problem="rising_bubble", gravity=True, version=0,
                             riemann="llf", bc=(2, 2, 1, 1, 2, 2)), 5, None),
    # the disk: point-source gravity field written by the init functor
    ("disk2d_point", dict(dim=2, nx=32, ny=32, problem="disk", mesh=SQUARE, bc=(2, 2, 2, 2),
                          extra="[gravity]\npoint=true\n"), 8, None),
    ("disk2d_static_v1", dict(dim=2, nx=30, ny=34, problem="disk", mesh=SQUARE, riemann="hllc",
                              version=1, bc=(2, 2, 2, 2),
                              extra="[gravity]\nstatic=true\nG=2.0\nsoften=0.05\nx=0.01\n"
                                    "[disk]\nradius=0.2\n"), 8, None),
    ("disk3d_point_v1", dict(dim=3, nx=14, ny=16, nz=12, problem="disk", mesh=SQUARE,
                             version=1, riemann="llf", bc=(2, 2, 2, 2, 2, 2),
                             extra="[gravity]\npoint=true\nz=0.05\n"), 5, None),
]


def make_case(name, kw, nsteps, seed):
    ini = hydro_ini(**kw)
    U0 = op.ref_initial_state(ini)
    r = op.RefSolver(ini)
    if seed is not None:
        U0 = perturbed(U0, seed)
    r.set_state(U0)
    g = r.ghost
    t, dt, it = [], [], []

    def stamp():
        a, b, c = r.time()
        t.append(a)
        dt.append(b)
        it.append(c)

    stamp()
    r.run(1)
    U1 = op.interior(r.get_state(), g)
    stamp()
    r.run(nsteps - 1)
    Un = op.interior(r.get_state(), g)
    stamp()
    np.savez_compressed(os.path.join(HERE, f"hydro_{name}.npz"), ini=ini, U0=U0, U1=U1, Un=Un,
                        nsteps=nsteps, t=np.array(t), dt=np.array(dt), perturbed=seed is not None,
                        gravity=op.ref_hydro_gravity_field(ini))
    return dict(case=name, nsteps=nsteps, shape=list(U0.shape))


def make_riemann():
    rng = np.random.default_rng(7)
    L = op.ref_probe_lib(64)
    out = {}
    for dim in (2, 3):
        nv = dim + 2
        n = 400
        qL = np.empty((n, nv))
        qR = np.empty((n, nv))
        for q in (qL, qR):
            q[:, 0] = np.exp(rng.uniform(-6, 3, n))        # rho
            q[:, 1] = np.exp(rng.uniform(-8, 4, n))        # p
            q[:, 2:] = rng.normal(0, 2, (n, nv - 2))       # velocities
        # edge cases: equal states, vacuum-like, pressure below the floor,
        # strong rarefaction, zero velocities, negative density
        qL[:8] = qR[:8]
        qL[8:16, 0] = 1e-12
        qR[16:24, 1] = -1.0
        qL[24:32, 2] = -30.0
        qR[24:32, 2] = 30.0
        qL[32:40, 2:] = 0.0
        qR[32:40, 2:] = 0.0
        qL[40:44, 0] = -1.0
        out[f"qL{dim}"] = qL
        out[f"qR{dim}"] = qR
        for solver in ("approx", "llf", "hll", "hllc"):
            if dim == 3 and solver == "hll":
                continue
            ini = hydro_ini(dim=dim, nx=8, riemann=solver).encode()
            F = np.zeros((n, nv))
            rp = ctypes.POINTER(ctypes.c_double)
            for q in range(n):
                l = np.ascontiguousarray(qL[q])
                r = np.ascontiguousarray(qR[q])
                f = np.zeros(nv)
                L.ref_hydro_riemann(ini, l.ctypes.data_as(rp), r.ctypes.data_as(rp),
                                    f.ctypes.data_as(rp))
                F[q] = f
            out[f"{solver}{dim}"] = F
    np.savez_compressed(os.path.join(HERE, "hydro_riemann.npz"), **out)


def main():
    if not op.ref_available(64):
        sys.exit("build oracle/_ref first (oracle/build_ref.sh)")
    manifest = [make_case(*c) for c in CASES]
    make_riemann()
    with open(os.path.join(HERE, "HYDRO_MANIFEST.json"), "w") as f:
        json.dump(manifest, f, indent=1)
    print(f"{len(manifest)} hydro cases + hydro_riemann.npz")


if __name__ == "__main__":
    main()
