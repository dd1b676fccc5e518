"""Regenerate the golden fixtures in tests/golden/ from the REFERENCE.

Runs ppkMHD's own MHD functors, compiled through the Kokkos-API shim into
oracle/_ref/libppkmhd_ref64.so (oracle/build_ref.sh), serially, on small
seeded cases, and stores inputs and outputs as .npz:

  steps_*.npz    initial interior + ghosts state, interior state after
                 n steps, t and dt (2D/3D, HLLD/HLL/LLF, slope types,
                 periodic/reflecting/outflow boundaries, perturbed states)
  riemann.npz    face fluxes of riemann_mhd for random and edge-case states
  emf.npz        compute_emf<EMFX/Y/Z> for random edge states
  params.npz     HydroParams fields parsed from .ini texts

  problem_*.npz  other initial conditions of SolverMHDMuscl<dim>::init
                 (blast, implode, Kelvin-Helmholtz, rotor, field loop,
                 linear wave): init-functor output, state after the
                 boundary fill, interior state after n steps

usage (from the repository root, where the reference tree is present):
    oracle/build_ref.sh && python tests/golden/make_golden.py [steps|problems|riemann|emf|params ...]
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle_py as op  # noqa: E402
from mhd_cases import ot_ini, perturb  # noqa: E402

STEP_CASES = [
    # name, ini kwargs, steps, perturbation seed (None = plain Orszag-Tang)
    ("ot2d_hlld", dict(dim=2, nx=24, ny=20), 12, None),
    ("ot2d_hlld_pert", dict(dim=2, nx=24, ny=20), 8, 11),
    ("ot2d_hll", dict(dim=2, nx=16, ny=18, riemann="hll"), 6, 12),
    ("ot2d_llf", dict(dim=2, nx=16, ny=18, riemann="llf"), 6, 13),
    ("ot2d_slope1", dict(dim=2, nx=16, ny=16, slope_type="1"), 6, 14),
    ("ot2d_bc_mixed", dict(dim=2, nx=20, ny=16, bc=(1, 2, 2, 1, 3, 3)), 8, 15),
    ("ot3d_hlld", dict(dim=3, nx=10, ny=12, nz=9), 5, None),
    ("ot3d_hlld_pert", dict(dim=3, nx=10, ny=12, nz=9), 4, 21),
    ("ot3d_hll", dict(dim=3, nx=8, ny=9, nz=10, riemann="hll"), 3, 22),
    ("ot3d_llf", dict(dim=3, nx=8, ny=9, nz=10, riemann="llf"), 3, 23),
    ("ot3d_bc_mixed", dict(dim=3, nx=9, ny=8, nz=10, bc=(1, 2, 3, 3, 2, 1)), 4, 24),
    # implementation versions 0 and 1 (trace + stored states; v0 is the
    # default of the reference's 3D Orszag-Tang .ini)
    ("v0_ot2d_hlld", dict(dim=2, nx=20, ny=18, version=0), 8, None),
    ("v0_ot2d_pert", dict(dim=2, nx=16, ny=14, version=0, bc=(1, 2, 3, 3, 3, 3)), 6, 31),
    ("v1_ot2d_pert", dict(dim=2, nx=16, ny=14, version=1), 6, 32),
    ("v0_ot3d_hlld", dict(dim=3, nx=12, ny=12, nz=6, zmax="0.25", version=0), 4, None),
    ("v0_ot3d_pert", dict(dim=3, nx=9, ny=10, nz=8, version=0, riemann="hll"), 3, 33),
    ("v1_ot3d_pert", dict(dim=3, nx=9, ny=8, nz=10, version=1, bc=(3, 3, 1, 2, 3, 3)), 3, 34),
]


def make_steps():
    for name, kw, nsteps, seed in STEP_CASES:
        ini = ot_ini(**kw)
        r = op.RefSolver(ini)
        U0 = r.get_state()
        if seed is not None:
            U0 = perturb(U0, seed)
            r.set_state(U0)
        t0, dt0, _ = r.time()
        r.run(1)
        U1 = op.interior(r.get_state())
        t1, dt1, _ = r.time()
        r.run(nsteps - 1)
        Un = op.interior(r.get_state())
        tn, dtn, itn = r.time()
        np.savez_compressed(os.path.join(HERE, f"steps_{name}.npz"), ini=np.array(ini), U0=U0,
                            U1=U1, Un=Un, nsteps=nsteps, t=np.array([t0, t1, tn]),
                            dt=np.array([dt0, dt1, dtn]), perturbed=seed is not None)
        print(f"steps_{name}: {nsteps} steps, t={tn:.6f}")


# Other problems of SolverMHDMuscl<dim>::init through the reference's own
# init functors (settings of the reference's .ini files, smaller grids).
def problem_ini(dim, n, problem, section="", bc=3, gamma0="1.666", cfl="0.8", version=2,
                mesh="", nsteps=1000) -> str:
    nx, ny = n[0], n[1]
    lines = ["[run]", f"solver_name=MHD_Muscl_{dim}D", "tEnd=10.0", f"nStepmax={nsteps}",
             "nOutput=0", "", "[mesh]", f"nx={nx}", f"ny={ny}"]
    if dim == 3:
        lines.append(f"nz={n[2]}")
    for f in ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax")[: 2 * dim]:
        lines.append(f"boundary_type_{f}={bc}")
    lines += [mesh, "", "[hydro]", f"gamma0={gamma0}", f"cfl={cfl}", "niter_riemann=10",
              "iorder=2", "slope_type=2", f"problem={problem}", "riemann=hlld", "smallr=1e-8",
              "smallc=1e-8", "", section, "", "[OTHER]", f"implementationVersion={version}"]
    return "\n".join(lines) + "\n"


PROBLEM_CASES = [
    # name, ini, steps
    ("rotor2d", problem_ini(2, (32, 32), "rotor", "[rotor]\nr0=0.1\nr1=0.115\nu0=1.0\np0=1.5",
                            bc=2, gamma0="1.4", cfl="0.4"), 8),
    ("rotor2d_v0", problem_ini(2, (24, 24), "rotor", "[rotor]\nr0=0.1\nr1=0.115\nu0=1.0\np0=1.5",
                               bc=2, gamma0="1.4", cfl="0.4", version=0), 6),
    ("blast2d", problem_ini(2, (24, 36), "blast", "[blast]\ndensity_in=1.0\ndensity_out=1.2",
                            mesh="xmin=0.0\nxmax=1.0\nymin=0.0\nymax=1.5"), 8),
    ("implode2d", problem_ini(2, (24, 24), "implode", "", bc=1, gamma0="1.4"), 8),
    ("field_loop2d", problem_ini(2, (32, 16), "field_loop",
                                 "[FieldLoop]\nradius=0.3\namplitude=0.001\nvflow=3",
                                 gamma0="1.4", cfl="0.4",
                                 mesh="xmin=-1.0\nxmax=1.0\nymin=-0.5\nymax=0.5"), 8),
    ("kh2d", problem_ini(2, (24, 24), "kelvin_helmholtz",
                         "[kh]\namplitude=0.01\nperturbation_sine_robertson=1\nmode=2\n"
                         "w0=0.1\ndelta=0.02\nd_in=2.0\nd_out=1.0\npressure=2.5"), 6),
    ("kh2d_sine", problem_ini(2, (20, 20), "kelvin_helmholtz",
                              "[kh]\nperturbation_sine=1\nperturbation_sine_robertson=0\n"
                              "mode=1\nw0=0.05\nd_in=2.0\nd_out=1.0\npressure=2.5"), 6),
    ("blast3d", problem_ini(3, (12, 12, 12), "blast", ""), 4),
    # (from its third step on the reference's own 3D rotor produces NaN
    # states at this size, and round-off-level differences can bring that
    # forward by a step; mhd_run reports MHD_ERR_NUMERIC there)
    ("rotor3d", problem_ini(3, (12, 12, 6), "rotor", "", bc=2, gamma0="1.4", cfl="0.4"), 1),
    ("implode3d", problem_ini(3, (10, 10, 10), "implode", "[implode]\nshape_region=1", bc=1,
                              gamma0="1.4"), 3),
    ("field_loop3d", problem_ini(3, (16, 8, 8), "field_loop",
                                 "[FieldLoop]\nradius=0.3\namplitude=0.001\nvflow=3",
                                 cfl="0.4", mesh="xmin=-1.0\nxmax=1.0\nymin=-0.5\nymax=0.5\n"
                                 "zmin=-0.5\nzmax=0.5"), 4),
    ("kh3d", problem_ini(3, (10, 10, 10), "kelvin_helmholtz",
                         "[kh]\nperturbation_sine_robertson=1\nmode=2\nw0=0.1\ndelta=0.05\n"
                         "d_in=2.0\nd_out=1.0\npressure=2.5"), 3),
    ("wave3d_fast", problem_ini(3, (16, 8, 8), "wave", "[wave]\ntype=0\namplitude=1e-6",
                                gamma0="1.6666666667", cfl="0.4",
                                mesh="xmax=3.0\nymax=1.5\nzmax=1.5"), 4),
    ("wave3d_alfven", problem_ini(3, (16, 8, 8), "wave", "[wave]\ntype=1\namplitude=1e-6",
                                  gamma0="1.6666666667", cfl="0.4",
                                  mesh="xmax=3.0\nymax=1.5\nzmax=1.5"), 4),
    ("unknown_is_ot", problem_ini(2, (16, 16), "FieldLoop", ""), 3),
]


def make_problems():
    for name, ini, nsteps in PROBLEM_CASES:
        Uinit = op.ref_initial_state(ini)
        r = op.RefSolver(ini)
        U0 = r.get_state()
        t0, dt0, _ = r.time()
        r.run(nsteps)
        Un = op.interior(r.get_state())
        tn, dtn, itn = r.time()
        np.savez_compressed(os.path.join(HERE, f"problem_{name}.npz"), ini=np.array(ini),
                            Uinit=Uinit, U0=U0, Un=Un, nsteps=nsteps, t=np.array([t0, tn]),
                            dt=np.array([dt0, dtn]))
        print(f"problem_{name}: {nsteps} steps, t={tn:.6f}")


def riemann_states(rng, n):
    """Random normal-frame states plus edge cases (degenerate HLLD branch,
    zero normal field, supersonic left/right flows)."""
    qs = []
    for _ in range(n):
        q = np.empty(8)
        q[0] = rng.uniform(0.05, 2.0)
        q[1] = rng.uniform(0.01, 2.0)
        q[2:5] = rng.normal(0, 1.0, 3)
        q[5:8] = rng.normal(0, 0.7, 3)
        qs.append(q)
    return np.array(qs)


def make_riemann():
    rng = np.random.default_rng(7)
    L = riemann_states(rng, 200)
    R = riemann_states(rng, 200)
    # edge cases
    ext_L, ext_R = [], []
    base = np.array([1.0, 1.0, 0.0, 0.0, 0.0, 0.5, 0.3, -0.2])
    ext_L.append(base.copy()); ext_R.append(base.copy())          # identical states
    a = base.copy(); a[5] = 0.0
    ext_L.append(a.copy()); ext_R.append(a * [1.2, 0.8, 1, 1, 1, 1, -1, 1])  # Bn = 0
    s = base.copy(); s[2] = 8.0
    ext_L.append(s.copy()); ext_R.append(s.copy())                # supersonic to the right
    s = base.copy(); s[2] = -8.0
    ext_L.append(s.copy()); ext_R.append(s.copy())                # supersonic to the left
    d = base.copy(); d[6] = 1e-12; d[7] = 0.0
    ext_L.append(d.copy()); ext_R.append(d * [0.9, 1.1, 1, 1, 1, 1, 1, 1])  # near-degenerate
    L = np.vstack([L, ext_L])
    R = np.vstack([R, ext_R])
    out = {}
    lib = op.ref_probe_lib(64)
    for solver in ("hlld", "hll", "llf"):
        ini = ot_ini(dim=2, nx=8, riemann=solver).encode()
        F = np.zeros_like(L)
        for n in range(len(L)):
            l = L[n].copy(); r = R[n].copy(); f = np.zeros(8)
            lib.ref_riemann(ini, l.ctypes.data_as(op._dp), r.ctypes.data_as(op._dp),
                            f.ctypes.data_as(op._dp))
            F[n] = f
        out[solver] = F
    np.savez_compressed(os.path.join(HERE, "riemann.npz"), qL=L, qR=R, **out,
                        ini_hlld=np.array(ot_ini(dim=2, nx=8, riemann="hlld")))
    print("riemann: %d state pairs x 3 solvers" % len(L))


def make_emf():
    rng = np.random.default_rng(9)
    n = 300
    Q = np.empty((n, 4, 8))
    Q[..., 0] = rng.uniform(0.05, 2.0, (n, 4))
    Q[..., 1] = rng.uniform(0.01, 2.0, (n, 4))
    Q[..., 2:5] = rng.normal(0, 1.0, (n, 4, 3))
    Q[..., 5:8] = rng.normal(0, 0.7, (n, 4, 3))
    # a slice with strong uniform advection to visit every region of the solver
    Q[:60, :, 2] += rng.choice([-6.0, 6.0], (60, 1))
    Q[30:90, :, 3] += rng.choice([-6.0, 6.0], (60, 1))
    lib = op.ref_probe_lib(64)
    ini_text = ot_ini(dim=3, nx=8)
    ini = ini_text.encode()
    E = np.zeros((n, 3))
    for m in range(n):
        for d in range(3):
            q = np.ascontiguousarray(Q[m])
            E[m, d] = lib.ref_compute_emf(ini, d, q.ctypes.data_as(op._dp))
    np.savez_compressed(os.path.join(HERE, "emf.npz"), qEdge=Q, emf=E, ini=np.array(ini_text))
    print("emf: %d edges x 3 directions" % n)


PARAM_INIS = {
    "ot2d_shipped_values": ot_ini(dim=2, nx=256),
    "ot3d": ot_ini(dim=3, nx=64, ny=64, nz=16, zmax="0.25", gamma0="1.666"),
    "gamma_5_3": ot_ini(dim=2, nx=128, gamma0="1.6666666666666667", cfl="0.8"),
    "odd_spacing": ot_ini(dim=2, nx=100, ny=30, cfl="0.45", slope_type="1"),
    "case_and_comments": (
        "[RUN]\nSolver_Name = MHD_Muscl_2D ; inline comment\ntEnd=0.5\n# comment\n"
        "[MESH]\nnx = 0x20\nny=24\nxmin=-0.5\nxmax=0.5\n[Hydro]\ngamma0 = 1.4\ncfl=0.7\n"
        "smallr=1e-9\nsmallc=1e-9\nriemann=hll\n[other]\nimplementationVersion=2\n"),
}


def make_params():
    lib = op.ref_probe_lib(64)
    rows = {}
    for name, ini in PARAM_INIS.items():
        out = np.zeros(10)
        lib.ref_params(ini.encode(), out.ctypes.data_as(op._dp))
        rows[name] = out
    np.savez_compressed(os.path.join(HERE, "params.npz"),
                        names=np.array(list(rows)), values=np.array(list(rows.values())),
                        inis=np.array(list(PARAM_INIS.values())),
                        fields=np.array(["gamma0", "cfl", "slope_type", "smallr", "smallc",
                                         "smallp", "dx", "dy", "dz", "tEnd"]))
    print("params: %d ini texts" % len(rows))


if __name__ == "__main__":
    if not op.ref_available(64):
        sys.exit("oracle/_ref/libppkmhd_ref64.so missing: run oracle/build_ref.sh first")
    parts = sys.argv[1:] or ["steps", "problems", "riemann", "emf", "params"]
    for part in parts:
        {"steps": make_steps, "problems": make_problems, "riemann": make_riemann,
         "emf": make_emf, "params": make_params}[part]()
    with open(os.path.join(HERE, "MANIFEST.json"), "w") as f:
        json.dump(sorted(n for n in os.listdir(HERE) if n.endswith(".npz")), f, indent=1)
