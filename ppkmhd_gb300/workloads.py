"""Seeded synthetic workloads: .ini texts and initial states (numpy, FP64,
LayoutLeft ``[var][k][j][i]`` with ghost cells).

* ``ot_ini``: the reference's Orszag-Tang settings (HLLD, slope_type 2,
  periodic; the keys of HydroParams::setup, HydroParams.cpp:27-217).
* ``perturbed_ot_3d``: the 3D Orszag-Tang state with a seeded uniform
  velocity perturbation (density kept, energy recomputed).
* ``ensemble_specs`` / ``ensemble_problem``: the ensemble of 2D Orszag-Tang
  problems of uneven size: N_p = round(exp(U(ln 64, ln 512))), B0_p =
  U(0.5, 1.5) / sqrt(4 pi), plus a random-phase Fourier velocity
  perturbation on the modes 1 <= |k|_inf <= 4 scaled to an rms of 5 % of
  v0 = 1.  The Orszag-Tang fields follow MHDInitFunctors2D.h:241-389 with B0
  replaced by B0_p.
* ``kelvin_helmholtz``: a 2D magnetised shear layer (periodic x, reflecting
  y): rho = 1 for |y - 0.5| < 0.25 and 2 outside, vx = +-0.5 with tanh
  smoothing of width 0.01, p = 2.5, Bx = 0.1, gamma = 1.4, and a seeded vy
  perturbation of amplitude 0.01 localised at the two interfaces.  The
  reference's own Kelvin-Helmholtz functor (MHDInitFunctors2D.h:420-560) fixes
  Bx = 0.5 and uses its own perturbation; this variant is injected through
  the state interface.
* ``turbulence_3d``: random-phase solenoidal velocity and field on the
  periodic cube (E(k) ~ k^-2 on 1 <= |k| <= 8, rms v = 1, rms B = 0.5,
  rho = p = 1), B the discrete curl of an edge vector potential.

All states include ghost cells; set_state refills them from the interior
with the boundary conditions, so their content does not matter.
"""
from __future__ import annotations

import math

import numpy as np

ID, IP, IU, IV, IW, IA, IB, IC = range(8)
GHOST = 3


def ot_ini(dim: int = 2, nx: int = 64, ny: int | None = None, nz: int | None = None, *,
           cfl: str = "0.8", gamma0: str = "1.666", tend: str = "100.0", nstepmax: int = 1000000,
           riemann: str = "hlld", slope_type: str = "2", bc=(3, 3, 3, 3, 3, 3),
           precision: int | None = None, fp_mode: str | None = None, version: int = 2,
           problem: str = "orszag_tang", xmax: str = "1.0", ymax: str = "1.0",
           zmax: str = "1.0") -> str:
    """A reference-style .ini text (values parsed like ConfigMap: floats through strtof)."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    small = "1e-7" if dim == 2 else "1e-8"
    lines = ["[run]", f"solver_name=MHD_Muscl_{dim}D", f"tEnd={tend}", f"nStepmax={nstepmax}",
             "nOutput=0", "nlog=0", "", "[mesh]", f"nx={nx}", f"ny={ny}",
             f"xmax={xmax}", f"ymax={ymax}"]
    if dim == 3:
        lines += [f"nz={nz}", f"zmax={zmax}"]
    names = ["xmin", "xmax", "ymin", "ymax", "zmin", "zmax"]
    for f in range(6 if dim == 3 else 4):
        lines.append(f"boundary_type_{names[f]}={bc[f]}")
    lines += ["", "[hydro]", f"gamma0={gamma0}", f"cfl={cfl}", "niter_riemann=10", "iorder=2",
              f"slope_type={slope_type}", f"problem={problem}", f"riemann={riemann}",
              f"smallr={small}", f"smallc={small}", "", "[OTHER]",
              f"implementationVersion={version}"]
    if precision is not None or fp_mode is not None:
        lines += ["", "[gb300]"]
        if precision is not None:
            lines.append(f"precision={precision}")
        if fp_mode is not None:
            lines.append(f"fp_mode={fp_mode}")
    return "\n".join(lines) + "\n"


def f32(x: str) -> float:
    """A parameter value as the reference reads it (strtof, then widened)."""
    return float(np.float32(float(x)))


def _centres(n: int, lo: float = 0.0, hi: float = 1.0):
    d = (hi - lo) / n
    return lo + d / 2 + (np.arange(n + 2 * GHOST) - GHOST) * d


def _energy_2d(U: np.ndarray, eint: np.ndarray | float) -> None:
    """U[IP] = internal energy + kinetic + magnetic with cell-centred B
    (face averages), on every cell but the last column/row."""
    bx = U[IA, :, :-1] + U[IA, :, 1:]
    by = U[IB, :-1, :] + U[IB, 1:, :]
    rho = U[ID]
    kin = 0.5 * (U[IU] ** 2 + U[IV] ** 2 + U[IW] ** 2) / rho
    mag = np.zeros_like(rho)
    mag[:, :-1] += 0.125 * bx ** 2
    mag[:-1, :] += 0.125 * by ** 2
    mag += 0.5 * U[IC] ** 2
    U[IP] = eint + kin + mag


def orszag_tang_2d(nx: int, ny: int | None = None, gamma0: float = f32("1.666"),
                   b0_scale: float = 1.0, dv: tuple | None = None) -> np.ndarray:
    """2D Orszag-Tang (MHDInitFunctors2D.h:241-389) with B0 = b0_scale / sqrt(4 pi)
    and an optional velocity perturbation (dvx, dvy) on the ghost-inclusive grid."""
    ny = nx if ny is None else ny
    TWOPI = 2 * math.pi
    B0 = b0_scale / math.sqrt(2 * TWOPI)
    p0 = gamma0 / (2 * TWOPI)
    d0 = gamma0 * p0
    x = _centres(nx)[None, :]
    y = _centres(ny)[:, None]
    U = np.zeros((8, ny + 2 * GHOST, nx + 2 * GHOST))
    vx = -np.sin(y * TWOPI) + 0 * x
    vy = np.sin(x * TWOPI) + 0 * y
    if dv is not None:
        vx = vx + dv[0]
        vy = vy + dv[1]
    U[ID] = d0
    U[IU] = d0 * vx
    U[IV] = d0 * vy
    U[IA] = -B0 * np.sin(y * TWOPI) + 0 * x
    U[IB] = B0 * np.sin(2.0 * x * TWOPI) + 0 * y
    _energy_2d(U, p0 / (gamma0 - 1.0))
    return U


def fourier_velocity(nx: int, ny: int, rng: np.random.Generator, kmax: int = 4,
                     rms: float = 0.05):
    """Random-phase sum of the periodic modes 1 <= max(|kx|, |ky|) <= kmax (one
    of each +-k pair), unit amplitude per mode, independent phases per
    component, scaled so that sqrt(<dvx^2 + dvy^2>) over the interior = rms."""
    TWOPI = 2 * math.pi
    x = _centres(nx)[None, :]
    y = _centres(ny)[:, None]
    modes = [(kx, ky) for kx in range(0, kmax + 1) for ky in range(-kmax, kmax + 1)
             if max(abs(kx), abs(ky)) >= 1 and (kx > 0 or ky > 0)]
    out = []
    for _ in range(2):
        f = np.zeros((ny + 2 * GHOST, nx + 2 * GHOST))
        for (kx, ky) in modes:
            f += np.cos(TWOPI * (kx * x + ky * y) + rng.uniform(0, TWOPI))
        out.append(f)
    g = GHOST
    norm = math.sqrt(float(np.mean(out[0][g:-g, g:-g] ** 2 + out[1][g:-g, g:-g] ** 2)))
    return out[0] * (rms / norm), out[1] * (rms / norm)


def ensemble_specs(n: int = 512, seed: int = 2024, nmin: int = 64, nmax: int = 512):
    """Per problem: size N (N x N interior), B0 scale and the seed of its
    perturbation, drawn from one seeded generator."""
    rng = np.random.default_rng(seed)
    sizes = np.rint(np.exp(rng.uniform(math.log(nmin), math.log(nmax), n))).astype(int)
    scales = rng.uniform(0.5, 1.5, n)
    seeds = rng.integers(0, 2 ** 31 - 1, n)
    return [dict(n=int(sizes[q]), b0_scale=float(scales[q]), seed=int(seeds[q])) for q in range(n)]


def ensemble_problem(spec: dict, precision: int | None = None, fp_mode: str | None = None,
                     cfl: str = "0.8"):
    """(.ini text, FP64 LayoutLeft state) of one ensemble problem."""
    n = spec["n"]
    ini = ot_ini(2, n, cfl=cfl, precision=precision, fp_mode=fp_mode)
    rng = np.random.default_rng(spec["seed"])
    dv = fourier_velocity(n, n, rng)
    return ini, orszag_tang_2d(n, b0_scale=spec["b0_scale"], dv=dv)


def perturbed_ot_3d(U: np.ndarray, seed: int = 1234, amp: float = 1e-3,
                    gamma0: float = f32("1.666")) -> np.ndarray:
    """Seeded uniform(-amp, amp) velocity perturbation of every cell of a 3D
    Orszag-Tang state, density kept, total energy recomputed with the
    perturbed kinetic energy (internal and magnetic energy unchanged)."""
    rng = np.random.default_rng(seed)
    U = U.copy()
    rho = U[ID]
    kin0 = 0.5 * (U[IU] ** 2 + U[IV] ** 2 + U[IW] ** 2) / rho
    for v in (IU, IV, IW):
        U[v] = U[v] + rho * rng.uniform(-amp, amp, rho.shape)
    kin1 = 0.5 * (U[IU] ** 2 + U[IV] ** 2 + U[IW] ** 2) / rho
    U[IP] = U[IP] - kin0 + kin1
    return U


def kh_ini(n: int, precision: int | None = 32, fp_mode: str | None = None, cfl: str = "0.8",
           tend: str = "100.0") -> str:
    return ot_ini(2, n, cfl=cfl, gamma0="1.4", tend=tend, bc=(3, 3, 1, 1, 3, 3),
                  precision=precision, fp_mode=fp_mode, problem="kelvin_helmholtz")


def kelvin_helmholtz(n: int, seed: int = 7, gamma0: float = f32("1.4")) -> np.ndarray:
    """Magnetised Kelvin-Helmholtz shear layer on [0,1]^2, n x n interior."""
    rng = np.random.default_rng(seed)
    x = _centres(n)[None, :]
    y = _centres(n)[:, None]
    w = 0.01
    inner = 0.5 * (np.tanh((y - 0.25) / w) - np.tanh((y - 0.75) / w))  # 1 inside, 0 outside
    rho = 2.0 - inner + 0 * x
    vx = (-0.5 + inner) + 0 * x  # +0.5 inside, -0.5 outside
    env = np.exp(-((y - 0.25) / 0.05) ** 2) + np.exp(-((y - 0.75) / 0.05) ** 2)
    TWOPI = 2 * math.pi
    phase = rng.uniform(0, TWOPI, 4)
    amp = rng.uniform(0.5, 1.0, 4)
    pert = sum(amp[m] * np.sin(TWOPI * (m + 1) * x + phase[m]) for m in range(4))
    pert = pert / np.max(np.abs(pert))
    vy = 0.01 * env * pert
    U = np.zeros((8, n + 2 * GHOST, n + 2 * GHOST))
    U[ID] = rho
    U[IU] = rho * vx
    U[IV] = rho * vy
    U[IA] = 0.1
    _energy_2d(U, 2.5 / (gamma0 - 1.0))
    return U


def turbulence_3d(n: int, seed: int = 11, kmin: float = 1.0, kmax: float = 8.0,
                  vrms: float = 1.0, brms: float = 0.5, rho: float = 1.0, p: float = 1.0,
                  gamma0: float = f32("1.6666666666666667"), dtype=np.float64) -> np.ndarray:
    """Random-phase solenoidal velocity and field on the periodic unit cube,
    spectrum E(k) ~ k^-2 on kmin <= |k| <= kmax (mode amplitudes ~ |k|^-2),
    rms |v| = vrms and rms |B| (face values) = brms, uniform rho and p.

    The velocity is projected onto divergence-free modes.  The face-centred
    field is the discrete curl of an edge-centred vector potential, so its
    discrete divergence vanishes to round-off."""
    from numpy.fft import fftfreq, irfftn, rfftfreq

    rng = np.random.default_rng(seed)
    k1 = fftfreq(n) * n
    kz = k1[:, None, None]
    ky = k1[None, :, None]
    kx = (rfftfreq(n) * n)[None, None, :]
    kk = np.sqrt(kx ** 2 + ky ** 2 + kz ** 2)
    band = (kk >= kmin) & (kk <= kmax)
    kk_safe = np.where(kk > 0, kk, 1.0)
    shape = kk.shape

    def random_vector(power):
        comps = [band * kk_safe ** power * np.exp(2j * np.pi * rng.random(shape))
                 * rng.standard_normal(shape) for _ in range(3)]
        return comps

    # velocity (cell values), solenoidal projection
    vx, vy, vz = random_vector(-2.0)
    kdotv = (kx * vx + ky * vy + kz * vz) / kk_safe ** 2
    vhat = [vx - kx * kdotv, vy - ky * kdotv, vz - kz * kdotv]
    v = [irfftn(c, s=(n, n, n), axes=(0, 1, 2)) for c in vhat]
    del vx, vy, vz, kdotv, vhat
    norm = vrms / np.sqrt(np.mean(v[0] ** 2 + v[1] ** 2 + v[2] ** 2))
    v = [c * norm for c in v]

    # vector potential on edges (|A| ~ |k|^-3): Ax at (x+h/2, y, z), Ay at
    # (x, y+h/2, z), Az at (x, y, z+h/2), grid points x = i / n
    ax, ay, az = random_vector(-3.0)
    half = np.pi / n  # 2 pi k * (h/2) with h = 1/n
    A = [irfftn(ax * np.exp(1j * half * kx), s=(n, n, n), axes=(0, 1, 2)),
         irfftn(ay * np.exp(1j * half * ky), s=(n, n, n), axes=(0, 1, 2)),
         irfftn(az * np.exp(1j * half * kz), s=(n, n, n), axes=(0, 1, 2))]
    del ax, ay, az
    h = 1.0 / n

    def d(f, axis):  # forward difference along axis (0 = z, 1 = y, 2 = x), periodic
        return (np.roll(f, -1, axis=axis) - f) / h

    Ax, Ay, Az = A
    Bx = d(Az, 1) - d(Ay, 0)   # at (x_i, y_{j+1/2}, z_{k+1/2})
    By = d(Ax, 0) - d(Az, 2)   # at (x_{i+1/2}, y_j, z_{k+1/2})
    Bz = d(Ay, 2) - d(Ax, 1)   # at (x_{i+1/2}, y_{j+1/2}, z_k)
    del A, Ax, Ay, Az
    bnorm = brms / np.sqrt(np.mean(Bx ** 2 + By ** 2 + Bz ** 2))
    Bx, By, Bz = Bx * bnorm, By * bnorm, Bz * bnorm

    g = GHOST
    U = np.zeros((8, n + 2 * g, n + 2 * g, n + 2 * g), dtype=dtype)
    sl = (slice(g, -g),) * 3
    U[(ID,) + sl] = rho
    for comp, var in zip(v, (IU, IV, IW)):
        U[(var,) + sl] = rho * comp
    for comp, var in zip((Bx, By, Bz), (IA, IB, IC)):
        U[(var,) + sl] = comp
    bcx = 0.5 * (Bx + np.roll(Bx, -1, axis=2))
    bcy = 0.5 * (By + np.roll(By, -1, axis=1))
    bcz = 0.5 * (Bz + np.roll(Bz, -1, axis=0))
    U[(IP,) + sl] = (p / (gamma0 - 1.0) + 0.5 * rho * (v[0] ** 2 + v[1] ** 2 + v[2] ** 2)
                     + 0.5 * (bcx ** 2 + bcy ** 2 + bcz ** 2))
    return U
