"""Configuration builders shared by the tests (no reference files are read).

The Orszag-Tang settings follow the reference's shipped parity fixtures
(settings/test_mhd_orszag_tang_{2D,3D}.ini): HLLD, slope_type 2, CFL 0.8,
gamma0 "1.666", smallr = smallc = 1e-7 (2D) / 1e-8 (3D), periodic.
"""
from __future__ import annotations


def ot_ini(dim: int = 2, nx: int = 32, ny: int | None = None, nz: int | None = None,
           riemann: str = "hlld", slope_type: str = "2", bc=(3, 3, 3, 3, 3, 3),
           gamma0: str = "1.666", cfl: str = "0.8", tend: str = "10.0", nstepmax: int = 1000,
           version: int = 2, precision: int | None = None, fp_mode: str | None = None,
           zmax: str = "1.0") -> str:
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    small = "1e-7" if dim == 2 else "1e-8"
    lines = [
        "[run]",
        f"solver_name=MHD_Muscl_{dim}D",
        f"tEnd={tend}",
        f"nStepmax={nstepmax}",
        "nOutput=0",
        "nlog=0",
        "",
        "[mesh]",
        f"nx={nx}",
        f"ny={ny}",
    ]
    if dim == 3:
        lines += [f"nz={nz}", f"zmax={zmax}"]
    names = ["xmin", "xmax", "ymin", "ymax", "zmin", "zmax"]
    for f in range(6 if dim == 3 else 4):
        lines.append(f"boundary_type_{names[f]}={bc[f]}")
    lines += [
        "",
        "[hydro]",
        f"gamma0={gamma0}",
        f"cfl={cfl}",
        "niter_riemann=10",
        "iorder=2",
        f"slope_type={slope_type}",
        "problem=orszag_tang",
        f"riemann={riemann}",
        f"smallr={small}",
        f"smallc={small}",
        "",
        "[OTHER]",
        f"implementationVersion={version}",
    ]
    if precision is not None or fp_mode is not None:
        lines += ["", "[gb300]"]
        if precision is not None:
            lines.append(f"precision={precision}")
        if fp_mode is not None:
            lines.append(f"fp_mode={fp_mode}")
    return "\n".join(lines) + "\n"


def perturb(U, seed: int, amp: float = 0.05):
    """Seeded perturbation of momentum and energy of a LayoutLeft state."""
    import numpy as np

    rng = np.random.default_rng(seed)
    U = U.copy()
    U[2:5] += amp * rng.standard_normal(U[2:5].shape) * U[0]
    U[1] += 2 * amp * np.abs(rng.standard_normal(U[1].shape))
    return U


def hydro_ini(dim: int = 2, nx: int = 24, ny: int | None = None, nz: int | None = None,
              problem: str = "implode", riemann: str = "approx", slope_type: str = "2",
              bc=(3, 3, 3, 3, 3, 3), gamma0: str = "1.4", cfl: str = "0.8", version: int = 0,
              tend: str = "10.0", nstepmax: int = 1000, gravity: bool = False,
              mesh: str = "", extra: str = "") -> str:
    """A .ini for the hydro-only MUSCL solver (Hydro_Muscl_2D/3D)."""
    ny = nx + 3 if ny is None else ny
    nz = nx - 2 if nz is None else nz
    names = ["xmin", "xmax", "ymin", "ymax", "zmin", "zmax"]
    lines = ["[run]", f"solver_name=Hydro_Muscl_{dim}D", f"tEnd={tend}", f"nStepmax={nstepmax}",
             "nOutput=0", "nlog=0", "", "[mesh]", f"nx={nx}", f"ny={ny}"]
    if dim == 3:
        lines.append(f"nz={nz}")
    lines += [f"boundary_type_{names[f]}={bc[f]}" for f in range(6 if dim == 3 else 4)]
    lines += [mesh, "", "[hydro]", f"gamma0={gamma0}", f"cfl={cfl}", f"riemann={riemann}",
              f"problem={problem}", f"slope_type={slope_type}", "smallr=1e-8", "smallc=1e-8", "",
              "[OTHER]", f"implementationVersion={version}", ""]
    if gravity:
        lines += ["[gravity]", "static=true", ""]
    return "\n".join(lines) + "\n" + extra


def hydro_perturbed(U0, seed: int):
    """A smooth seeded perturbation of a hydro state: up to 5 % on density
    and energy, 0.05 on the momenta (the state stays physical)."""
    import numpy as np

    rng = np.random.default_rng(seed)
    U = U0.copy()
    grids = np.meshgrid(*[np.linspace(0, 2 * np.pi, n) for n in U.shape[1:]], indexing="ij")
    for v in range(U.shape[0]):
        ph = rng.uniform(0, 2 * np.pi, len(grids))
        wave = np.prod([np.sin((q + 1) * g + p) for q, (g, p) in enumerate(zip(grids, ph))], axis=0)
        if v in (0, 1):
            U[v] *= 1.0 + 0.05 * wave
        else:
            U[v] += 0.05 * wave
    return U
