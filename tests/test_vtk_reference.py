"""The .vti writer (mhd_write_vtk, ppkmhd_gb300/host/IO_VTK.cpp) against the
reference's own save_VTK_2D / save_VTK_3D (src/utils/io/IO_VTK.cpp:24-410),
compiled through the Kokkos-API shim into oracle/_ref: the same state and
.ini give the same file, byte for byte, in 2D and 3D, raw appended binary
and ASCII.  Host only (no device); skipped where oracle/_ref is not built
(the reference tree is absent)."""
import os

import numpy as np
import pytest

from mhd_cases import ot_ini


def _ini(dim, nx, ny, nz, outdir, prefix, ascii_):
    base = ot_ini(dim=dim, nx=nx, ny=ny, nz=nz)
    return base + ("\n[output]\n"
                   f"outputDir={outdir}\n"
                   f"outputPrefix={prefix}\n"
                   f"outputVtkAscii={'true' if ascii_ else 'false'}\n")


@pytest.mark.parametrize("dim,ascii_", [(2, False), (3, False), (2, True), (3, True)])
def test_vti_bytes_equal_reference_writer(mhdlib, oracle, tmp_path, dim, ascii_):
    if not oracle.ref_available(64):
        pytest.skip("oracle/_ref not built (reference sources absent)")
    nx, ny, nz = 13, 9, 7
    g = 3
    shape = (8, ny + 2 * g, nx + 2 * g) if dim == 2 else (8, nz + 2 * g, ny + 2 * g, nx + 2 * g)
    rng = np.random.default_rng(5 + dim)
    U = rng.standard_normal(shape) * np.array([1, 2, 3, 4, 5, 6, 7, 8]).reshape(
        (8,) + (1,) * (len(shape) - 1))
    mine_dir, ref_dir = tmp_path / "mine", tmp_path / "ref"
    mine_dir.mkdir()
    ref_dir.mkdir()
    name = mhdlib.write_vtk(_ini(dim, nx, ny, nz, str(mine_dir), "run", ascii_), U, 12)
    assert name.endswith("run_0000012.vti") and os.path.exists(name)
    oracle.ref_save_vtk(_ini(dim, nx, ny, nz, str(ref_dir), "run", ascii_), U, 12)
    ref = ref_dir / "run_0000012.vti"
    assert ref.exists()
    a, b = open(name, "rb").read(), ref.read_bytes()
    assert len(a) == len(b) and a == b


@pytest.mark.parametrize("dim,ascii_", [(2, False), (3, True)])
def test_vti_bytes_equal_reference_writer_hydro(mhdlib, oracle, tmp_path, dim, ascii_):
    """The same for a hydro-only solver state (dim + 2 variables, ghost 2)."""
    if not oracle.ref_available(64):
        pytest.skip("oracle/_ref not built (reference sources absent)")
    from mhd_cases import hydro_ini

    nx, ny, nz = 11, 8, 6
    g, nv = 2, dim + 2
    shape = (nv, ny + 2 * g, nx + 2 * g) if dim == 2 else (nv, nz + 2 * g, ny + 2 * g, nx + 2 * g)
    U = np.random.default_rng(9 + dim).standard_normal(shape)

    def ini(outdir):
        return hydro_ini(dim=dim, nx=nx, ny=ny, nz=nz) + (
            f"\n[output]\noutputDir={outdir}\noutputPrefix=h\n"
            f"outputVtkAscii={'true' if ascii_ else 'false'}\n")

    mine_dir, ref_dir = tmp_path / "mine", tmp_path / "ref"
    mine_dir.mkdir()
    ref_dir.mkdir()
    name = mhdlib.write_vtk(ini(str(mine_dir)), U, 3)
    oracle.ref_save_vtk(ini(str(ref_dir)), U, 3)
    assert open(name, "rb").read() == (ref_dir / "h_0000003.vti").read_bytes()
