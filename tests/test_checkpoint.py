"""Checkpoint / restart (mhd_checkpoint_save / mhd_checkpoint_load): a run
continued from a checkpoint is bitwise the uninterrupted run; the header
carries the grid, precision and time; mismatched or damaged files are
rejected with MHD_ERR_INVALID_ARG."""
import struct

import numpy as np
import pytest

from mhd_cases import ot_ini


HEADER = struct.Struct("<8s8I2dq2i7d")


@pytest.mark.gpu
@pytest.mark.parametrize("dim,precision", [(2, 64), (3, 32), (2, 32)])
def test_restart_continues_bitwise(mhdlib, tmp_path, dim, precision):
    ini = ot_ini(dim=dim, nx=32, ny=24, nz=16, precision=precision)
    a = mhdlib.MHDSolver.from_ini(ini)
    a.init_problem()
    a.run(7)
    path = str(tmp_path / "state.ckpt")
    a.checkpoint_save(path, times_saved=3)
    t7, dt7, _ = a.time()
    a.run(9)
    ref = a.get_state()
    with open(path, "rb") as f:
        h = HEADER.unpack(f.read(HEADER.size))
    # format 2 carries the low parts of the compensated FP32 state
    assert h[0] == b"PPKMHDCK" and h[1] == (2 if precision == 32 else 1) and h[2] == dim
    assert h[3:6] == (32, 24, 16 if dim == 3 else 1)
    assert h[8] == precision // 8 and h[9] == t7 and h[11] == 7 and h[12] == 3
    b = mhdlib.MHDSolver.from_ini(ini)
    assert b.checkpoint_load(path) == 3
    t, _, it = b.time()
    assert t == t7 and it == 0   # iteration count restarts, as in the reference
    b.run(9)
    assert np.array_equal(b.get_state(), ref)
    assert b.time()[0] == a.time()[0]
    # restart_reset_totaltime
    c = mhdlib.MHDSolver.from_ini(ini)
    c.checkpoint_load(path, reset_time=True)
    assert c.time()[0] == 0.0


@pytest.mark.gpu
def test_checkpoint_rejects_mismatch(mhdlib, tmp_path):
    a = mhdlib.MHDSolver.from_ini(ot_ini(dim=2, nx=32))
    a.init_problem()
    path = str(tmp_path / "a.ckpt")
    a.checkpoint_save(path)
    other = mhdlib.MHDSolver.from_ini(ot_ini(dim=2, nx=40))
    with pytest.raises(mhdlib.MHDError) as e:
        other.checkpoint_load(path)
    assert e.value.code == mhdlib.MHD_ERR_INVALID_ARG and "grid" in str(e.value)
    f32 = mhdlib.MHDSolver.from_ini(ot_ini(dim=2, nx=32, precision=32))
    with pytest.raises(mhdlib.MHDError) as e:
        f32.checkpoint_load(path)
    assert "precision" in str(e.value)
    data = open(path, "rb").read()
    open(path, "wb").write(data[: len(data) // 2])
    with pytest.raises(mhdlib.MHDError) as e:
        a.checkpoint_load(path)
    assert "truncated" in str(e.value)
    with pytest.raises(mhdlib.MHDError):
        a.checkpoint_load(str(tmp_path / "missing.ckpt"))


def _upscale_reference(Uc, dim, g=3):
    """copy_buffer with restart_upscale (IO_HDF5.h:1603-1694), restated:
    fine cell i <- coarse (i + g) // 2 per axis; the face-centred normal field
    averages the two coarse faces where i + g is odd."""
    Uc = np.asarray(Uc)
    fine_shape = tuple(2 * (n - 2 * g) + 2 * g for n in Uc.shape[1:])
    idx = [(np.arange(n) + g) // 2 for n in fine_shape]
    grids = np.meshgrid(*idx, indexing="ij")
    par = [((np.arange(n) + g) % 2) for n in fine_shape]
    U = np.empty((8,) + fine_shape, dtype=Uc.dtype)
    for v in range(8):
        U[v] = Uc[v][tuple(grids)]
    # axes of the [var][k][j][i] arrays: x is the last one
    axes = {5: dim, 6: dim - 1, 7: dim - 2}
    for v, ax in axes.items():
        if v == 7 and dim == 2:
            continue
        odd = par[ax - 1].astype(bool)
        shifted = [g_.copy() for g_ in grids]
        shifted[ax - 1] = shifted[ax - 1] + 1
        avg = (Uc[v][tuple(grids)] + Uc[v][tuple(shifted)]) / 2
        m = odd.reshape([-1 if a == ax - 1 else 1 for a in range(dim)])
        U[v] = np.where(m, avg, U[v])
    return U


@pytest.mark.gpu
@pytest.mark.parametrize("dim,precision", [(2, 64), (3, 64), (3, 32)])
def test_restart_upscale_from_half_resolution(mhdlib, tmp_path, dim, precision):
    coarse = mhdlib.MHDSolver.from_ini(ot_ini(dim=dim, nx=16, ny=12, nz=10, precision=precision))
    coarse.init_problem()
    coarse.run(5)
    path = str(tmp_path / "coarse.ckpt")
    coarse.checkpoint_save(path, times_saved=2)
    Uc = coarse.get_state()
    t5 = coarse.time()[0]
    fine = mhdlib.MHDSolver.from_ini(ot_ini(dim=dim, nx=32, ny=24, nz=20, precision=precision))
    assert fine.checkpoint_load_upscaled(path) == 2
    assert fine.time()[0] == t5
    expect = _upscale_reference(Uc, dim)
    got = fine.get_state()
    # interior cells as the reference's copy_buffer builds them (the ghost
    # cells are refilled by the boundary conditions)
    assert np.array_equal(mhdlib.interior(got), mhdlib.interior(expect))
    # the averaged face field keeps the discrete divergence at round-off
    _, _, divb_max = fine.diagnostics()
    assert divb_max < (1e-12 if precision == 64 else 1e-4), divb_max
    assert fine.run(3) == 3
    # a same-size context refuses the half-resolution file, and vice versa
    with pytest.raises(mhdlib.MHDError):
        fine.checkpoint_load(path)
    with pytest.raises(mhdlib.MHDError):
        coarse.checkpoint_load_upscaled(path)
