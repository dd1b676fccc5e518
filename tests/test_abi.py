"""C-ABI library: loads, exports every declared symbol, parses .ini like
the reference, validates arguments, and reports a missing GPU cleanly.
No compute calls are made here (CPU-only machine)."""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ppkmhd_gb300.h")
GOLDEN = os.path.join(ROOT, "tests", "golden")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mhd_[a-z_0-9]+)\s*\(", src)))


def test_header_declares_expected_api():
    names = declared_functions()
    for n in ("mhd_create", "mhd_destroy", "mhd_step", "mhd_run", "mhd_set_state",
              "mhd_get_state", "mhd_params_from_ini", "mhd_diagnostics", "mhd_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol(mhdlib):
    out = subprocess.run(["nm", "-D", "--defined-only", mhdlib.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT\s+(mhd_\w+)", out))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    # and the Python binding knows every one of them
    assert set(declared_functions()) == set(mhdlib.SIGNATURES)


def test_version_string(mhdlib):
    assert b"sm_103a" in mhdlib.lib().mhd_version()


def test_params_from_ini_matches_reference(mhdlib):
    z = np.load(os.path.join(GOLDEN, "params.npz"))
    for name, ini, ref in zip(z["names"], z["inis"], z["values"]):
        p = mhdlib.params_from_ini(str(ini))
        gamma0, cfl, slope, smallr, smallc = p.gamma0, p.cfl, p.slope_type, p.smallr, p.smallc
        assert [gamma0, cfl, slope, smallr, smallc] == list(ref[:5]), name
        assert p.tEnd == ref[9], name
        assert (p.xmax - p.xmin) / p.nx == ref[6], name


def test_ini_parsing_rules(mhdlib):
    ini = ("[RUN]\nSOLVER_NAME=MHD_Muscl_3D ; comment\nnStepmax=5\n   77\ntEnd=2.5;x\n"
           "[mesh]\nnx=0x10\nny=12\nnz=8\nboundary_type_xmin=1\nboundary_type_zmax=2\n"
           "[hydro]\ngamma0=1.4\nriemann=llf\n[OTHER]\nimplementationVersion=2\n"
           "[gb300]\nprecision=32\n")
    p = mhdlib.params_from_ini(ini)
    assert p.dim == 3 and p.nx == 16 and p.ny == 12 and p.nz == 8
    # an indented line replaces the previous key's value; ';' without a
    # preceding space is not a comment, so strtof reads "2.5" and stops
    assert p.nStepmax == 77
    assert p.tEnd == 2.5
    assert list(p.boundary) == [1, 1, 1, 1, 1, 2]
    assert p.riemann == mhdlib.MHD_RIEMANN_LLF
    assert p.precision == 32
    assert p.gamma0 == float(np.float32(1.4))


def test_unknown_solver_is_a_parse_error(mhdlib):
    # the MOOD and spectral-difference solvers are not part of this library
    for name in ("Hydro_Mood_2D", "Hydro_SDM_3D", "unknown"):
        with pytest.raises(mhdlib.MHDError) as e:
            mhdlib.params_from_ini(f"[run]\nsolver_name={name}\n")
        assert e.value.code == mhdlib.MHD_ERR_PARSE


@pytest.mark.parametrize("field,value", [("dim", 4), ("ghost", 2), ("nx", 2), ("riemann", 0),
                                         ("implementation_version", 3), ("precision", 16),
                                         ("gamma0", 1.0)])
def test_create_rejects_bad_parameters(mhdlib, field, value):
    p = mhdlib.default_params()
    p.nx = p.ny = 16
    setattr(p, field, value)
    with pytest.raises(mhdlib.MHDError) as e:
        mhdlib.MHDSolver(p)
    assert e.value.code == mhdlib.MHD_ERR_INVALID_ARG


def test_grid_size_limit(mhdlib):
    """Kernels index inside an array with 32-bit offsets: ghost-inclusive
    cells x 8 variables must stay below 4e9 (806^3 x 8 = 4.19e9 is refused
    before any device work; 3 cells per direction is the smallest grid)."""
    p = mhdlib.default_params()
    p.dim, p.nx, p.ny, p.nz = 3, 800, 800, 800
    with pytest.raises(mhdlib.MHDError) as e:
        mhdlib.MHDSolver(p)
    assert e.value.code == mhdlib.MHD_ERR_INVALID_ARG and "too large" in str(e.value)
    p.nx = p.ny = p.nz = 2
    with pytest.raises(mhdlib.MHDError) as e:
        mhdlib.MHDSolver(p)
    assert e.value.code == mhdlib.MHD_ERR_INVALID_ARG


def test_fp32_exact_is_rejected(mhdlib):
    p = mhdlib.default_params()
    p.nx = p.ny = 16
    p.precision, p.fp_mode = mhdlib.MHD_FP32, mhdlib.MHD_FP_EXACT
    with pytest.raises(mhdlib.MHDError):
        mhdlib.MHDSolver(p)


def test_null_arguments_do_not_crash(mhdlib):
    L = mhdlib.lib()
    assert L.mhd_create(None, None) == mhdlib.MHD_ERR_INVALID_ARG
    assert L.mhd_step(None) == mhdlib.MHD_ERR_INVALID_ARG
    assert L.mhd_destroy(None) == mhdlib.MHD_ERR_INVALID_ARG
    assert L.mhd_last_error(None) == b"null context"


def test_no_gpu_is_reported(mhdlib):
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    p = mhdlib.default_params()
    p.nx = p.ny = 16
    with pytest.raises(mhdlib.MHDError) as e:
        mhdlib.MHDSolver(p)
    assert e.value.code == mhdlib.MHD_ERR_NO_DEVICE
