"""The C++ driver (ppkmhd_gb300/lib/ppkmhd_gb300_run, the flow of the
reference's main.cpp): VTK .vti output (IO_VTK.cpp:24-410 layout: ImageData,
cell data, raw appended Float64 arrays with UInt64 byte counts) equal to the
library's state, and a restart from the driver's own checkpoint ending
bitwise where the uninterrupted run ends."""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "ppkmhd_gb300", "lib", "ppkmhd_gb300_run")


def read_vti(path):
    data = open(path, "rb").read()
    head, _, raw = data.partition(b"<AppendedData encoding=\"raw\">")
    text = head.decode()
    ext = [int(x) for x in re.search(r'WholeExtent="([^"]+)"', text).group(1).split()]
    names = re.findall(r'Name="([^"]+)" format="appended" offset="(\d+)"', text)
    start = raw.index(b"_") + 1
    nx, ny, nz = ext[1], ext[3], max(ext[5], 1)
    out = {}
    for name, off in names:
        p = start + int(off)
        nbytes = int(np.frombuffer(raw[p:p + 8], dtype="<u8")[0])
        assert nbytes == nx * ny * nz * 8
        arr = np.frombuffer(raw[p + 8:p + 8 + nbytes], dtype="<f8")
        out[name] = arr.reshape((nz, ny, nx) if ext[5] > 0 else (ny, nx))
    return text, out


def ini_text(outdir, prefix, extra=""):
    return f"""[run]
solver_name=MHD_Muscl_2D
tEnd=0.05
nStepmax=1000
nOutput=2
nlog=0
[mesh]
nx=32
ny=24
boundary_type_xmin=3
boundary_type_xmax=3
boundary_type_ymin=3
boundary_type_ymax=3
[hydro]
gamma0=1.666
cfl=0.8
slope_type=2
problem=orszag_tang
riemann=hlld
smallr=1e-7
smallc=1e-7
[output]
outputDir={outdir}
outputPrefix={prefix}
[OTHER]
implementationVersion=2
{extra}
"""


def run_driver(tmp_path, name, text):
    path = tmp_path / f"{name}.ini"
    path.write_text(text)
    r = subprocess.run([EXE, str(path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


@pytest.mark.gpu
def test_driver_vtk_matches_library_state(mhdlib, tmp_path):
    out = run_driver(tmp_path, "a", ini_text(tmp_path, "ot"))
    assert "Perf" in out
    files = sorted(f for f in os.listdir(tmp_path) if f.endswith(".vti"))
    assert files[0] == "ot_0000000.vti" and len(files) >= 3
    text, fields = read_vti(tmp_path / files[-1])
    assert 'type="ImageData"' in text and 'header_type="UInt64"' in text
    assert 'WholeExtent="0 32 0 24 0 0"' in text
    assert list(fields) == ["rho", "energy", "rho_vx", "rho_vy", "rho_vz", "bx", "by", "bz"]
    # the same run through the library
    s = mhdlib.MHDSolver.from_ini(ini_text(tmp_path, "x"))
    s.init_problem()
    s.run(100000)
    U = mhdlib.interior(s.get_state())
    for v, name in enumerate(fields):
        assert np.array_equal(fields[name], U[v]), name


@pytest.mark.gpu
def test_driver_restart_from_checkpoint(tmp_path):
    run_driver(tmp_path, "full", ini_text(tmp_path, "full", "[gb300]\ncheckpoint=true"))
    ckpts = sorted(f for f in os.listdir(tmp_path) if f.startswith("full") and f.endswith(".ckpt"))
    assert len(ckpts) >= 3
    mid = ckpts[1]
    out = run_driver(tmp_path, "re", ini_text(
        tmp_path, "re", f"[gb300]\ncheckpoint=false\n[run]\nrestart_enabled=1\n"
        f"restart_filename={tmp_path / mid}"))
    assert "restarted run" in out
    last_full = sorted(f for f in os.listdir(tmp_path) if f.startswith("full_") and f.endswith(".vti"))[-1]
    last_re = sorted(f for f in os.listdir(tmp_path) if f.startswith("re_") and f.endswith(".vti"))[-1]
    _, a = read_vti(tmp_path / last_full)
    _, b = read_vti(tmp_path / last_re)
    for name in a:
        assert np.array_equal(a[name], b[name]), name
