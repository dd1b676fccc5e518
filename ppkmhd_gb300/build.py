"""Build the in-tree CUDA library ``ppkmhd_gb300/lib/libppkmhd_gb300.so``.

nvcc compiles for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``),
one translation unit per arithmetic variant and solver plus the host layer, in
parallel; g++ links.  No CMake, no torch extension machinery: the library
exposes the plain C ABI of include/ppkmhd_gb300.h.

usage: python -m ppkmhd_gb300.build [--jobs N] [--force]
"""
from __future__ import annotations

import argparse
import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
OBJ = os.path.join(PKG, "build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libppkmhd_gb300.so")
EXE = os.path.join(LIBDIR, "ppkmhd_gb300_run")

GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-ffp-contract=off", "--prec-div=true", "--prec-sqrt=true",
               "-I", os.path.join(ROOT, "include"), "-I", CSRC]
CXX_COMMON = ["-std=c++17", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall",
              "-I", os.path.join(ROOT, "include"), "-I", CSRC, "-I", HOST]

VARIANTS = [
    # tag, real type, factory, fmad
    ("v_f64x", "double", "create_core_f64x", "false"),
    ("v_f64", "double", "create_core_f64", "true"),
    ("v_f32", "float", "create_core_f32", "true"),
]

HOST_SOURCES = ["ConfigMap.cpp", "HydroParams.cpp", "SolverBase.cpp", "SolverFactory.cpp",
                "SolverMHDMusclGPU.cpp", "IO_VTK.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))


def _sources_digest() -> str:
    h = hashlib.sha256()
    for d in (CSRC, HOST, os.path.join(ROOT, "include")):
        for name in sorted(os.listdir(d)):
            p = os.path.join(d, name)
            if os.path.isfile(p):
                h.update(name.encode())
                with open(p, "rb") as f:
                    h.update(f.read())
    h.update(" ".join(GENCODE + NVCC_COMMON + CXX_COMMON).encode())
    return h.hexdigest()


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(jobs: int | None = None, force: bool = False, verbose: bool = False) -> str:
    """Compile everything (skipped when sources are unchanged); returns the library path."""
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    stamp = os.path.join(OBJ, "sources.sha256")
    digest = _sources_digest()
    if (not force and os.path.exists(LIB) and os.path.exists(stamp)
            and open(stamp).read() == digest):
        return LIB
    jobs = jobs or min(8, os.cpu_count() or 4)
    cmds = []
    objs = []
    for tag, real, factory, fmad in VARIANTS:
        o = os.path.join(OBJ, f"mhd_{tag}.o")
        objs.append(o)
        cmds.append([nvcc(), *GENCODE, *NVCC_COMMON, f"--fmad={fmad}", "-Xptxas", "-v",
                     f"-DMHD_VARIANT_TAG={tag}", f"-DMHD_REAL={real}", f"-DMHD_FACTORY={factory}",
                     f"-DMHD_EXACT_BUILD={1 if fmad == 'false' else 0}",
                     "-c", os.path.join(CSRC, "mhd_variant.cu"), "-o", o])
        o = os.path.join(OBJ, f"hydro_{tag}.o")
        objs.append(o)
        cmds.append([nvcc(), *GENCODE, *NVCC_COMMON, f"--fmad={fmad}", "-Xptxas", "-v",
                     f"-DMHD_VARIANT_TAG={tag}", f"-DMHD_REAL={real}",
                     f"-DMHD_HYDRO_FACTORY={factory.replace('create_core', 'create_hydro_core')}",
                     f"-DMHD_EXACT_BUILD={1 if fmad == 'false' else 0}",
                     "-c", os.path.join(CSRC, "hydro_variant.cu"), "-o", o])
        o = os.path.join(OBJ, f"mhd_ensemble_{tag}.o")
        objs.append(o)
        cmds.append([nvcc(), *GENCODE, *NVCC_COMMON, f"--fmad={fmad}", "-Xptxas", "-v",
                     f"-DMHD_VARIANT_TAG={tag}", f"-DMHD_REAL={real}",
                     f"-DMHD_ENSEMBLE_FACTORY={factory.replace('create_core', 'create_ensemble')}",
                     f"-DMHD_EXACT_BUILD={1 if fmad == 'false' else 0}",
                     "-c", os.path.join(CSRC, "mhd_ensemble.cu"), "-o", o])
    o = os.path.join(OBJ, "mhd_mlp.o")
    objs.append(o)
    cmds.append([nvcc(), *GENCODE, *NVCC_COMMON, "--fmad=true", "-Xptxas", "-v",
                 "-c", os.path.join(CSRC, "mhd_mlp.cu"), "-o", o])
    o = os.path.join(OBJ, "mhd_noalloc.o")
    objs.append(o)
    cmds.append([nvcc(), *GENCODE, *NVCC_COMMON, "--fmad=true", "-Xptxas", "-v",
                 "-c", os.path.join(CSRC, "mhd_noalloc.cu"), "-o", o])
    for src in ("mhd_capi.cpp", "mhd_init.cpp", "hydro_init.cpp"):
        o = os.path.join(OBJ, src.replace(".cpp", ".o"))
        objs.append(o)
        cmds.append(["g++", *CXX_COMMON, "-c", os.path.join(CSRC, src), "-o", o])
    for src in HOST_SOURCES:
        o = os.path.join(OBJ, src.replace(".cpp", ".o"))
        objs.append(o)
        cmds.append(["g++", *CXX_COMMON, "-I", os.path.join(cuda_home(), "include"),
                     "-c", os.path.join(HOST, src), "-o", o])
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        logs = list(ex.map(_run, cmds))
    with open(os.path.join(OBJ, "ptxas.log"), "w") as f:
        f.write("\n".join(logs))
    cudalib = os.path.join(cuda_home(), "lib64")
    tmp = LIB + ".tmp"
    _run(["g++", "-shared", "-o", tmp, *objs, "-L", cudalib, "-Wl,-rpath," + cudalib,
          "-lcudart", "-fopenmp"])
    os.replace(tmp, LIB)
    _run(["g++", *CXX_COMMON, os.path.join(HOST, "main.cpp"), "-o", EXE, "-L", LIBDIR,
          "-Wl,-rpath,$ORIGIN", "-lppkmhd_gb300", "-L", cudalib, "-Wl,-rpath," + cudalib,
          "-lcudart"])
    with open(stamp, "w") as f:
        f.write(digest)
    if verbose:
        print("\n".join(logs))
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    print(build(a.jobs, a.force, a.verbose))
    sys.exit(0)
