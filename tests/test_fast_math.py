"""Accuracy of the fast builds' FP64 reciprocal and square root.

The fast FP64 build replaces the library's correctly rounded reciprocal by
one third-order Newton step on the hardware approximation and the IEEE
square root by one third-order Householder correction of x times the
hardware reciprocal-square-root approximation
(ppkmhd_gb300/csrc/mhd_physics.cuh).  This test compiles
tests/fast_math_kernels.cu against that header and checks their error bounds
on 2^20 log-uniform arguments over [1e-30, 1e30] against correctly rounded
host references, and that the arguments outside the fast ranges (zeros,
subnormals, |x| >= 2^1021, infinities, NaN, negative square-root arguments)
get exactly the library function's result; and that the exact build's
integer comparison (exact_gt) answers as the FP comparison on every pair of
those special values, and that its Alfven-speed maximum with one quotient
(alfven_max5_exact) equals the four-quotient maximum bit for bit on 2^20
random, tied, nearly tied and special operand sets.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.gpu
def test_fast_fp64_reciprocal_and_sqrt_error_bounds(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "fast_math_kernels")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", exe,
                    os.path.join(HERE, "fast_math_kernels.cu")], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=300).stdout
    res, special = {}, {}
    for line in out.splitlines():
        f = line.split()
        if f[0].startswith("special_"):
            special[f[0][8:]] = (int(f[2]), int(f[4]))
        else:
            res[f[0]] = (float(f[2]), float(f[4]))
    assert set(special) == {"rcp", "fsqrt", "gt", "alfven"}, out
    for name, (bad, total) in special.items():
        assert total > 900 and bad == 0, (name, bad, total)
    # library references: correctly rounded (rsqrt within its documented bound)
    assert res["drcp_rn"][0] <= 0.5 and res["sqrt"][0] <= 0.5
    assert res["rsq"][0] <= 0.52
    # fast reciprocal: relative error e0^3 of the seed on top of one rounding
    assert res["rcp"][0] <= 0.52 and res["rcp"][1] >= 0.999
    # square root: the seed's relative error e0 leaves 2.5 e0^3 after the
    # correction, on top of the roundings of s = x y and the final FMA
    print({k: v[0] for k, v in res.items()})
    assert res["fsqrt"][0] <= 0.8 and res["fsqrt"][1] >= 0.5
