"""The block-matching kernel divides each squared-difference sum by the
patch norm k^2 C with a multiply and one correction step instead of a
division (div_norm, vbm3d_gb300/csrc/bm2_impl.cuh).  Block matching must
reproduce the reference's float quotient (src/vbm3d.cpp:1010), so this test
checks the formula against IEEE division for every float the kernel sends
through it (2^-100 up to FLT_MAX), for the four norms of the staged kernel:
49 and 147 (k = 7, one or three channels), 64 and 192 (k = 8).  Runs on the
CPU: the C library's fmaf and the float operations here round once, as the
kernel's __fmaf_rn / __fmul_rn do."""
import os
import platform
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_div_norm_exact_for_every_float(tmp_path):
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("gcc not found")
    exe = str(tmp_path / "div_norm_check")
    flags = ["-O2", "-ffp-contract=off", "-fopenmp"]
    if platform.machine() in ("x86_64", "AMD64"):
        flags.append("-mfma")  # hardware fmaf (otherwise the C library's software FMA, just slower)
    subprocess.check_call([cc, *flags, os.path.join(HERE, "div_norm_check.c"), "-lm", "-o", exe])
    out = subprocess.check_output([exe, "49", "147", "64", "192"], text=True, timeout=600)
    res = {float(a): int(b) for a, b in (line.split() for line in out.strip().splitlines())}
    assert res == {49.0: 0, 147.0: 0, 64.0: 0, 192.0: 0}, res
