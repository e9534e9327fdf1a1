"""Builds and runs the drop-in shim's test driver (tests/dropin_host/):
the shim vbm3d_gb300/dropin/vbm3d_dropin.cpp compiled against a stand-in of
the reference's vbm3d.h, linked to the GPU library.  Test infrastructure."""
import os
import shutil
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HOST = os.path.join(ROOT, "tests", "dropin_host")
LIBDIR = os.path.join(ROOT, "vbm3d_gb300", "_build")


def build_driver(outdir):
    from vbm3d_gb300 import build
    build.build()
    cxx = shutil.which("g++")
    if cxx is None:
        return None
    exe = os.path.join(str(outdir), "dropin_driver")
    subprocess.check_call([cxx, "-std=c++11", "-O1", "-Wall", "-Werror", "-I", HOST, "-I", os.path.join(ROOT, "include"),
                           os.path.join(HOST, "dropin_driver.cpp"),
                           os.path.join(ROOT, "vbm3d_gb300", "dropin", "vbm3d_dropin.cpp"),
                           "-L", LIBDIR, "-lvbm3d_gb300", "-Wl,-rpath," + LIBDIR, "-o", exe])
    return exe


def run_driver(exe, workdir, mode, noisy, sigma, fflow=None, bflow=None, basic=None, color_space=True, tag="x"):
    """noisy [F, C, H, W]; flows [frames, channels, H, W] or None.  Returns
    (exit status, first output, second output) with outputs [F, C, H, W]."""
    F, C, H, W = noisy.shape
    inp = os.path.join(str(workdir), "in_%s.bin" % tag)
    out = os.path.join(str(workdir), "out_%s.bin" % tag)
    def shape(fl):  # width, height, frames, channels of a [frames, channels, H, W] flow
        return [0, 0, 0, 0] if fl is None else [fl.shape[3], fl.shape[2], fl.shape[0], fl.shape[1]]

    with open(inp, "wb") as f:
        np.array([W, H, F, C] + shape(fflow) + shape(bflow) + [int(color_space)], np.int32).tofile(f)
        np.array([sigma], np.float32).tofile(f)
        np.ascontiguousarray(noisy, np.float32).tofile(f)
        if mode == "step2":
            np.ascontiguousarray(basic, np.float32).tofile(f)
        for fl in (fflow, bflow):
            if fl is not None:
                np.ascontiguousarray(fl, np.float32).tofile(f)
    res = subprocess.run([exe, mode, inp, out], capture_output=True, text=True)
    a = b = None
    if os.path.exists(out):
        data = np.fromfile(out, np.float32)
        if data.size == 2 * noisy.size:
            a, b = data[:noisy.size].reshape(noisy.shape), data[noisy.size:].reshape(noisy.shape)
    return res.returncode, a, b, res.stderr
