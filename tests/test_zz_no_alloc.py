"""The allocation-free step-1 entry point (vbm3d_gpu_step1_noalloc), for
callers that cannot let the library allocate device memory: it must give the
results of vbm3d_gpu_step1, call after call, with its fixed table, and the
device's free memory must not drop during a call.

Collected last on purpose: a failure here comes after every other test ran.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import vbm3d_gb300 as vb  # noqa: E402
from vbm3d_gb300._abi import Dims  # noqa: E402
from vbm3d_gb300.synth import make_clip  # noqa: E402

TOL = 1e-3  # max |difference| of num / den on the 0-255 scale, as in the parity tests


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from vbm3d_gb300 import build
    build.build()
    L = vb.load()
    vp = C.c_void_p
    L.vbm3d_gpu_step1_noalloc.argtypes = [C.POINTER(vb.Params), vp, vp, vp, Dims, C.c_float, C.c_int, vp, vp, vp]
    return L


def call(fn, p, noisy, sigma, cs, num, den):
    f, c, h, w = noisy.shape
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    return fn(C.byref(p), C.c_void_p(noisy.data_ptr()), None, None, Dims(w, h, f, c), sigma, int(cs),
              C.c_void_p(num.data_ptr()), C.c_void_p(den.data_ptr()), stream)


def ratio(num, den, fb):
    return np.where(den == 0, fb, num / np.where(den == 0, 1, den))


@pytest.mark.parametrize("shape,sigma,cs", [((96, 80, 6, 3), 25.0, True), ((120, 72, 7, 1), 20.0, False)])
def test_noalloc_matches_step1_twice(lib, shape, sigma, cs):
    w, h, f, c = shape
    _, noisy_np, _, _ = make_clip(w, h, f, c, sigma, seed=2024)
    noisy = torch.from_numpy(noisy_np).cuda()
    p = vb.default_params(1, sigma)
    ref_num, ref_den = torch.empty_like(noisy), torch.empty_like(noisy)
    assert call(lib.vbm3d_gpu_step1, p, noisy, sigma, cs, ref_num, ref_den) == 0, lib.vbm3d_last_error()
    torch.cuda.synchronize()
    want = ratio(ref_num.cpu().numpy(), ref_den.cpu().numpy(), noisy_np)
    for _ in range(2):  # the fixed table keeps the previous call's contents
        num = torch.full_like(noisy, 7.0)
        den = torch.full_like(noisy, 7.0)
        assert call(lib.vbm3d_gpu_step1_noalloc, p, noisy, sigma, cs, num, den) == 0, lib.vbm3d_last_error()
        torch.cuda.synchronize()
        got = ratio(num.cpu().numpy(), den.cpu().numpy(), noisy_np)
        assert np.abs(got - want).max() <= TOL
        np.testing.assert_allclose(den.cpu().numpy(), ref_den.cpu().numpy(), rtol=1e-5, atol=1e-9)


def test_noalloc_rejects_oversized_calls(lib):
    # 1920x1080 RGB step 1: 57,600 reference patches per frame, 9 table
    # words each; 17 frames exceed the 8 Mi-word table.
    p = vb.default_params(1, 30.0)
    f, c, h, w = 17, 3, 1080, 1920
    fake = C.c_void_p(256)  # never dereferenced: the size check comes first
    rc = lib.vbm3d_gpu_step1_noalloc(C.byref(p), fake, None, None, Dims(w, h, f, c), 30.0, 1, fake, fake, None)
    assert rc == 2 and b"exceed" in lib.vbm3d_last_error()


# Run in a fresh process, so that no earlier test's allocations hide one.
# The kernels are warmed up first (vbm3d_gpu_step1 on a small clip, then
# vbm3d_gpu_step1_noalloc on it, which loads the module holding the fixed
# table); then one call on three 1080p RGB frames, whose 6.2 MB table a
# pool allocation would have to reserve anew.
FREE_MEMORY_PROBE = r"""
import ctypes as C, sys, torch
sys.path.insert(0, sys.argv[1])
import vbm3d_gb300 as vb
from vbm3d_gb300._abi import Dims
L = vb.load()
vp = C.c_void_p
for fn in (L.vbm3d_gpu_step1, L.vbm3d_gpu_step1_noalloc):
    fn.argtypes = [C.POINTER(vb.Params), vp, vp, vp, Dims, C.c_float, C.c_int, vp, vp, vp]
def call(fn, x, num, den):
    f, c, h, w = x.shape
    p = vb.default_params(1, 30.0)
    rc = fn(C.byref(p), vp(x.data_ptr()), None, None, Dims(w, h, f, c), 30.0, 1, vp(num.data_ptr()),
            vp(den.data_ptr()), None)
    assert rc == 0, L.vbm3d_last_error()
g = torch.Generator(device="cuda").manual_seed(5)
small = torch.rand((3, 3, 64, 80), device="cuda", generator=g) * 255
big = torch.rand((3, 3, 1080, 1920), device="cuda", generator=g) * 255
sn, sd, bn, bd = (torch.empty_like(small), torch.empty_like(small), torch.empty_like(big), torch.empty_like(big))
call(L.vbm3d_gpu_step1, small, sn, sd)
call(L.vbm3d_gpu_step1_noalloc, small, sn, sd)
call(L.vbm3d_gpu_step1_noalloc, small, sn, sd)
torch.cuda.synchronize()
free0 = torch.cuda.mem_get_info()[0]
call(L.vbm3d_gpu_step1_noalloc, big, bn, bd)
torch.cuda.synchronize()
free1 = torch.cuda.mem_get_info()[0]
print("free memory drop: %d bytes" % (free0 - free1))
assert free0 - free1 < (2 << 20), free0 - free1
"""


def test_noalloc_does_not_allocate(lib):
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    res = subprocess.run([sys.executable, "-c", FREE_MEMORY_PROBE, root], capture_output=True, text=True,
                         timeout=600)
    assert res.returncode == 0, res.stdout + res.stderr
