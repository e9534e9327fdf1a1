"""CPU-side checks of the C ABI: the library loads, exports every symbol the
header declares, and its host logic (defaults, noise table, grid, argument
validation) matches the oracle.  No kernel runs here."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import vbm3d_gb300 as vb
from oracle.pyoracle import Oracle
from vbm3d_gb300._abi import Dims, Params

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "vbm3d_gb300.h")


@pytest.fixture(scope="module")
def lib():
    from vbm3d_gb300 import build
    build.build()
    return vb.load()


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(vbm3d_\w+)\s*\(", src, flags=re.M)))


def test_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 12, syms
    for s in syms:
        assert hasattr(lib, s), s


def test_default_params_match_oracle(lib):
    o = Oracle()
    for step in (1, 2):
        for sigma in (5.0, 20.0, 30.0, 30.5, 40.0):
            assert vb.default_params(step, sigma).as_dict() == o.default_params(step, sigma).as_dict()


def test_sigma_table_matches_oracle(lib):
    o = Oracle()
    for c in (1, 3):
        for cs in (False, True):
            np.testing.assert_array_equal(np.array(vb.sigma_table(25.0, c, cs), np.float32), o.sigma_table(25.0, c, cs))


def test_ref_count_matches_oracle_grid(lib):
    o = Oracle()
    for (w, h, f) in [(176, 144, 10), (960, 540, 50), (1920, 1080, 30), (33, 17, 3)]:
        for step, sigma in [(1, 20), (2, 20), (2, 40)]:
            p = o.default_params(step, sigma)
            d = Dims(w, h, f, 1)
            rows, cols = o.grid(p, d)
            assert vb.ref_count(p, d) == len(rows) * len(cols) * f


def status_of(lib, fn, *args):
    return getattr(lib, fn)(*args)


@pytest.mark.parametrize("bad,code", [
    (dict(kt=5), 2),            # temporal patches above 4 frames
    (dict(T_2D=1, k=7), 1),     # bior1.5 needs k == 8
    (dict(T_2D=5), 1),
    (dict(p=0), 1),
    (dict(N=0), 1),
    (dict(Nb=0), 1),
    (dict(N=64), 2),
    (dict(Ns=17), 2),
    (dict(k=20, T_2D=0), 2),
])
def test_invalid_parameters_rejected_before_any_launch(lib, bad, code):
    p = vb.default_params(1, 20.0).replace(**bad)
    fake = C.c_void_p(16)  # never dereferenced: validation fails first
    rc = lib.vbm3d_gpu_step1(C.byref(p), fake, None, None, Dims(64, 48, 4, 1), 20.0, 0, fake, fake, None)
    assert rc == code, (rc, lib.vbm3d_last_error())
    assert lib.vbm3d_last_error()


def test_invalid_dims_rejected(lib):
    p = vb.default_params(1, 20.0)
    fake = C.c_void_p(16)
    for d, code in [(Dims(0, 48, 4, 1), 1), (Dims(64, 48, 4, 2), 2), (Dims(64, 48, 4, 4), 2), (Dims(7, 48, 4, 1), 1),
                    (Dims(60000, 60000, 2, 1), 2)]:
        rc = lib.vbm3d_gpu_step1(C.byref(p), fake, None, None, d, 20.0, 0, fake, fake, None)
        assert rc == code, (d.width, d.channels, rc, lib.vbm3d_last_error())
    # a window too small to hold Nb positions: the reference reads past its end
    p1 = p.replace(Ns=1)
    assert lib.vbm3d_gpu_step1(C.byref(p1), fake, None, None, Dims(64, 48, 4, 1), 20.0, 0, fake, fake, None) == 1
    assert lib.vbm3d_gpu_step1(None, fake, None, None, Dims(64, 48, 4, 1), 20.0, 0, fake, fake, None) == 1
    assert lib.vbm3d_gpu_step2(C.byref(p), fake, None, None, None, Dims(64, 48, 4, 1), 20.0, 0, fake, fake, None) == 1


def test_status_strings(lib):
    for code in range(7):
        assert lib.vbm3d_status_string(code).startswith(b"VBM3D_")


def reference_src():
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    where = subprocess.check_output(["sh", os.path.join(root, "oracle", "build_ref.sh"), "--where"], text=True)
    return os.path.join(where.strip(), "src")


REFERENCE_SRC = reference_src()


@pytest.mark.skipif(not os.path.isdir(REFERENCE_SRC), reason="reference sources not present")
def test_dropin_shim_compiles_against_reference_headers(tmp_path):
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cmd = ["g++", "-std=c++11", "-O1", "-w", "-c", os.path.join(root, "vbm3d_gb300", "dropin", "vbm3d_dropin.cpp"),
           "-I", os.path.join(root, "oracle", "fftw_shim"), "-I", REFERENCE_SRC,
           "-I", os.path.join(REFERENCE_SRC, "Utilities"), "-I", os.path.join(root, "include"),
           "-o", str(tmp_path / "dropin.o")]
    subprocess.check_call(cmd)
    syms = subprocess.check_output(["nm", "-C", str(tmp_path / "dropin.o")], text=True)
    for name in ("vbm3d_1st_step(", "vbm3d_2nd_step(", "run_vbm3d("):
        assert any(name in line and " T " in line for line in syms.splitlines()), name


def test_batch_rejects_bad_clips_before_any_cuda_call(lib):
    from vbm3d_gb300._abi import BatchConfig, Clip
    fake = C.c_void_p(16)  # never dereferenced: validation fails first
    h = C.c_void_p()
    assert lib.vbm3d_batch_create(None, 0, 0, None, C.byref(h), None) == 1
    p16 = vb.default_params(2, 20.0).replace(N=16)
    clips = (Clip * 2)()
    clips[0] = Clip(Dims(64, 48, 4, 3), 20.0, None, None, fake, None, None, None, fake)
    clips[1] = Clip(Dims(64, 48, 4, 1), 20.0, None, C.pointer(p16), fake, None, None, None, fake)
    assert lib.vbm3d_batch_create(clips, 2, 1, None, C.byref(h), None) == 2
    assert b"clip 1 step 2" in lib.vbm3d_last_error()
    clips[1] = Clip(Dims(64, 48, 4, 1), 20.0, None, None, None, None, None, None, fake)
    assert lib.vbm3d_batch_create(clips, 2, 1, None, C.byref(h), None) == 1
    clips[1] = Clip(Dims(64, 48, 4, 2), 20.0, None, None, fake, None, None, None, fake)
    assert lib.vbm3d_batch_create(clips, 2, 1, None, C.byref(h), None) == 2
    clips[1] = Clip(Dims(64, 48, 4, 1), 20.0, None, None, fake, None, None, None, fake)
    bad = BatchConfig(bm1_tile=4, bm1_warps=3)
    assert lib.vbm3d_batch_create(clips, 2, 1, C.byref(bad), C.byref(h), None) == 1
    bad = BatchConfig(bm1_tile=4)
    assert lib.vbm3d_batch_create(clips, 2, 1, C.byref(bad), C.byref(h), None) == 1
    assert not h.value


def test_tvl1_rejects_bad_options_before_any_cuda_call(lib):
    from vbm3d_gb300._abi import TvParams
    p = TvParams()
    assert lib.vbm3d_tvl1_default_params(C.byref(p)) == 0
    assert (p.tau, p.lambda_, p.theta, p.nscales, p.fscale, p.zfactor, p.nwarps) == (
        0.25, np.float32(0.2), np.float32(0.3), 100, 2, 0.5, 5)
    ns, fs = C.c_int(), C.c_int()
    assert lib.vbm3d_tvl1_scales(960, 540, C.byref(p), C.byref(ns), C.byref(fs)) == 0 and (ns.value, fs.value) == (7, 2)
    fake = C.c_void_p(16)
    for bad in (dict(tau=0.3), dict(zfactor=1.0), dict(nwarps=0), dict(epsilon=0.0), dict(lambda_=-1.0)):
        q = TvParams()
        lib.vbm3d_tvl1_default_params(C.byref(q))
        for k, v in bad.items():
            setattr(q, k, v)
        assert lib.vbm3d_gpu_tvl1_pairs(fake, fake, 1, 64, 48, C.byref(q), fake, None, None) == 1
    assert lib.vbm3d_gpu_tvl1_pairs(fake, fake, 0, 64, 48, C.byref(p), fake, None, None) == 1
    assert lib.vbm3d_gpu_tvl1_video(fake, 64, 48, 1, C.byref(p), fake, fake, None) == 1


def test_multiscaler_rejects_bad_arguments_before_any_cuda_call(lib):
    fake = C.c_void_p(16)
    outs = (C.c_void_p * 3)(fake, fake, fake)
    # an empty level (8 >> 4 == 0), no planes, no levels, a NULL output level
    assert lib.vbm3d_gpu_ms_decompose(fake, 8, 8, 1, 5, outs, None) == 1
    assert lib.vbm3d_gpu_ms_decompose(fake, 8, 8, 0, 1, outs, None) == 1
    assert lib.vbm3d_gpu_ms_decompose(fake, 8, 8, 1, 0, outs, None) == 1
    assert lib.vbm3d_gpu_ms_decompose(fake, 8, 8, 1, 3, (C.c_void_p * 3)(fake, None, fake), None) == 1
    assert lib.vbm3d_gpu_ms_decompose(None, 8, 8, 1, 1, outs, None) == 1
    # a recomposition ratio above 1 would make the reference copy past the level
    assert lib.vbm3d_gpu_ms_recompose(outs, 8, 8, 1, 2, C.c_float(1.5), fake, None) == 1
    assert lib.vbm3d_gpu_ms_recompose(outs, 8, 8, 1, 2, C.c_float(float("nan")), fake, None) == 1
    # a coarse block larger than the fine image
    assert lib.vbm3d_gpu_ms_merge_coarse(fake, fake, 8, 8, 16, 16, 1, C.c_float(0.9), fake, None) == 1
    assert lib.vbm3d_gpu_ms_merge_coarse(fake, None, 8, 8, 4, 4, 1, C.c_float(0.5), fake, None) == 1
