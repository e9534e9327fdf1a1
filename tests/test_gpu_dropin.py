"""The drop-in shim on the GPU: a C++ program written against the
reference's API (run_vbm3d, vbm3d_1st_step, vbm3d_2nd_step of src/vbm3d.h)
runs the GPU library through vbm3d_gb300/dropin/vbm3d_dropin.cpp, with flows
of F - 1 frames as the reference's main.cpp loads them from flow files
(src/main.cpp:360, :369).  Checked against the oracle given the same flows
padded to F frames (the steps never read a flow's last frame), and against
the C ABI called directly.  Tolerances as in test_gpu_parity: 1e-3 max-abs
on the 0-255 scale for one step, 0.01 dB PSNR end to end."""
import numpy as np
import pytest

from dropin_util import build_driver, run_driver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import vbm3d_gb300 as vb  # noqa: E402
from oracle.pyoracle import Oracle  # noqa: E402
from vbm3d_gb300.synth import make_clip, psnr  # noqa: E402

TOL = 1e-3


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    e = build_driver(tmp_path_factory.mktemp("dropin"))
    if e is None:
        pytest.skip("g++ not found")
    return e


@pytest.fixture(scope="module")
def clip():
    # a moving grating with its exact flow, RGB, sigma 25
    return make_clip(80, 64, 7, 3, 25.0, 91, with_flow=True)


def ratio(num, den, fb):
    return np.where(den == 0, fb, num / np.where(den == 0, 1, den)).astype(np.float32)


def test_run_with_file_flows(exe, tmp_path, clip):
    clean, noisy, ff, bf = clip
    F = noisy.shape[0]
    assert not ff[F - 1].any() and not bf[F - 1].any()  # make_clip's flows: F frames, the last one zero
    rc, basic, final, err = run_driver(exe, tmp_path, "run", noisy, 25.0, ff[:F - 1], bf[:F - 1], tag="f1")
    assert rc == 0, err
    o = Oracle()
    p1, p2 = o.default_params(1, 25.0), o.default_params(2, 25.0)
    ob, of = o.run(25.0, noisy, p1, p2, ff, bf, color_space=True, threads=4)
    assert np.abs(basic - ob).max() <= TOL
    assert abs(psnr(clean, final) - psnr(clean, of)) <= 0.01
    # the flows were used: without them the oracle's basic estimate differs
    zb, _ = o.run(25.0, noisy, p1, p2, None, None, color_space=True, threads=4)
    assert np.abs(zb - ob).max() > 0.1
    # F-frame flows give the same result as F - 1-frame flows
    rc, basic2, _, err = run_driver(exe, tmp_path, "run", noisy, 25.0, ff, bf, tag="f2")
    assert rc == 0, err
    assert np.abs(basic2 - basic).max() <= TOL


def test_steps_with_file_flows_match_the_c_abi(exe, tmp_path, clip):
    _, noisy, ff, bf = clip
    F = noisy.shape[0]
    o = Oracle()
    yuv = o.color_transform(noisy, True)
    rc, num, den, err = run_driver(exe, tmp_path, "step1", yuv, 25.0, ff[:F - 1], bf[:F - 1], tag="s1")
    assert rc == 0, err
    dev = torch.device("cuda:0")
    p1 = vb.default_params(1, 25.0)
    gnum, gden = vb.step1(torch.from_numpy(yuv).to(dev), p1, 25.0, torch.from_numpy(ff).to(dev),
                          torch.from_numpy(bf).to(dev), True)
    torch.cuda.synchronize()
    gnum, gden = gnum.cpu().numpy(), gden.cpu().numpy()
    np.testing.assert_allclose(den, gden, rtol=1e-5, atol=1e-9)
    assert np.abs(ratio(num, den, yuv) - ratio(gnum, gden, yuv)).max() <= TOL
    onum, oden = o.step(1, o.default_params(1, 25.0), 25.0, yuv, None, ff, bf, True)
    basic = ratio(onum, oden, yuv)
    assert np.abs(ratio(num, den, yuv) - basic).max() <= TOL
    rc, num2, den2, err = run_driver(exe, tmp_path, "step2", yuv, 25.0, ff[:F - 1], bf[:F - 1], basic=basic, tag="s2")
    assert rc == 0, err
    o2n, o2d = o.step(2, o.default_params(2, 25.0), 25.0, yuv, basic, ff, bf, True)
    assert np.abs(ratio(num2, den2, basic) - ratio(o2n, o2d, basic)).max() <= TOL


def test_host_entry_points_take_f_minus_1_frame_flows(clip):
    # vbm3d_run_host / vbm3d_step_host copy only a flow's first F - 1 frames
    # (the steps never read the last): F - 1-frame host flows give the same
    # bits as F-frame ones (deterministic aggregation, so runs compare bit
    # for bit)
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    _, noisy, ff, bf = clip
    F = noisy.shape[0]
    with vb.Deterministic(True):
        a = vb.run_host(noisy, 25.0, fflow=ff, bflow=bf, color_space=True)
        b = vb.run_host(noisy, 25.0, fflow=np.ascontiguousarray(ff[:F - 1]), bflow=np.ascontiguousarray(bf[:F - 1]),
                        color_space=True)
    for u, v in zip(a, b):
        np.testing.assert_array_equal(u, v)
    with pytest.raises(ValueError):
        vb.run_host(noisy, 25.0, fflow=np.ascontiguousarray(ff[:F - 2]), color_space=True)
