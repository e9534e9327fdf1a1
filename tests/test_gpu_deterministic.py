"""The deterministic aggregation mode (vbm3d_set_deterministic) against the
oracle, which aggregates in the reference's order
(src/vbm3d.cpp:612-650, :860-924).

Bars:
  * step 1 with bior1.5 (the reference's default at k = 8): its per-group
    estimates are the reference's bits (bior1.5 float loops, Haar, hard
    threshold, weights), so numerator and denominator must equal the
    oracle's bit for bit;
  * step 1 with the DCT and step 2: within 1e-3 of the oracle (the DCT's
    float rounding differs from FFTW's);
  * end to end with the default parameters: the basic estimate bit-exact,
    so step 2 matches on the same basic estimate as the oracle and the final
    estimate is within 1e-3 at every value (not only in PSNR);
  * two runs give identical bits.
"""
import numpy as np
import pytest

from golden_util import load, names

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import vbm3d_gb300 as vb  # noqa: E402
from oracle.pyoracle import Oracle  # noqa: E402
from vbm3d_gb300.synth import make_clip, psnr  # noqa: E402

TOL = 1e-3


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    vb.load()
    return torch.device("cuda:0")


@pytest.fixture(autouse=True)
def deterministic_mode():
    with vb.Deterministic(True):
        yield


def gpu(a, dev):
    return None if a is None else torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def ratio(num, den, fb):
    return np.where(den == 0, fb, num / np.where(den == 0, 1, den)).astype(np.float32)


BIOR_CASES = [n for n in names() if load(n)["p1"].T_2D == vb.BIOR and load(n)["p1"].kt == 1]


@pytest.mark.parametrize("name", BIOR_CASES)
def test_step1_bior_bit_exact_golden(dev, name):
    g = load(name)
    o = Oracle()
    vid1 = o.color_transform(g["noisy"], True) if g["color_space"] else g["noisy"]
    num, den = vb.step1(gpu(vid1, dev), g["p1"], g["sigma"], gpu(g["fflow"], dev), gpu(g["bflow"], dev),
                        g["color_space"])
    torch.cuda.synchronize()
    onum, oden = o.step(1, g["p1"], g["sigma"], vid1, None, g["fflow"], g["bflow"], g["color_space"])
    np.testing.assert_array_equal(den.cpu().numpy(), oden)
    np.testing.assert_array_equal(num.cpu().numpy(), onum)


@pytest.mark.parametrize("shape,sigma,flow,seed", [
    ((96, 72, 7, 3), 20.0, True, 21),
    ((120, 64, 9, 1), 40.0, False, 22),
    ((77, 53, 6, 3), 10.0, False, 23),    # widths not a multiple of the 32-pixel segments
])
def test_step1_bior_bit_exact_synthetic(dev, shape, sigma, flow, seed):
    w, h, f, c = shape
    _, noisy, ff, bf = make_clip(w, h, f, c, sigma, seed, with_flow=flow)
    o = Oracle()
    vid1 = o.color_transform(noisy, True)
    p1 = vb.default_params(1, sigma)
    assert p1.T_2D == vb.BIOR
    num, den = vb.step1(gpu(vid1, dev), p1, sigma, gpu(ff, dev), gpu(bf, dev), True)
    torch.cuda.synchronize()
    onum, oden = o.step(1, p1, sigma, vid1, None, ff, bf, True, threads=4)
    np.testing.assert_array_equal(den.cpu().numpy(), oden)
    np.testing.assert_array_equal(num.cpu().numpy(), onum)


@pytest.mark.parametrize("t2d", [vb.DCT, vb.BIOR])
def test_end_to_end_every_value(dev, t2d):
    clean, noisy, ff, bf = make_clip(112, 80, 8, 3, 25.0, 31, with_flow=True)
    o = Oracle()
    p1, p2 = vb.default_params(1, 25.0).replace(T_2D=t2d), vb.default_params(2, 25.0)
    gb, gf = vb.run_host(noisy, 25.0, p1, p2, fflow=ff, bflow=bf, color_space=True)
    ob, of = o.run(25.0, noisy, p1, p2, ff, bf, color_space=True, threads=4)
    if t2d == vb.BIOR:
        # the colour transform back to RGB is the oracle's, on the same bits
        np.testing.assert_array_equal(gb, ob)
    else:
        assert np.abs(gb - ob).max() <= TOL
    assert np.abs(gf - of).max() <= TOL
    assert abs(psnr(clean, gf) - psnr(clean, of)) <= 0.01


@pytest.mark.parametrize("name", names())
def test_run_golden_every_value(dev, name):
    g = load(name)
    if g["p1"].kt > 1 or g["p2"].kt > 1 or g["p1"].N > 8 or g["p2"].N > 8:
        pytest.skip("outside the deterministic mode's limits (kt == 1, N <= 8)")
    basic, final = vb.run(gpu(g["noisy"], dev), g["sigma"], g["p1"], g["p2"], gpu(g["fflow"], dev),
                          gpu(g["bflow"], dev), g["color_space"])
    torch.cuda.synchronize()
    basic, final = basic.cpu().numpy(), final.cpu().numpy()
    assert np.abs(basic - g["basic"]).max() <= TOL
    assert np.abs(final - g["final"]).max() <= TOL


def test_runs_are_bit_reproducible(dev):
    _, noisy, ff, bf = make_clip(96, 64, 7, 3, 30.0, 41, with_flow=True)
    a = vb.run_host(noisy, 30.0, fflow=ff, bflow=bf, color_space=True)
    b = vb.run_host(noisy, 30.0, fflow=ff, bflow=bf, color_space=True)
    x = gpu(noisy, dev)
    c = vb.run(x, 30.0, fflow=gpu(ff, dev), bflow=gpu(bf, dev), color_space=True)
    torch.cuda.synchronize()
    for u, v in zip(a, b):
        np.testing.assert_array_equal(u, v)
    for u, v in zip(a, c):
        np.testing.assert_array_equal(u, v.cpu().numpy())


def test_dense_buckets(dev):
    # a constant clip: every distance ties, every group holds the first
    # patches of the partial_sort order, so many groups share patches (the
    # long bucket lists of the overflow path)
    flat = np.full((5, 3, 40, 64), 50.0, np.float32)
    o = Oracle()
    p1 = vb.default_params(1, 5.0)
    num, den = vb.step1(gpu(flat, dev), p1, 5.0)
    torch.cuda.synchronize()
    onum, oden = o.step(1, p1, 5.0, flat)
    np.testing.assert_array_equal(den.cpu().numpy(), oden)
    np.testing.assert_array_equal(num.cpu().numpy(), onum)


def test_unsupported_shapes_rejected(dev):
    _, noisy, _, _ = make_clip(48, 40, 5, 1, 20.0, 5)
    p1 = vb.default_params(1, 20.0).replace(kt=2, T_2D=vb.DCT)
    with pytest.raises(vb.VBM3DError) as e:
        vb.step1(gpu(noisy, dev), p1, 20.0)
    assert e.value.status == 2
    vb.set_deterministic(False)
    vb.step1(gpu(noisy, dev), p1, 20.0)  # the atomic path takes kt = 2
    torch.cuda.synchronize()
