"""GPU multiscaler DCT pyramid (vbm3d_gpu_ms_*) through the C ABI against the
golden vectors of the reference's own programs (tests/golden/multiscaler)
and the CPU restatement (oracle/ms_oracle.py).

Tolerance: the reference transforms with FFTW in float, the restatement in
double rounded to float, the GPU with float products of cosine matrices, so
values agree to float rounding of sums over a whole row or column: max
|diff| <= REL * max |reference| with REL = 4e-6 for the fixtures and the
restatement at up to 160 columns, and 2e-5 at 1080p (sums over 1920 terms).
"""
import glob
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import vbm3d_gb300 as vb  # noqa: E402
from oracle import ms_oracle as M  # noqa: E402
from oracle.pyoracle import Oracle  # noqa: E402
from vbm3d_gb300.synth import make_clip, psnr  # noqa: E402

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "multiscaler", "*.npz")))
REL = 4e-6
RATIOS = (0.7, 0.8, 0.5)


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    vb.load()
    return torch.device("cuda:0")


def gpu(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(dev)


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def assert_close(got, want, rel=REL):
    assert got.shape == want.shape
    err = float(np.abs(got.astype(np.float64) - want).max())
    assert err <= rel * float(np.abs(want).max()), (err, float(np.abs(want).max()))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_golden(dev, path):
    g = np.load(path)
    img, levels = g["img"], int(g["levels"])
    lv = vb.ms_decompose(gpu(img, dev), levels)
    for i, x in enumerate(lv):
        assert_close(host(x), g["level_%d" % i])
    ref_levels = [gpu(g["level_%d" % i], dev) for i in range(levels)]
    for f in RATIOS:
        assert_close(host(vb.ms_recompose(ref_levels, f)), g["recompose_%g" % f])
        if levels > 1:
            assert_close(host(vb.ms_merge_coarse(gpu(img, dev), ref_levels[1], f)), g["merge_%g" % f])


@pytest.mark.parametrize("shape,levels", [((2, 3, 120, 160), 3), ((1, 97, 131), 4), ((5, 64, 64), 1)])
def test_restatement(dev, shape, levels):
    rng = np.random.default_rng(len(shape) * 100 + levels)
    img = (rng.random(shape) * 255).astype(np.float32)
    planes = img.reshape(-1, shape[-2], shape[-1])
    lv = vb.ms_decompose(gpu(img, dev), levels)
    want = M.decompose(planes, levels)
    for x, w in zip(lv, want):
        assert tuple(x.shape) == tuple(shape[:-2]) + w.shape[1:]
        assert_close(host(x).reshape(w.shape), w)
    rec = vb.ms_recompose(lv, 0.7)
    assert_close(host(rec).reshape(planes.shape), M.recompose([host(x).reshape(w.shape) for x, w in zip(lv, want)],
                                                              0.7))


def test_roundtrip_1080p(dev):
    # the pyramid is exact in exact arithmetic: recompose(decompose(x)) = x
    rng = np.random.default_rng(11)
    img = (rng.random((1, 1080, 1920)) * 255).astype(np.float32)
    x = gpu(img, dev)
    lv = vb.ms_decompose(x, 3)
    assert [tuple(t.shape) for t in lv] == [(1, 1080, 1920), (1, 540, 960), (1, 270, 480)]
    out = host(vb.ms_recompose(lv, 0.7))
    assert_close(out, img, rel=2e-5)
    assert_close(host(lv[0]), img, rel=2e-5)


def test_level_zero_of_a_video_is_the_video(dev):
    _, noisy, _, _ = make_clip(64, 48, 4, 3, 20.0, 77)
    lv = vb.ms_decompose(gpu(noisy, dev), 2)
    assert tuple(lv[1].shape) == (4, 3, 24, 32)
    assert_close(host(lv[0]), noisy, rel=4e-6)


def test_invalid_arguments(dev):
    x = gpu(np.zeros((1, 8, 8), np.float32), dev)
    with pytest.raises(vb.VBM3DError):
        vb.ms_decompose(x, 5)  # 8 >> 4 == 0: an empty level
    lv = vb.ms_decompose(x, 2)
    with pytest.raises(vb.VBM3DError):
        vb.ms_recompose(lv, 1.5)  # the reference would copy past the level
    with pytest.raises(ValueError):
        vb.ms_recompose([lv[0], lv[0]], 0.7)
    with pytest.raises(TypeError):
        vb.ms_decompose(x.double(), 2)


def test_multiscale_pipeline_matches_oracle_pipeline(dev):
    """src/utils/VBM3Ddenoising_multiscale.sh on the GPU against the same
    chain on the CPU oracles: decompose, VBM3D per level at the script's
    truncated sigma, recompose with ratio 0.7."""
    sigma, levels, factor = 25.0, 3, 0.7
    clean, noisy, _, _ = make_clip(96, 80, 6, 3, sigma, 4321)
    out, den = vb.multiscale_denoise(gpu(noisy, dev), sigma, levels, factor)
    out = host(out)

    o = Oracle()
    f, c, h, w = noisy.shape
    lv = M.decompose(noisy.reshape(f * c, h, w), levels)
    clean_lv = M.decompose(clean.reshape(f * c, h, w), levels)
    oden = []
    for i, x in enumerate(lv):
        s = M.level_sigma(sigma, i)
        v = x.reshape(f, c, x.shape[1], x.shape[2])
        _, d = o.run(s, v, o.default_params(1, s), o.default_params(2, s), color_space=True, threads=4)
        oden.append(d.reshape(f * c, x.shape[1], x.shape[2]))
        ref = clean_lv[i].reshape(v.shape)
        assert abs(psnr(ref, host(den[i])) - psnr(ref, d)) <= 0.01, i
    oout = M.recompose(oden, factor).reshape(noisy.shape)
    assert abs(psnr(clean, out) - psnr(clean, oout)) <= 0.01
    assert psnr(clean, out) > psnr(clean, noisy) + 5
