"""GPU TV-L1 optical flow (vbm3d_gpu_tvl1_*) against the reference's own
flows (golden vectors of tests/golden/tvl1, made by tvl1flow_lib.c) and the
oracle restatement.

Per pixel the arithmetic is the reference's; the order of the error sum that
ends each warping is not, so a warping can stop one iteration apart from the
reference when its error lands within rounding of epsilon^2.  The bar:
iteration counts within one of the oracle's, flows within 0.02 px max-abs
and 1e-4 px mean-abs of the reference, and VBM3D driven by the GPU flows
within 0.01 dB of VBM3D driven by the reference's flows.
"""
import glob
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import vbm3d_gb300 as vb  # noqa: E402
from oracle.pyoracle import Oracle, TvlOracle  # noqa: E402
from vbm3d_gb300.synth import make_clip, psnr  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "tvl1")
NAMES = sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
KEYS = ["tau", "lambda_", "theta", "nscales", "fscale", "zfactor", "nwarps", "epsilon"]


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    vb.load()
    return torch.device("cuda:0")


def gpu(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(dev)


def opts(vals):
    return {k: (int(v) if k in ("nscales", "fscale", "nwarps") else float(v)) for k, v in zip(KEYS, vals)}


def close(got, want):
    d = np.abs(got - want)
    assert d.max() <= 0.02 and d.mean() <= 1e-4, (float(d.max()), float(d.mean()))


@pytest.mark.parametrize("name", NAMES)
def test_flow_matches_reference_golden(dev, name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    kw = opts(z["opts"])
    flow, it = vb.tvl1_flow(gpu(z["I0"], dev), gpu(z["I1"], dev), vb.tvl1_params(**kw), iterations=True)
    close(flow.cpu().numpy(), z["flow"])
    tv = TvlOracle()
    _, oit = tv.flow(z["I0"], z["I1"], tv.default_params(**kw), iters=True)
    assert np.abs(it[0] - oit).max() <= 1, (it[0].tolist(), oit.tolist())


def test_batched_pairs_equal_single_pairs(dev):
    frames = []
    for s in range(4):
        _, noisy, _, _ = make_clip(72, 56, 2, 1, 15.0, 600 + s, vmax=3.0)
        frames.append(noisy[:, 0])
    I0 = gpu(np.stack([f[0] for f in frames]), dev)
    I1 = gpu(np.stack([f[1] for f in frames]), dev)
    p = vb.tvl1_params(fscale=0)
    batch = vb.tvl1_flow(I0, I1, p).cpu().numpy()
    tv = TvlOracle()
    for q in range(4):
        single = vb.tvl1_flow(I0[q].contiguous(), I1[q].contiguous(), p).cpu().numpy()
        close(batch[q], single)
        close(batch[q], tv.flow(frames[q][0], frames[q][1], tv.default_params(fscale=0)))


def test_video_flows_layout(dev):
    _, noisy, _, _ = make_clip(64, 48, 5, 1, 10.0, 610, vmax=3.0)
    video = noisy[:, 0]
    ff, bf = vb.tvl1_video(gpu(video, dev))
    ff, bf = ff.cpu().numpy(), bf.cpu().numpy()
    tv = TvlOracle()
    p = tv.default_params()
    for t in range(4):
        close(ff[t], tv.flow(video[t], video[t + 1], p))   # motion t -> t + 1
        close(bf[t], tv.flow(video[t + 1], video[t], p))   # motion t + 1 -> t
    assert not ff[4].any() and not bf[4].any()


def test_vbm3d_with_gpu_flows(dev):
    # the denoiser driven by GPU flows against the same denoiser driven by
    # the oracle's flows (the reference pipeline: flows of the noisy clip)
    clean, noisy, _, _ = make_clip(64, 48, 6, 1, 20.0, 620, vmax=3.0)
    ff, bf = vb.tvl1_video(gpu(noisy[:, 0], dev))
    tv = TvlOracle()
    p = tv.default_params()
    off = np.zeros_like(ff.cpu().numpy())
    obf = np.zeros_like(off)
    for t in range(5):
        off[t] = tv.flow(noisy[t, 0], noisy[t + 1, 0], p)
        obf[t] = tv.flow(noisy[t + 1, 0], noisy[t, 0], p)
    _, fin_gpu = vb.run(gpu(noisy, dev), 20.0, fflow=ff, bflow=bf)
    _, fin_ref = Oracle().run(20.0, noisy, Oracle().default_params(1, 20.0), Oracle().default_params(2, 20.0),
                              off, obf, color_space=False, threads=4)
    assert abs(psnr(clean, fin_gpu.cpu().numpy()) - psnr(clean, fin_ref)) <= 0.01
