"""Differentiation form at the full-size workload of the acceptance bar:
RGB 480x270x16, AWGN sigma 25, colour transform on (YUV working space).

  * the frozen linearisation of each step against the FP64 CPU
    restatement of the same map (oracle_linear_apply): relative error of
    L x, and of the adjoint through <L x, g> = <x, L^T g>;
  * central finite differences (h = 1e-3, 32 random directions) of step 2
    with the basic estimate fixed, against L d: relative error of the
    directional derivatives g^T J d;
  * Monte-Carlo SURE where it is exact: step 2 with the basic estimate held
    fixed is the linear map L of its noisy input (groups and Wiener gains
    come from the basic estimate), so tr(L) estimated with Hutchinson
    probes is an unbiased estimate of its divergence and SURE is unbiased
    for its MSE.  The basic estimate is computed from an independent noise
    realisation of the same clean clip, so that it does not depend on the
    noisy input the estimator is scored on; SURE must then track the true
    MSE over a sweep of step 2's sigma and pick its minimiser.
Each part prints one `LINEAR {...}` line with its figures.
"""
import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import vbm3d_gb300 as vb  # noqa: E402
from oracle.pyoracle import Oracle  # noqa: E402
from vbm3d_gb300.synth import make_clip  # noqa: E402

W, H, F, SIGMA = 480, 270, 16, 25.0
THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    vb.load()
    return torch.device("cuda:0")


def gpu(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(dev)


@pytest.fixture(scope="module")
def case(dev):
    clean, noisy, _, _ = make_clip(W, H, F, 3, SIGMA, 5000)
    o = Oracle()
    yuv = o.color_transform(noisy, True)
    p1, p2 = vb.default_params(1, SIGMA), vb.default_params(2, SIGMA)
    y = gpu(yuv, dev)
    basic = vb.normalize(*vb.step1(y, p1, SIGMA, color_space=True), y)
    L1 = vb.LinearStep(1, y, SIGMA, p1, color_space=True)
    L2 = vb.LinearStep(2, y, SIGMA, p2, basic=basic, color_space=True)
    torch.cuda.synchronize()
    return dict(clean=clean, noisy=noisy, yuv=yuv, y=y, basic=basic, p1=p1, p2=p2, L1=L1, L2=L2, o=o)


@pytest.mark.parametrize("step", [1, 2])
def test_fp64_map_and_adjoint(case, dev, step):
    o, yuv, L, p = case["o"], case["yuv"], case["L%d" % step], case["p%d" % step]
    basic = case["basic"].cpu().numpy() if step == 2 else None
    rng = np.random.default_rng(100 + step)
    x = rng.normal(0, 10, yuv.shape).astype(np.float32)
    g = rng.normal(0, 1, yuv.shape).astype(np.float32)
    want = o.linear(step, p, SIGMA, yuv, x, basic=basic, color_space=True, threads=THREADS)
    got = L.apply(gpu(x, dev)).cpu().numpy().astype(np.float64)
    fwd_err = float(np.linalg.norm(got - want) / np.linalg.norm(want))
    ltg = L.apply(gpu(g, dev), adjoint=True).cpu().numpy().astype(np.float64)
    a = float(np.dot(want.ravel(), g.astype(np.float64).ravel()))
    b = float(np.dot(x.astype(np.float64).ravel(), ltg.ravel()))
    adj_err = abs(a - b) / abs(a)
    print("LINEAR " + json.dumps(dict(check="fp64", step=step, workload="RGB %dx%dx%d sigma %g" % (W, H, F, SIGMA),
                                      forward_rel_err=fwd_err, adjoint_dot_rel_err=adj_err)))
    assert fwd_err < 1e-5
    assert adj_err < 1e-5


def test_central_finite_differences(case, dev):
    # step 2 with the basic estimate fixed: g^T (f(y + h d) - f(y - h d)) / 2h
    # against g^T L d for 32 random directions; the float output carries
    # ~1e-4 of aggregation-order rounding, which h = 1e-3 amplifies per value
    # and the projection on g averages out
    y, b, p2, L = case["y"], case["basic"], case["p2"], case["L2"]
    rng = np.random.default_rng(7)
    g = gpu(rng.normal(0, 1, case["yuv"].shape), dev).double()
    h = 1e-3

    def f2(v):
        return vb.normalize(*vb.step2(v, b, p2, SIGMA, color_space=True), b)

    errs = []
    for _ in range(32):
        d = gpu(rng.normal(0, 1, case["yuv"].shape), dev)
        fd = (f2(y + h * d).double() - f2(y - h * d).double()) / (2 * h)
        ld = L.apply(d).double()
        a, c = float((g * fd).sum()), float((g * ld).sum())
        errs.append(abs(a - c) / float(torch.linalg.norm(g) * torch.linalg.norm(ld)))
    print("LINEAR " + json.dumps(dict(check="central differences, step 2 (basic fixed)", h=h, directions=32,
                                      max_rel_err=max(errs), mean_rel_err=float(np.mean(errs)))))
    assert max(errs) < 2e-3


def test_sure_exact_for_step2_with_fixed_basic(case, dev):
    from vbm3d_gb300.sure import sure_step2_fixed_basic
    clean = gpu(case["clean"], dev)
    y = gpu(case["noisy"], dev)
    # the basic estimate from an independent noise realisation of the same
    # clean clip (a stream of its own, so the pilot does not depend on y)
    rng = np.random.default_rng(5077)
    noisy2 = (case["clean"] + np.float32(SIGMA) * rng.standard_normal(case["clean"].shape, dtype=np.float32))
    y2 = vb.color_transform(gpu(noisy2, dev), True)
    basic = vb.normalize(*vb.step1(y2, vb.default_params(1, SIGMA), SIGMA, color_space=True), y2)
    rows = []
    for sf in (12.0, 18.0, 22.0, 25.0, 30.0, 40.0):
        r = sure_step2_fixed_basic(y, SIGMA, sf, basic, clean=clean, probes=8)
        rows.append({k: r[k] for k in ("sigma_f", "mse", "sure", "sure_fd")})
    mse = np.array([r["mse"] for r in rows])
    sure = np.array([r["sure"] for r in rows])
    # SURE - MSE = (|n|^2 / n - sigma^2) - 2 <n, f - x> / n + 2 sigma^2 div / n
    # for one noise realisation n: its first term, the realisation's sample
    # variance less sigma^2 (standard deviation sigma^2 sqrt(2 / n) = 0.35
    # here), is the same at every sigma_f; with it taken out (the test knows
    # the noise) what remains is the estimator's own error: the cross term
    # against the divergence, and the probes' error
    noise = case["noisy"].astype(np.float64) - case["clean"].astype(np.float64)
    offset = float(np.mean(noise ** 2)) - SIGMA ** 2
    rel = np.abs(sure - offset - mse) / mse
    print("LINEAR " + json.dumps(dict(check="SURE, step 2 with a fixed basic estimate", rows=rows,
                                      noise_variance_offset=offset, max_rel_err_after_offset=float(rel.max()),
                                      max_rel_err=float((np.abs(sure - mse) / mse).max()))))
    assert rel.max() < 0.02, rows
    assert int(np.argmin(sure)) == int(np.argmin(mse)), rows
