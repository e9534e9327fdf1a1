"""Differentiation form: the frozen linearisation of each step (groups,
masks / Wiener gains and weights frozen at the forward pass) and its
hand-written adjoint, through the C ABI (vbm3d_linear_*).

Checks: the map applied to the noisy input is the forward step; forward
applications match the FP64 CPU restatement of the same map
(oracle_linear_apply); the adjoint satisfies <L x, g> = <x, L^T g> against
that FP64 map; central finite differences of the forward step agree with
L d; a torch.autograd.Function built on it (test harness only) gives the
adjoint as its gradient; and the exact Monte-Carlo SURE built on it tracks
the true MSE over a sweep of the filter's sigma.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import vbm3d_gb300 as vb  # noqa: E402
from oracle.pyoracle import Oracle  # noqa: E402
from vbm3d_gb300.synth import make_clip  # noqa: E402

SIGMA = 25.0


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    vb.load()
    return torch.device("cuda:0")


@pytest.fixture(scope="module")
def clip():
    clean, noisy, _, _ = make_clip(64, 48, 6, 3, SIGMA, 500)
    return clean, noisy


@pytest.fixture(scope="module")
def oracle():
    return Oracle()


def gpu(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(dev)


def basic_of(oracle, noisy, p1):
    num, den = oracle.step(1, p1, SIGMA, noisy, color_space=True, threads=4)
    return np.where(den == 0, noisy, num / np.where(den == 0, 1, den)).astype(np.float32)


@pytest.fixture(scope="module")
def steps(dev, clip, oracle):
    _, noisy = clip
    p1 = vb.default_params(1, SIGMA)
    p2 = vb.default_params(2, SIGMA)
    basic = basic_of(oracle, noisy, p1)
    y, b = gpu(noisy, dev), gpu(basic, dev)
    L1 = vb.LinearStep(1, y, SIGMA, p1, color_space=True)
    L2 = vb.LinearStep(2, y, SIGMA, p2, basic=b, color_space=True)
    torch.cuda.synchronize()
    return dict(y=y, b=b, basic=basic, p1=p1, p2=p2, L1=L1, L2=L2)


def test_map_of_the_noisy_input_is_the_forward_step(dev, clip, steps, oracle):
    _, noisy = clip
    out1 = steps["L1"].apply(steps["y"]).cpu().numpy()
    assert np.abs(out1 - steps["basic"]).max() <= 1e-3
    n2, d2 = oracle.step(2, steps["p2"], SIGMA, noisy, steps["basic"], color_space=True, threads=4)
    out2 = steps["L2"].apply(steps["y"]).cpu().numpy()
    mask = d2 > 0
    ref2 = n2 / np.where(mask, d2, 1)
    assert np.abs(out2[mask] - ref2[mask]).max() <= 1e-3


@pytest.mark.parametrize("step", [1, 2])
def test_forward_matches_fp64_map(dev, clip, steps, oracle, step):
    _, noisy = clip
    rng = np.random.default_rng(step)
    x = rng.normal(0, 10, noisy.shape).astype(np.float32)
    L = steps["L%d" % step]
    got = L.apply(gpu(x, dev)).cpu().numpy().astype(np.float64)
    want = oracle.linear(step, steps["p%d" % step], SIGMA, noisy, x, basic=steps["basic"] if step == 2 else None,
                         color_space=True)
    err = np.linalg.norm(got - want) / np.linalg.norm(want)
    assert err < 1e-5, err


@pytest.mark.parametrize("step", [1, 2])
def test_adjoint_against_fp64_map(dev, clip, steps, oracle, step):
    _, noisy = clip
    rng = np.random.default_rng(10 + step)
    L = steps["L%d" % step]
    for _ in range(3):
        x = rng.normal(0, 1, noisy.shape).astype(np.float32)
        g = rng.normal(0, 1, noisy.shape).astype(np.float32)
        lx = oracle.linear(step, steps["p%d" % step], SIGMA, noisy, x, basic=steps["basic"] if step == 2 else None,
                           color_space=True)
        ltg = L.apply(gpu(g, dev), adjoint=True).cpu().numpy().astype(np.float64)
        a = float(np.dot(lx.ravel(), g.astype(np.float64).ravel()))
        b = float(np.dot(x.astype(np.float64).ravel(), ltg.ravel()))
        assert abs(a - b) <= 1e-5 * max(abs(a), 1e-12), (a, b)
        # and the GPU's own pair
        lx_gpu = L.apply(gpu(x, dev)).cpu().numpy().astype(np.float64)
        c = float(np.dot(lx_gpu.ravel(), g.astype(np.float64).ravel()))
        assert abs(c - b) <= 1e-5 * max(abs(c), 1e-12), (c, b)


def test_central_finite_differences(dev, clip, steps):
    # Step 2 with the basic estimate fixed is exactly linear in the noisy
    # input (its groups and Wiener gains come from the basic estimate), so
    # its central differences are L2 d.  Directional derivatives
    # g^T (f(y + h d) - f(y - h d)) / 2h, h = 1e-3, 32 random directions; the
    # step's float output carries ~1e-4 of rounding (atomic aggregation
    # order), which h = 1e-3 amplifies per pixel and the projection averages.
    # (Step 1 groups and thresholds its own input: its frozen map is the
    # derivative only where no group or mask changes, so it is checked
    # against the FP64 map and the adjoint identity instead.)
    _, noisy = clip
    rng = np.random.default_rng(7)
    g = gpu(rng.normal(0, 1, noisy.shape), dev).double()
    p2, b = steps["p2"], steps["b"]
    h = 1e-3

    def f2(y):
        return vb.normalize(*vb.step2(y, b, p2, SIGMA, color_space=True), b)

    for step, f, L, tol in ((2, f2, steps["L2"], 2e-3),):
        for _ in range(32):
            d = rng.normal(0, 1, noisy.shape).astype(np.float32)
            fd = (f(gpu(noisy + h * d, dev)).double() - f(gpu(noisy - h * d, dev)).double()) / (2 * h)
            ld = L.apply(gpu(d, dev)).double()
            a, c = float((g * fd).sum()), float((g * ld).sum())
            scale = float(torch.linalg.norm(g) * torch.linalg.norm(ld))
            assert abs(a - c) <= tol * scale, (step, a, c, scale)
    # Step 2 with the basic estimate fixed is exactly linear in the noisy
    # input: with a large step the whole difference quotient matches L2 d.
    d = rng.normal(0, 1, noisy.shape).astype(np.float32)
    H = 1.0
    fd = ((f2(gpu(noisy + H * d, dev)).double() - f2(gpu(noisy - H * d, dev)).double()) / (2 * H)).cpu().numpy()
    ld = steps["L2"].apply(gpu(d, dev)).cpu().numpy().astype(np.float64)
    assert np.linalg.norm(fd - ld) / np.linalg.norm(ld) < 5e-4


class LinearFn(torch.autograd.Function):
    """Test-harness autograd wrapper: forward L x, backward L^T g."""

    @staticmethod
    def forward(ctx, x, L):
        ctx.L = L
        return L.apply(x.contiguous())

    @staticmethod
    def backward(ctx, g):
        return ctx.L.apply(g.contiguous(), adjoint=True), None


def test_autograd_wrapper(dev, clip, steps):
    _, noisy = clip
    rng = np.random.default_rng(3)
    x = gpu(rng.normal(0, 1, noisy.shape), dev).requires_grad_(True)
    w = gpu(rng.normal(0, 1, noisy.shape), dev)
    loss = (LinearFn.apply(x, steps["L2"]) * w).sum()
    loss.backward()
    want = steps["L2"].apply(w, adjoint=True)
    assert torch.allclose(x.grad, want, rtol=1e-6, atol=1e-7)


def test_mc_sure_tracks_mse(dev, clip):
    # SURE of the hard-threshold estimate over a sweep of the filter's sigma.
    # With the divergence from finite differences of the forward step
    # (Monte-Carlo SURE) it tracks the true MSE; with the divergence of the
    # frozen linearisation it misses the jump terms of hard thresholding
    # (Stein's identity needs a continuous estimator) and is biased low.
    from vbm3d_gb300.sure import mc_sure
    clean, noisy = clip
    y = gpu(noisy, dev)
    c = torch.from_numpy(clean).to(dev)
    sweep = [10.0, 15.0, 20.0, 25.0, 35.0, 50.0]
    fd, lin, mse = [], [], []
    for sf in sweep:
        r = mc_sure(y, SIGMA, sf, clean=c, stage="basic", probes=3)
        fd.append(r["sure_fd"])
        lin.append(r["sure_linear"])
        mse.append(r["mse"])
    fd, lin, mse = np.array(fd), np.array(lin), np.array(mse)
    assert abs(int(np.argmin(fd)) - int(np.argmin(mse))) <= 1, (fd, mse)
    assert np.max(np.abs(fd - mse) / mse) < 0.3, (fd, mse)
    assert np.all(lin < mse), (lin, mse)
