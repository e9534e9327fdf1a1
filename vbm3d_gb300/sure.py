"""Monte-Carlo SURE (Stein's unbiased risk estimate) for tuning the filter
without clean frames.

SURE(f) = ||f(y) - y||^2 / n - sigma^2 + 2 sigma^2 div f(y) / n, for y with
i.i.d. Gaussian noise of standard deviation sigma.  Two divergence
estimators are provided, both with Hutchinson probes b ~ N(0, I):
  * "fd": b^T (f(y + eps b) - f(y)) / eps with eps = sigma / 20 (Monte-Carlo
    SURE with a finite difference of the forward pass);
  * "linear": b^T J b with J the frozen linearisation (vbm3d_linear_*: the
    groups, masks / Wiener gains and weights of the pass at y held fixed),
    exact for that linear map.  VBM3D's hard thresholding and block matching
    are discontinuous in y, so the linearisation misses the jump terms of
    Stein's identity and this estimate is biased low; it is reported for
    comparison.
The steps run in YUV for RGB input (colour transform on), so the estimate
is T^-1 f(T y) and the linearised divergence tr(T^-1 L T).
"""
import torch

import vbm3d_gb300 as vb


def _estimate(y_rgb, sigma_f, stage, p1, p2):
    yy = vb.color_transform(y_rgb.clone(), True) if y_rgb.shape[1] == 3 else y_rgb.clone()
    basic = vb.normalize(*vb.step1(yy, p1, sigma_f, color_space=True), yy)
    if stage == "basic":
        out = basic
    else:
        out = vb.normalize(*vb.step2(yy, basic, p2, sigma_f, color_space=True), basic)
    if y_rgb.shape[1] == 3:
        out = vb.color_transform(out.clone(), False)
    return out, yy, basic


def mc_sure(y, sigma_true, sigma_f, clean=None, stage="basic", probes=3, seed=0, p1=None, p2=None):
    """SURE of the basic (stage="basic") or final estimate of the filter run
    at sigma_f, for noise level sigma_true.  Returns a dict with both SURE
    estimates, their divergences and, when `clean` is given, the true MSE."""
    p1 = vb.default_params(1, sigma_f) if p1 is None else p1
    p2 = vb.default_params(2, sigma_f) if p2 is None else p2
    f, yy, basic = _estimate(y, sigma_f, stage, p1, p2)
    rgb = y.shape[1] == 3
    if stage == "basic":
        L = vb.LinearStep(1, yy, sigma_f, p1, color_space=True)
    else:
        L = vb.LinearStep(2, yy, sigma_f, p2, basic=basic, color_space=True)
    gen = torch.Generator(device=y.device).manual_seed(seed)
    eps = sigma_true / 20.0
    div_fd = div_lin = 0.0
    for _ in range(probes):
        b = torch.randn(y.shape, generator=gen, device=y.device)
        fe, _, _ = _estimate(y + eps * b, sigma_f, stage, p1, p2)
        div_fd += float((b.double() * (fe.double() - f.double())).sum()) / eps
        tb = vb.color_transform(b.clone(), True) if rgb else b
        jb = L.apply(tb)
        jb = vb.color_transform(jb, False) if rgb else jb
        div_lin += float((b.double() * jb.double()).sum())
    L.close()
    div_fd /= probes
    div_lin /= probes
    n = y.numel()
    res = float(((f.double() - y.double()) ** 2).sum()) / n
    out = dict(sigma_f=sigma_f, div_fd=div_fd, div_linear=div_lin,
               sure_fd=res - sigma_true ** 2 + 2 * sigma_true ** 2 * div_fd / n,
               sure_linear=res - sigma_true ** 2 + 2 * sigma_true ** 2 * div_lin / n)
    if clean is not None:
        out["mse"] = float(((f.double() - clean.double()) ** 2).mean())
    return out


def sure_step2_fixed_basic(y, sigma_true, sigma_f, basic, clean=None, probes=2, seed=0, p2=None):
    """SURE of step 2 (Wiener) run at sigma_f with the basic estimate held
    fixed: `basic` is given in the working colour space (YUV for RGB input)
    and does not depend on y.  Then the estimate f(y) = T^-1 L T y is exactly
    linear in y (groups and Wiener gains come from `basic`; aggregation is
    linear), so b^T J b with J = T^-1 L T is an unbiased estimate of its
    divergence and SURE is unbiased for its MSE.  Returns sure (linearised
    divergence), sure_fd (finite-difference divergence, for comparison) and,
    when `clean` is given, the true MSE."""
    p2 = vb.default_params(2, sigma_f) if p2 is None else p2
    rgb = y.shape[1] == 3

    def estimate(v):
        vv = vb.color_transform(v.clone(), True) if rgb else v.clone()
        out = vb.normalize(*vb.step2(vv, basic, p2, sigma_f, color_space=True), basic)
        return (vb.color_transform(out.clone(), False) if rgb else out), vv

    f, yy = estimate(y)
    L = vb.LinearStep(2, yy, sigma_f, p2, basic=basic, color_space=True)
    gen = torch.Generator(device=y.device).manual_seed(seed)
    eps = sigma_true / 20.0
    div_lin = div_fd = 0.0
    for _ in range(probes):
        b = torch.randn(y.shape, generator=gen, device=y.device)
        tb = vb.color_transform(b.clone(), True) if rgb else b
        jb = L.apply(tb)
        jb = vb.color_transform(jb, False) if rgb else jb
        div_lin += float((b.double() * jb.double()).sum())
        fe, _ = estimate(y + eps * b)
        div_fd += float((b.double() * (fe.double() - f.double())).sum()) / eps
    L.close()
    div_lin /= probes
    div_fd /= probes
    n = y.numel()
    res = float(((f.double() - y.double()) ** 2).sum()) / n
    out = dict(sigma_f=sigma_f, div=div_lin, div_fd=div_fd,
               sure=res - sigma_true ** 2 + 2 * sigma_true ** 2 * div_lin / n,
               sure_fd=res - sigma_true ** 2 + 2 * sigma_true ** 2 * div_fd / n)
    if clean is not None:
        out["mse"] = float(((f.double() - clean.double()) ** 2).mean())
    return out
