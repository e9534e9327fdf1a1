"""Differentiation workload: RGB 480x270x16, sigma = 25 (seeded synthetic clip).

    python -m vbm3d_gb300.linear_case

Prints one JSON line: the time of the forward steps, of building each
step's frozen linearisation, of applying it and of applying its adjoint
(CUDA events, 3 warm-up + 10 timed repetitions), the adjoint/forward ratios,
and a 16-value sweep of the filter's sigma with Monte-Carlo SURE (finite-
difference and linearised divergence) against the true MSE of the basic and
final estimates.
"""
import json

import numpy as np
import torch

import vbm3d_gb300 as vb
from vbm3d_gb300.sure import mc_sure, sure_step2_fixed_basic
from vbm3d_gb300.synth import make_clip

W, H, F, C, SIGMA = 480, 270, 16, 3, 25.0


def timed(fn, reps=10, warm=3):
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def main():
    clean, noisy, _, _ = make_clip(W, H, F, C, SIGMA, seed=5000)
    dev = torch.device("cuda:0")
    y = torch.from_numpy(noisy).to(dev)
    c = torch.from_numpy(clean).to(dev)
    p1, p2 = vb.default_params(1, SIGMA), vb.default_params(2, SIGMA)
    yy = vb.color_transform(y.clone(), True)
    basic = vb.normalize(*vb.step1(yy, p1, SIGMA, color_space=True), yy)
    out = {"workload": "RGB %dx%dx%d, sigma=%g, colour transform on" % (W, H, F, SIGMA)}
    out["forward_step1_ms"] = timed(lambda: vb.step1(yy, p1, SIGMA, color_space=True))
    out["forward_step2_ms"] = timed(lambda: vb.step2(yy, basic, p2, SIGMA, color_space=True))
    L1 = vb.LinearStep(1, yy, SIGMA, p1, color_space=True)
    L2 = vb.LinearStep(2, yy, SIGMA, p2, basic=basic, color_space=True)
    out["create_step1_ms"] = timed(lambda: vb.LinearStep(1, yy, SIGMA, p1, color_space=True).close(), reps=3, warm=1)
    out["create_step2_ms"] = timed(lambda: vb.LinearStep(2, yy, SIGMA, p2, basic=basic, color_space=True).close(),
                                   reps=3, warm=1)
    x = torch.randn_like(y)
    for name, L in (("step1", L1), ("step2", L2)):
        out["jvp_%s_ms" % name] = timed(lambda: L.apply(x))
        out["adjoint_%s_ms" % name] = timed(lambda: L.apply(x, adjoint=True))
        out["adjoint_over_forward_%s" % name] = out["adjoint_%s_ms" % name] / out["forward_%s_ms" % name]
    # consistency on this workload: <L x, g> = <x, L^T g>
    g = torch.randn_like(y)
    for name, L in (("step1", L1), ("step2", L2)):
        a = float((L.apply(x).double() * g.double()).sum())
        b = float((x.double() * L.apply(g, adjoint=True).double()).sum())
        out["dot_rel_err_%s" % name] = abs(a - b) / abs(a)
    sweep = [float(s) for s in np.linspace(10.0, 55.0, 16)]
    rows = []
    for sf in sweep:
        rb = mc_sure(y, SIGMA, sf, clean=c, stage="basic", probes=2)
        rf = mc_sure(y, SIGMA, sf, clean=c, stage="final", probes=2)
        rows.append({"sigma_f": round(sf, 2),
                     "basic": {k: round(rb[k], 3) for k in ("mse", "sure_fd", "sure_linear")},
                     "final": {k: round(rf[k], 3) for k in ("mse", "sure_fd", "sure_linear")}})
    out["sure_sweep"] = rows
    # step 2 with a fixed basic estimate: exact divergence of a linear map
    rng = np.random.default_rng(5077)  # an independent noise realisation of the same clean clip
    noisy2 = (clean + np.float32(SIGMA) * rng.standard_normal(clean.shape, dtype=np.float32)).astype(np.float32)
    y2 = vb.color_transform(torch.from_numpy(noisy2).to(dev), True)
    b2 = vb.normalize(*vb.step1(y2, p1, SIGMA, color_space=True), y2)
    fixed = []
    for sf in (12.0, 18.0, 22.0, 25.0, 30.0, 40.0):
        r = sure_step2_fixed_basic(y, SIGMA, sf, b2, clean=c, probes=8)
        fixed.append({k: round(r[k], 3) for k in ("sigma_f", "mse", "sure", "sure_fd")})
    out["sure_step2_fixed_basic"] = fixed
    # the realisation's sample noise variance less sigma^2: the part of
    # SURE - MSE common to every sigma_f
    out["noise_variance_offset"] = float(np.mean((noisy.astype(np.float64) - clean) ** 2) - SIGMA ** 2)
    out["sure_step2_fixed_basic_max_rel_err"] = max(abs(r["sure"] - r["mse"]) / r["mse"] for r in fixed)
    out["sure_step2_fixed_basic_argmin"] = [min(fixed, key=lambda r: r[k])["sigma_f"] for k in ("mse", "sure")]
    for st in ("basic", "final"):
        mse = [r[st]["mse"] for r in rows]
        for kind in ("sure_fd", "sure_linear"):
            s = [r[st][kind] for r in rows]
            out["%s_%s_argmin_sigma" % (st, kind)] = rows[int(np.argmin(s))]["sigma_f"]
            out["%s_%s_max_rel_err" % (st, kind)] = float(np.max(np.abs(np.array(s) - mse) / np.array(mse)))
        out["%s_mse_argmin_sigma" % st] = rows[int(np.argmin(mse))]["sigma_f"]
    print(json.dumps(out))


if __name__ == "__main__":
    main()
