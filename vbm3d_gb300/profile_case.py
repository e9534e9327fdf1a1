"""One VBM3D run (both steps) on seeded synthetic data, for profilers.

    python -m vbm3d_gb300.profile_case --width 1280 --height 720 --frames 16 [--runs 5]
    python -m vbm3d_gb300.profile_case --batch 64 [--scale 0.5]
    python -m vbm3d_gb300.profile_case --tvl1 --width 960 --height 540 --frames 16

Plain form: one clip; launch order (colour transform on): color, bm (step
1), filter<1>, normalize, bm (step 2), filter<2>, normalize, color x3; with
--runs > 1 it also prints the median time of a run (CUDA events, the first
run left out).
Batched form: the first `--batch` clips of the uneven-batch workload
(synth.batch_specs, sides times `--scale`), one batch with a fixed
configuration (no tuning pass), run once without the graph so that every
kernel is its own launch (prep, block matching of step 1 per class,
filtering of step 1 per table set, mid, the same for step 2, final), then
once more through vbm3d_batch_profile, which prints each work launch.
TV-L1: forward and backward flows of a one-channel clip with the options of
the reference's flow scripts (vbm3d_gpu_tvl1_video), run twice.
Multiscaler (--ms LEVELS): the DCT pyramid of a clip (vbm3d_gpu_ms_decompose)
and its recomposition with ratio 0.7 (vbm3d_gpu_ms_recompose), run
`--runs` times; launch order per run: cosine matrices, the forward
transform's two products, two products per level; then the recomposition's
cosine matrices, per level two products (and a block copy from level 1),
the inverse transform's two products.
"""
import argparse

import torch

import vbm3d_gb300 as vb
from vbm3d_gb300.synth import batch_specs, make_clip

FIXED = dict(bm1_tile=4, bm1_warps=4, filter1_tile=32, filter1_warps=8, bm2_tile=4, bm2_warps=4, filter2_tile=32,
             filter2_warps=8, no_graph=1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--width", type=int, default=1280)
    ap.add_argument("--height", type=int, default=720)
    ap.add_argument("--frames", type=int, default=16)
    ap.add_argument("--channels", type=int, default=3)
    ap.add_argument("--sigma", type=float, default=30.0)
    ap.add_argument("--runs", type=int, default=1)
    ap.add_argument("--batch", type=int, default=0, help="batched form over this many clips")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--tvl1", action="store_true", help="TV-L1 flows of a one-channel clip")
    ap.add_argument("--ms", type=int, default=0, help="multiscaler DCT pyramid with this many levels")
    ap.add_argument("--deterministic", action="store_true",
                    help="plain form: the deterministic aggregation (vbm3d_set_deterministic)")
    ap.add_argument("--bm-tile", type=int, default=FIXED["bm1_tile"], help="batched block matching: refs per item")
    ap.add_argument("--bm-warps", type=int, default=FIXED["bm1_warps"], help="batched block matching: warps per block")
    ap.add_argument("--plain", action="store_true", help="with --batch: the clips looped through the plain path")
    ap.add_argument("--tuned", action="store_true", help="with --batch: the autotuner's configuration")
    ap.add_argument("--filter-tile", type=int, default=FIXED["filter1_tile"], help="batched filtering: refs per item")
    ap.add_argument("--filter-warps", type=int, default=FIXED["filter1_warps"],
                    help="batched filtering: warps per block")
    a = ap.parse_args()
    if a.ms:
        _, noisy, _, _ = make_clip(a.width, a.height, a.frames, a.channels, a.sigma, seed=4000, vmax=6.0)
        x = torch.from_numpy(noisy).cuda()
        for _ in range(a.runs):
            vb.ms_recompose(vb.ms_decompose(x, a.ms), 0.7)
        torch.cuda.synchronize()
        print("ok")
        return
    if a.tvl1:
        _, noisy, _, _ = make_clip(a.width, a.height, a.frames, 1, a.sigma, seed=4000, vmax=6.0)
        v = torch.from_numpy(noisy[:, 0].copy()).cuda()
        for _ in range(2):
            vb.tvl1_video(v)
        torch.cuda.synchronize()
        print("ok")
        return
    if a.batch:
        clips = []
        for i, (w, h, f, c, s) in enumerate(batch_specs(scale=a.scale)[:a.batch]):
            _, noisy, _, _ = make_clip(w, h, f, c, s, 4000 + i)
            clips.append(dict(noisy=torch.from_numpy(noisy).cuda(), sigma=s))
        if a.plain:
            times = []
            for _ in range(a.runs):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for c in clips:
                    vb.run(c["noisy"].clone(), c["sigma"], color_space=True)
                e1.record()
                torch.cuda.synchronize()
                times.append(e0.elapsed_time(e1))
            if a.runs > 1:
                print("plain loop over %d clips: %.2f ms per run (median of %d)"
                      % (len(clips), sorted(times[1:])[len(times[1:]) // 2], a.runs - 1))
            print("ok")
            return
        cfg = dict(FIXED, bm1_tile=a.bm_tile, bm2_tile=a.bm_tile, bm1_warps=a.bm_warps, bm2_warps=a.bm_warps,
                   filter1_tile=a.filter_tile, filter2_tile=a.filter_tile, filter1_warps=a.filter_warps,
                   filter2_warps=a.filter_warps)
        b = vb.Batch(clips, color_space=True, config=None if a.tuned else cfg)
        for _ in range(a.runs):
            b.run()
        torch.cuda.synchronize()
        for l in b.profile():
            print("launch phase %d k %d C %d: %d clips, %d refs, %d x %d, %.2f ms"
                  % (l["phase"], l["k"], l["channels"], l["clips"], l["refs"], l["tile"], l["warps"], l["ms"]))
        print("ok")
        return
    _, noisy, _, _ = make_clip(a.width, a.height, a.frames, a.channels, a.sigma, seed=4000, vmax=6.0)
    x0 = torch.from_numpy(noisy).cuda()
    x = x0.clone()
    vb.set_deterministic(a.deterministic)
    times = []
    for _ in range(a.runs):
        x.copy_(x0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        vb.run(x, a.sigma, color_space=a.channels == 3)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    if a.runs > 1:  # the first run pays the module loading and the memory pool's growth
        ms = sorted(times[1:])[len(times[1:]) // 2]
        print("plain%s %dx%dx%dx%d sigma %g: %.2f ms per run (median of %d), %.1f Mpix-frames/s"
              % (" (deterministic)" if a.deterministic else "", a.width, a.height, a.frames, a.channels, a.sigma,
                 ms, a.runs - 1,
                 a.width * a.height * a.frames / 1e6 / (ms / 1e3)))
    print("ok")


if __name__ == "__main__":
    main()
