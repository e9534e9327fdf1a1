"""One VBM3D run (both steps) on a seeded synthetic clip, for profilers.

    python -m vbm3d_gb300.profile_case --width 1280 --height 720 --frames 16

Launch order inside one run (colour transform on): color, bm (step 1),
filter<1>, normalize, bm (step 2), filter<2>, normalize, color x3.
"""
import argparse

import torch

import vbm3d_gb300 as vb
from vbm3d_gb300.synth import make_clip


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--width", type=int, default=1280)
    ap.add_argument("--height", type=int, default=720)
    ap.add_argument("--frames", type=int, default=16)
    ap.add_argument("--channels", type=int, default=3)
    ap.add_argument("--sigma", type=float, default=30.0)
    ap.add_argument("--runs", type=int, default=1)
    a = ap.parse_args()
    _, noisy, _, _ = make_clip(a.width, a.height, a.frames, a.channels, a.sigma, seed=4000, vmax=6.0)
    x0 = torch.from_numpy(noisy).cuda()
    for _ in range(a.runs):
        x = x0.clone()
        vb.run(x, a.sigma, color_space=a.channels == 3)
    torch.cuda.synchronize()
    print("ok")


if __name__ == "__main__":
    main()
