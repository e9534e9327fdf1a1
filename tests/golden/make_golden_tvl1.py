"""Generates the TV-L1 golden vectors in tests/golden/tvl1/*.npz from the
REFERENCE'S OWN CODE (oracle/_ref/libtvl1_ref.so: tvl1flow/tvl1flow_lib.c
compiled by oracle/build_ref.sh, single thread, no FP contraction).

    sh oracle/build_ref.sh /path/to/vbm3d && python tests/golden/make_golden_tvl1.py

Each fixture stores the two frames, the options (tau, lambda, theta,
nscales, fscale, zfactor, nwarps, epsilon) and the reference's flow
[2, H, W] from I0 to I1.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.pyoracle import TvlOracle, TvlRef  # noqa: E402
from vbm3d_gb300.synth import make_clip  # noqa: E402

CASES = [
    # name, W, H, sigma, seed, vmax, option overrides
    ("scripts_64x48", 64, 48, 20.0, 201, 3.0, {}),                    # the flow scripts' options (fscale 2)
    ("cli_96x72", 96, 72, 10.0, 202, 3.0, dict(fscale=0, lambda_=0.15)),  # the CLI defaults
    ("odd_123x77_fs1", 123, 77, 25.0, 203, 4.0, dict(fscale=1)),
    ("clean_160x96", 160, 96, 0.0, 204, 5.0, dict(fscale=0, nwarps=3)),
    ("flat_32x24", 32, 24, 0.0, 205, 0.0, dict(fscale=0)),            # constant frames: no normalisation, zero gradient
]


def main():
    o, r = TvlOracle(), TvlRef()
    out_dir = os.path.join(HERE, "tvl1")
    os.makedirs(out_dir, exist_ok=True)
    for name, W, H, sigma, seed, vmax, over in CASES:
        clean, noisy, _, _ = make_clip(W, H, 2, 1, max(sigma, 1e-6), seed, vmax=vmax)
        frames = clean if sigma == 0.0 else noisy
        I0, I1 = frames[0, 0].copy(), frames[1, 0].copy()
        if name.startswith("flat"):
            I0[:] = 77.0
            I1[:] = 77.0
        p = o.default_params(**over)
        flow = r.flow(I0, I1, p)
        opts = np.array([p.tau, p.lambda_, p.theta, p.nscales, p.fscale, p.zfactor, p.nwarps, p.epsilon], np.float64)
        path = os.path.join(out_dir, name + ".npz")
        np.savez_compressed(path, I0=I0, I1=I1, opts=opts, flow=flow)
        print(name, os.path.getsize(path), float(np.abs(flow).mean()))


if __name__ == "__main__":
    main()
