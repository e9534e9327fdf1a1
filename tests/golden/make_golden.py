"""Generates the golden vectors in tests/golden/*.npz from the REFERENCE'S
OWN CODE (oracle/_ref/libvbm3d_ref_exact.so, built by oracle/build_ref.sh
from the tehret/vbm3d sources with -O2 -ffp-contract=off and the FFTW shim).

Run in a checkout where the reference sources were available:
    sh oracle/build_ref.sh /path/to/vbm3d && python tests/golden/make_golden.py

Each fixture stores its inputs (so the tests never regenerate them) and the
reference's outputs: block-matching tables of both steps, the step-1
numerator/denominator, and run_vbm3d's basic and final estimates
(single-thread path, src/vbm3d.cpp:142-211).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.pyoracle import Oracle, RefLib  # noqa: E402
from vbm3d_gb300._abi import dims_of  # noqa: E402
from vbm3d_gb300.synth import make_clip  # noqa: E402

CASES = [
    # name, W, H, F, C, sigma, seed, flows, color_space, step-1 / step-2 overrides
    ("gray_dct", 40, 32, 6, 1, 20.0, 101, False, False, dict(T_2D=0), {}),
    ("gray_default", 40, 32, 5, 1, 20.0, 102, False, False, {}, {}),
    ("rgb_color", 32, 28, 4, 3, 25.0, 103, False, True, {}, {}),
    ("rgb_flow_s40", 32, 28, 4, 3, 40.0, 104, True, False, {}, {}),
    ("rgb_bior_s20", 32, 24, 4, 3, 20.0, 105, False, True, dict(T_2D=1), dict(k=8, p=4, T_2D=1)),
    ("gray_hadamard", 32, 28, 5, 1, 30.0, 106, True, False, dict(T_3D=2), dict(T_3D=2)),
    ("gray_kt2_mc", 32, 28, 5, 1, 20.0, 107, True, False, dict(kt=2, T_2D=0, mc=1), dict(kt=2, mc=1)),
    ("ties_quantized", 36, 30, 5, 1, 5.0, 108, False, False, {}, {}),
]


def main():
    o, r = Oracle(), RefLib(exact=True)
    for name, W, H, F, C, sigma, seed, flows, cs, o1, o2 in CASES:
        clean, noisy, ff, bf = make_clip(W, H, F, C, sigma, seed, with_flow=flows)
        if name == "ties_quantized":
            noisy = np.round(clean / 16.0 + np.random.default_rng(seed).normal(0, 0.6, clean.shape)).astype(np.float32)
        p1 = o.default_params(1, sigma).replace(**o1)
        p2 = o.default_params(2, sigma).replace(**o2)
        d = dims_of(noisy)
        out = dict(noisy=noisy, sigma=np.float32(sigma), color_space=np.int32(cs),
                   p1=np.array(list(p1.as_dict().values()), np.float64),
                   p2=np.array(list(p2.as_dict().values()), np.float64))
        if flows:
            out.update(fflow=ff, bflow=bf)
        # step-1 block matching on noisy (video as the step sees it)
        vid1 = o.color_transform(noisy, True) if cs else noisy
        pidx1 = o.ref_indices(p1, d)
        bm1 = r.similar(p1, vid1, pidx1, ff, bf)
        out.update({"bm1_" + k: v for k, v in bm1.items()})
        num, den = r.step(1, p1, sigma, vid1, None, ff, bf, color_space=cs)
        if name in ("gray_dct", "rgb_color"):
            out.update(num1=num, den1=den)
        basic, final = r.run(sigma, noisy, p1, p2, ff, bf, color_space=cs, threads=1)
        out.update(basic=basic, final=final)
        # step-2 block matching on the reference's basic estimate (in the
        # colour space the step sees)
        basic_ws = np.where(den == 0, vid1, num / np.where(den == 0, 1, den)).astype(np.float32)
        bm2 = r.similar(p2, basic_ws, o.ref_indices(p2, d), ff, bf)
        out.update({"bm2_" + k: v for k, v in bm2.items()})
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **out)
        print(name, os.path.getsize(path))


if __name__ == "__main__":
    main()
