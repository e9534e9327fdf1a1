"""Generates the multiscaler golden vectors in tests/golden/multiscaler/*.npz
from the REFERENCE'S OWN CODE (oracle/_ref/libms_ref.so: the programs
multiscaler/decompose.cpp, recompose.cpp and merge_coarse.cpp over
multiscaler/multiscaler.cpp, built by oracle/build_ref.sh against the FFTW
stand-in in oracle/fftw_shim and an in-memory image table in place of iio).

    sh oracle/build_ref.sh /path/to/vbm3d && python tests/golden/make_golden_multiscaler.py

Each fixture stores a planar image `img` [C, H, W], the level count, the
levels `level_<i>` that `decompose` writes, and for each recomposition
ratio f in RATIOS the image `recompose_<f>` that `recompose` makes from
those levels and `merge_<f>` that `merge_coarse img level_1` makes.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.ms_oracle import MsRef  # noqa: E402
from vbm3d_gb300.synth import make_clip  # noqa: E402

RATIOS = (0.7, 0.8, 0.5)
CASES = [
    # name, C, H, W, levels, seed
    ("rgb_48x64_l3", 3, 48, 64, 3, 301),     # the script's 3 levels
    ("gray_37x53_l3", 1, 37, 53, 3, 302),    # odd sizes: levels 18x26, 9x13
    ("rgb_45x31_l4", 3, 45, 31, 4, 303),     # 4 levels down to 5x3
    ("gray_16x16_l2", 1, 16, 16, 2, 304),
]


def main():
    r = MsRef()
    out_dir = os.path.join(HERE, "multiscaler")
    os.makedirs(out_dir, exist_ok=True)
    for name, c, h, w, levels, seed in CASES:
        _, noisy, _, _ = make_clip(w, h, 1, c, 20.0, seed)
        img = np.ascontiguousarray(noisy[0], dtype=np.float32)
        lv = r.decompose(img, levels)
        rec = {"img": img, "levels": np.int32(levels)}
        for i, x in enumerate(lv):
            rec["level_%d" % i] = x
        for f in RATIOS:
            rec["recompose_%g" % f] = r.recompose(lv, f)
            if levels > 1:
                rec["merge_%g" % f] = r.merge_coarse(img, lv[1], f)
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), **rec)
        print(name, [x.shape for x in lv])


if __name__ == "__main__":
    main()
