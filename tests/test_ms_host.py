"""Host-side helpers of the multiscale path (no GPU): the pyramid's level
shapes and the noise level each level is denoised with."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import vbm3d_gb300 as vb  # noqa: E402


def test_level_sigma_is_bc_with_scale_2():
    # sigma=$(bc <<< "scale=2; $NOISE / ${R_PYR}^$lvl"), R_PYR=2
    # (src/utils/VBM3Ddenoising_multiscale.sh:25, :51): the quotient
    # truncated to two decimals
    cases = {(25, 0): 25.0, (25, 1): 12.5, (25, 2): 6.25, (25, 3): 3.12, (10, 3): 1.25, (5, 3): 0.62,
             (1, 3): 0.12, (30, 2): 7.5, (17.5, 2): 4.37, (40, 5): 1.25, (3, 5): 0.09, (12.34, 1): 6.17}
    for (sigma, level), want in cases.items():
        assert vb.ms_level_sigma(sigma, level) == want, (sigma, level)


def test_level_shapes_halve_by_integer_division():
    assert vb.ms_level_shapes((5, 3, 1080, 1920), 3) == [(5, 3, 1080, 1920), (5, 3, 540, 960), (5, 3, 270, 480)]
    assert vb.ms_level_shapes((7, 33, 17), 4) == [(7, 33, 17), (7, 16, 8), (7, 8, 4), (7, 4, 2)]
    assert vb.ms_level_shapes((9, 6), 1) == [(9, 6)]
