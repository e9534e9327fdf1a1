"""The multiscaler restatement (oracle/ms_oracle.py) against the reference's
own programs: the golden vectors they produced (tests/golden/multiscaler)
and, where the reference sources were available at build time, the programs
themselves (oracle/_ref/libms_ref.so).  CPU only."""
import glob
import os

import numpy as np
import pytest

from oracle import ms_oracle as M

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "multiscaler", "*.npz")))
RATIOS = (0.7, 0.8, 0.5)


def close(a, b):
    """Equal to float rounding: both sides evaluate the transforms in double
    and round once to float (scipy's FFT, the reference's direct sums), so
    they differ by single-ulp roundings; the bound is two ulps of the
    largest value (values near zero carry the ulps of the sums that made
    them)."""
    assert a.shape == b.shape
    return float(np.abs(a.astype(np.float64) - b).max()) <= 2.0 ** -22 * float(np.abs(b).max())


def test_golden_present():
    assert len(GOLDEN) == 4


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_restatement_matches_golden(path):
    g = np.load(path)
    img, levels = g["img"], int(g["levels"])
    lv = M.decompose(img, levels)
    for i, x in enumerate(lv):
        ref = g["level_%d" % i]
        assert close(x, ref), i
    for f in RATIOS:
        rec = M.recompose([g["level_%d" % i] for i in range(levels)], f)
        assert close(rec, g["recompose_%g" % f])
        if levels > 1:
            assert close(M.merge_coarse(img, g["level_1"], f), g["merge_%g" % f])


@pytest.mark.skipif(not M.MsRef.available(), reason="reference multiscaler not built here")
@pytest.mark.parametrize("shape,levels", [((1, 29, 41), 3), ((3, 40, 24), 2), ((2, 33, 66), 5)])
def test_restatement_matches_reference_programs(shape, levels):
    rng = np.random.default_rng(sum(shape) + levels)
    img = (rng.random(shape) * 255).astype(np.float32)
    r = M.MsRef()
    lv_ref = r.decompose(img, levels)
    lv = M.decompose(img, levels)
    assert [x.shape for x in lv] == [x.shape for x in lv_ref]
    assert all(close(a, b) for a, b in zip(lv, lv_ref))
    for f in (0.7, 0.3, 1.0):
        assert close(M.recompose(lv_ref, f), r.recompose(lv_ref, f))
    if levels > 1:
        assert close(M.merge_coarse(img, lv_ref[1], 0.6), r.merge_coarse(img, lv_ref[1], 0.6))


def test_block_count_is_the_float_loop_bound():
    # j < n * factor with the product in float: 135 * 0.7f rounds to 94.5
    assert M.block_count(135, 0.7) == 95
    assert M.block_count(10, 0.7) == 7      # 10 * 0.7f rounds to 7.0
    assert M.block_count(540, 0.7) == 378
    assert M.block_count(100, 0.8) == 80
    assert M.block_count(37, 0.3) == 12
    assert M.block_count(7, 1.0) == 7
    assert M.block_count(7, 0.0) == 0


def test_level_sizes_halve_by_integer_division():
    assert M.level_sizes(1080, 1920, 3) == [(1080, 1920), (540, 960), (270, 480)]
    assert M.level_sizes(45, 31, 4) == [(45, 31), (22, 15), (11, 7), (5, 3)]


def test_level_sigma_truncates_like_bc():
    # sigma=$(bc <<< "scale=2; $NOISE / 2^$lvl")
    assert [M.level_sigma(25, l) for l in range(4)] == [25.0, 12.5, 6.25, 3.12]
    assert M.level_sigma(30, 2) == 7.5
    assert M.level_sigma(10, 3) == 1.25
    assert M.level_sigma(15, 2) == 3.75


def test_roundtrip_restores_the_image():
    rng = np.random.default_rng(7)
    img = (rng.random((2, 40, 56)) * 255).astype(np.float32)
    for f in (0.7, 1.0):
        out = M.recompose(M.decompose(img, 3), f)
        assert np.abs(out - img).max() < 1e-3


def test_level_zero_is_the_image():
    rng = np.random.default_rng(8)
    img = (rng.random((1, 32, 48)) * 255).astype(np.float32)
    assert np.abs(M.decompose(img, 1)[0] - img).max() < 1e-3
