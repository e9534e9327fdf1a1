"""Pins the CPU oracle (oracle/vbm3d_oracle.c) to golden vectors produced by
the reference's own code: every comparison is bit-exact."""
import numpy as np
import pytest

from golden_util import load, names
from oracle.pyoracle import Oracle
from vbm3d_gb300._abi import dims_of


@pytest.fixture(scope="module")
def oracle():
    return Oracle()


def test_golden_present():
    assert len(names()) >= 8


@pytest.mark.parametrize("name", names())
def test_block_matching_step1(oracle, name):
    g = load(name)
    vid = oracle.color_transform(g["noisy"], True) if g["color_space"] else g["noisy"]
    res = oracle.similar(g["p1"], vid, g["fflow"], g["bflow"])
    for key in ("idx", "dist", "nsimp", "nsx"):
        np.testing.assert_array_equal(res[key], g["bm1_" + key], err_msg=key)


@pytest.mark.parametrize("name", names())
def test_block_matching_step2(oracle, name):
    g = load(name)
    vid1 = oracle.color_transform(g["noisy"], True) if g["color_space"] else g["noisy"]
    num, den = oracle.step(1, g["p1"], g["sigma"], vid1, None, g["fflow"], g["bflow"], g["color_space"])
    basic = np.where(den == 0, vid1, num / np.where(den == 0, 1, den)).astype(np.float32)
    res = oracle.similar(g["p2"], basic, g["fflow"], g["bflow"])
    for key in ("idx", "dist", "nsimp", "nsx"):
        np.testing.assert_array_equal(res[key], g["bm2_" + key], err_msg=key)


@pytest.mark.parametrize("name", [n for n in names() if n in ("gray_dct", "rgb_color")])
def test_step1_aggregation(oracle, name):
    g = load(name)
    vid1 = oracle.color_transform(g["noisy"], True) if g["color_space"] else g["noisy"]
    num, den = oracle.step(1, g["p1"], g["sigma"], vid1, None, g["fflow"], g["bflow"], g["color_space"])
    np.testing.assert_array_equal(num, g["num1"])
    np.testing.assert_array_equal(den, g["den1"])


@pytest.mark.parametrize("name", names())
@pytest.mark.parametrize("threads", [1, 3])
def test_run_vbm3d(oracle, name, threads):
    g = load(name)
    basic, final = oracle.run(g["sigma"], g["noisy"], g["p1"], g["p2"], g["fflow"], g["bflow"],
                              g["color_space"], threads=threads)
    np.testing.assert_array_equal(basic, g["basic"])
    np.testing.assert_array_equal(final, g["final"])


def test_default_params(oracle):
    p = oracle.default_params(1, 20.0)
    assert (p.k, p.p, p.N, p.Nf, p.Ns, p.Npr, p.Nb, p.T_2D) == (8, 6, 8, 4, 7, 5, 2, 1)
    assert p.tau == 3000 and abs(p.d - 49 * 255 / 64) < 1e-4 and abs(p.lambda3D - 2.7) < 1e-6
    p = oracle.default_params(2, 20.0)
    assert (p.k, p.p, p.T_2D, p.tau) == (7, 3, 0, 1500)
    p = oracle.default_params(2, 40.0)
    assert (p.k, p.p, p.tau) == (8, 4, 3000)
    assert oracle.default_params(1, 40.0).tau == 4500


def test_grid_matches_reference_counts(oracle):
    # refs/frame counts of the reference's single-thread grid (src/vbm3d.cpp:471-489)
    for (w, h), step, sigma, want in [((176, 144), 1, 20, 696), ((176, 144), 2, 20, 2726),
                                      ((1920, 1080), 1, 30, 57600), ((1920, 1080), 2, 30, 229401),
                                      ((960, 540), 2, 40, 32026)]:
        p = oracle.default_params(step, sigma)
        rows, cols = oracle.grid(p, dims_of(np.zeros((1, 1, h, w), np.float32)))
        assert len(rows) * len(cols) == want


def test_kaiser_symmetric(oracle):
    for k in (4, 6, 7, 8, 12):
        w = oracle.kaiser(k)
        np.testing.assert_array_equal(w, w.T)
        np.testing.assert_array_equal(w, w[::-1, ::-1])
    np.testing.assert_array_equal(oracle.kaiser(5), np.ones((5, 5), np.float32))
    assert oracle.kaiser(8)[0, 0] == np.float32(0.1924) and oracle.kaiser(7)[3, 3] == np.float32(1.0)


def test_transform_roundtrips(oracle):
    rng = np.random.default_rng(0)
    x = rng.normal(0, 50, 64).astype(np.float32)
    for k in (4, 7, 8):
        b = rng.normal(0, 50, k * k).astype(np.float32)
        np.testing.assert_allclose(oracle.block("dct2d_inverse", oracle.block("dct2d_forward", b, k), k), b, atol=1e-3)
    # The reference's bior1.5 tables (src/lib_transforms.cpp:141-148, :281-288)
    # are not an exact inverse pair: inverse(forward(x)) is within ~4% of x.
    rt = oracle.block("bior2d_inverse", oracle.block("bior2d_forward", x))
    assert 1e-3 < np.abs(rt - x).max() < 0.05 * np.abs(x).max()
    for n in (1, 2, 4, 8, 16):
        v = rng.normal(0, 50, n).astype(np.float32)
        np.testing.assert_allclose(oracle.haar(oracle.haar(v), inverse=True), v, atol=1e-3)


def test_color_roundtrip_is_the_references(oracle):
    rng = np.random.default_rng(1)
    v = rng.uniform(0, 255, (2, 3, 8, 9)).astype(np.float32)
    back = oracle.color_transform(oracle.color_transform(v, True), False)
    # the reference's inverse uses different literals: close, not exact
    assert np.abs(back - v).max() < 0.1
