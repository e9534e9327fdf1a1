"""CPU: the TV-L1 restatement (oracle/tvl1_oracle.c) against golden vectors
made by the reference's own tvl1flow_lib.c (tests/golden/tvl1/, generated
by tests/golden/make_golden_tvl1.py), bit for bit; and against the compiled
reference itself on fresh inputs where it is present."""
import glob
import os

import numpy as np
import pytest

from oracle.pyoracle import TvlOracle, TvlRef
from vbm3d_gb300.synth import make_clip

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "tvl1")
NAMES = sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_tvl1(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


def params_of(o, opts):
    keys = ["tau", "lambda_", "theta", "nscales", "fscale", "zfactor", "nwarps", "epsilon"]
    kw = {k: (int(v) if k in ("nscales", "fscale", "nwarps") else float(v)) for k, v in zip(keys, opts)}
    return o.default_params(**kw)


@pytest.fixture(scope="module")
def tv():
    return TvlOracle()


def test_golden_present():
    assert len(NAMES) >= 5


@pytest.mark.parametrize("name", NAMES)
def test_restatement_equals_reference_golden(tv, name):
    g = load_tvl1(name)
    got = tv.flow(g["I0"], g["I1"], params_of(tv, g["opts"]))
    np.testing.assert_array_equal(got, g["flow"])


@pytest.mark.skipif(not TvlRef.available(), reason="reference sources not built here")
@pytest.mark.parametrize("shape,fs,seed", [((57, 41), 0, 1), ((80, 60), 2, 2), ((33, 90), 1, 3)])
def test_restatement_equals_compiled_reference(tv, shape, fs, seed):
    w, h = shape
    _, noisy, _, _ = make_clip(w, h, 2, 1, 15.0, 300 + seed, vmax=3.0)
    p = tv.default_params(fscale=fs)
    np.testing.assert_array_equal(tv.flow(noisy[0, 0], noisy[1, 0], p), TvlRef().flow(noisy[0, 0], noisy[1, 0], p))


def test_scales_rule(tv):
    # main.c: min(nscales, 1 + log(hypot/16) / log(1/zfactor)), truncated
    p = tv.default_params()
    assert tv.scales(960, 540, p)[0] == 7
    assert tv.scales(64, 48, p)[0] == 3
    assert tv.scales(1920, 1080, tv.default_params(nscales=4))[0] == 4


def test_translation_recovered(tv):
    # a textured frame shifted by (2, 1) pixels: the flow of the interior is (2, 1)
    rng = np.random.default_rng(0)
    base = np.cumsum(np.cumsum(rng.normal(0, 1, (80, 100)), 0), 1).astype(np.float32)
    I0 = base[10:70, 10:90].copy()
    I1 = base[9:69, 8:88].copy()   # I1(x, y) = I0(x - 2, y - 1): motion (2, 1)
    f = tv.flow(I0, I1, tv.default_params(fscale=0))
    inner = (slice(10, -10), slice(10, -10))
    assert abs(float(np.median(f[0][inner])) - 2.0) < 0.1
    assert abs(float(np.median(f[1][inner])) - 1.0) < 0.1
