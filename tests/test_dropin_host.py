"""The drop-in shim on the CPU: it builds against the stand-in of the
reference's vbm3d.h and rejects flows whose size main.cpp would reject
(src/main.cpp:372-376) before any CUDA call."""
import numpy as np
import pytest

from dropin_util import build_driver, run_driver


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    e = build_driver(tmp_path_factory.mktemp("dropin"))
    if e is None:
        pytest.skip("g++ not found")
    return e


@pytest.mark.parametrize("fshape", [(3, 2, 24, 32), (6, 2, 24, 32), (4, 2, 24, 30), (4, 3, 24, 32)])
def test_flow_size_mismatch_rejected(exe, tmp_path, fshape):
    # a video of 5 frames: flows of 5 or 4 frames are valid (the GPU tests
    # run both); other frame counts, another width or a channel count other
    # than 2 are the mismatch
    noisy = np.zeros((5, 1, 24, 32), np.float32)
    bad = np.zeros(fshape, np.float32)
    good = np.zeros((4, 2, 24, 32), np.float32)
    rc, a, b, err = run_driver(exe, tmp_path, "run", noisy, 20.0, bad, good, color_space=False, tag="r")
    assert rc == 1 and "VBM3D_ERR_SIZE_MISMATCH" in err, (rc, err)
    # the steps cannot return an error: they report it and leave num / den zero
    rc, num, den, err = run_driver(exe, tmp_path, "step1", noisy, 20.0, good, bad, color_space=False, tag="s")
    assert rc == 0 and "VBM3D_ERR_SIZE_MISMATCH" in err
    assert not num.any() and not den.any()
